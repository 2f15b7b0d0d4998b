"""The command-line front end (dune-copasi-gb300, mirroring src/dune_copasi.cc): configuration
file plus --key=value options, VTK output every writer.time_step, reduce operators after
every step with an error ending the run."""

import os
import subprocess
import xml.etree.ElementTree as ET

import pytest

import cases

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "dune-copasi_gb300", "dune-copasi-gb300")


def _run(args):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=300)


def test_cli_evolves_writes_vtk_and_reduces(dcgpu_lib, tmp_path):
    cfg = tmp_path / "decay.ini"
    # the L2-error check of the case trips for implicit Euler with dt = 0.1: drop it here
    cfg.write_text(cases.DECAY_INI.replace("err.error.expression = e: e > 5e-3\n", ""))
    out = tmp_path / "out"
    p = _run(["--config=%s" % cfg, "--model.writer.vtk.path=%s" % out, "--model.writer.time_step=0.2"])
    assert p.returncode == 0, p.stdout + p.stderr
    assert "successfully finished" in p.stdout
    assert "mass :=" in p.stdout
    pvd = ET.parse(out / "out-domain.pvd").getroot()
    times = [float(d.get("timestep")) for d in pvd.iter("DataSet")]
    assert times == [pytest.approx(0.0), pytest.approx(0.2), pytest.approx(0.4)]


def test_cli_reduction_error_and_bad_options(dcgpu_lib, tmp_path):
    cfg = tmp_path / "decay.ini"
    cfg.write_text(cases.DECAY_INI)
    p = _run(["--config=%s" % cfg])
    assert p.returncode == 1
    assert "Reduction on the token 'err'" in p.stderr
    assert _run(["--config=%s" % (tmp_path / "missing.ini")]).returncode == 1
    assert _run(["--config=%s" % cfg, "--model.time_step_operator.type=Nonsense"]).returncode == 1
    dump = _run(["--config=%s" % cfg, "--dump-config", "--grid.cells=3 3"])
    assert dump.returncode == 0 and "grid.cells=3 3" in dump.stdout
