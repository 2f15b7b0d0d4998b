"""The command-line front end's option handling, which needs no GPU (src/dune_copasi.cc's
--help / --version / --dump-config / --config / --key=value, and its argument errors)."""

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "dune-copasi_gb300", "dune-copasi-gb300")


def _run(args):
    if not os.path.exists(CLI):
        pytest.skip("command-line front end not built")
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=60)


def test_help_and_version():
    h = _run(["--help"])
    assert h.returncode == 0 and "--config=<string>" in h.stdout and "--dump-config" in h.stdout
    assert _run(["-h"]).returncode == 0
    v = _run(["--version"])
    assert v.returncode == 0 and "dune-copasi-gb300" in v.stdout


def test_dump_config_merges_file_and_options(tmp_path):
    cfg = tmp_path / "m.ini"
    cfg.write_text("[grid]\ncells = 4 4\n")
    p = _run(["--config=%s" % cfg, "--grid.cells=8 8", "--model.time_step_operator.time_end=2", "--dump-config"])
    assert p.returncode == 0
    # the file first, then the options in order (later keys win when the text is parsed)
    assert p.stdout.index("cells = 4 4") < p.stdout.index("grid.cells=8 8")
    assert p.stdout.rstrip().endswith("model.time_step_operator.time_end=2")


def test_argument_errors(tmp_path):
    bad = _run(["positional"])
    assert bad.returncode == 1 and "Invalid argument 'positional'" in bad.stderr
    assert _run(["--no-value-option"]).returncode == 1
    missing = _run(["--config=%s" % (tmp_path / "missing.ini")])
    assert missing.returncode == 1 and "does not exist" in missing.stderr


def test_model_creation_without_gpu_fails_loudly(tmp_path):
    """No CPU fallback: without a CUDA device the run stops at model creation."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    cfg = tmp_path / "m.ini"
    cfg.write_text("[grid]\ncells = 2 2\n[compartments.d]\nexpression = 1\n"
                   "[model.scalar_field.u]\ncompartment = d\n")
    p = _run(["--config=%s" % cfg])
    assert p.returncode == 1 and "Invalid configuration" in p.stderr
