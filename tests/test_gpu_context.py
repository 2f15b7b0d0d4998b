"""GPU parity of the parser-context extras: grayscale TIFF images, functions tabulated with
``interpolate = true`` and interpolation tables, in initial conditions and in the terms the
kernels evaluate; and the reference's rejections of unsupported context types."""

import numpy as np
import pytest

import cases
import tiff_files as TF
from oracle.model import OracleModel
from test_gpu_parity import STEP_TOL, _run_both, assert_newton_per_stage

pytestmark = pytest.mark.gpu


def _images(tmp_path, compression="lzw"):
    a = str(tmp_path / "A.tif")
    b = str(tmp_path / "B.tif")
    TF.write_tiff(a, TF.seeded_image(40, 40, 16, seed=1), bits=16, resolution=(40, 1), compression=compression,
                  predictor=compression == "lzw")
    TF.write_tiff(b, TF.seeded_image(25, 31, 8, seed=2), bits=8, photometric=0, resolution=(25, 1),
                  compression="packbits" if compression != "none" else "none")
    return a, b


def test_tiff_initial_state_matches_oracle(dcgpu_lib, tmp_path):
    """Initial concentrations read from the images: identical nodal values."""
    ini = cases.context_ini(*_images(tmp_path))
    om = OracleModel(ini)
    gm = dcgpu_lib.Model(ini)
    assert np.array_equal(gm.state(), om.initial_state())
    gm.close()


@pytest.mark.parametrize("compression", ["none", "lzw"])
def test_context_extras_time_stepping_matches_oracle(dcgpu_lib, tmp_path, compression):
    ini = cases.context_ini(*_images(tmp_path, compression))
    records = _run_both(dcgpu_lib, ini, None)
    assert records
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (t, name, e)
        assert_newton_per_stage(n_o, n_g, (t,))


@pytest.mark.parametrize("section,msg", [
    ("[parser_context.q]\ntype = random_field\n", "random fields"),
    ("[parser_context.q]\ntype = cell_data\n", "cell data"),
    ("[parser_context.q]\ntype = tiff\npath = /nonexistent/im.tif\n", "does not exists"),
])
def test_unsupported_context_types_rejected(dcgpu_lib, section, msg):
    ini, _ = cases.small_heat(n=8, steps=1)
    with pytest.raises(dcgpu_lib.DcError) as e:
        dcgpu_lib.Model(ini + "\n" + section)
    assert e.value.status == 4 and msg in str(e.value)
