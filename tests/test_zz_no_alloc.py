"""The allocation-free residual entry point (dc_assemble_residual_noalloc).

It exists for callers that cannot allocate device memory when they need a residual; it
stages the state and the residual in a fixed array compiled into the library instead of
buffers allocated on first use.  Checked here through the C ABI against the regular
entry point dc_assemble on two calls in a row (the second with a different state, so
leftovers from the first call would show), within the assembly tolerance of the other
parity tests, and for its documented rejections.  This file is collected last so that a
run stopping at the first failure has already run every other test; it also passes when
run alone in a fresh process (the first call does the per-device set-up).
"""

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

ASM_TOL = 1e-12


def _check_against_regular(dcgpu_lib, ini, form_scales, seed):
    gm = dcgpu_lib.Model(ini)
    rng = np.random.default_rng(seed)
    x0 = gm.state()
    for call in range(2):
        x = x0 + 0.05 * rng.uniform(-1.0, 1.0, gm.ndof) * (call + 1)
        t = 0.0125 * (call + 1)
        for cm, ca in form_scales:
            ref, _ = gm.assemble(x, t, cm, ca, residual=True, jacobian=False)
            got = gm.residual_noalloc(x, t, cm, ca)
            scale = max(np.abs(ref).max(), 1e-300)
            assert np.abs(got - ref).max() <= ASM_TOL * scale, (call, cm, ca)
    gm.close()


def test_noalloc_residual_matches_dc_assemble(dcgpu_lib):
    ini, _ = cases.small_gray_scott(n=24)
    _check_against_regular(dcgpu_lib, ini, [(1.0, 0.0), (0.0, 1.0), (-1.0, 0.29)], seed=3)


def test_noalloc_residual_with_interfaces(dcgpu_lib):
    ini, _ = cases.small_two_compartment(n=16)
    _check_against_regular(dcgpu_lib, ini, [(1.0, 0.0), (0.0, 1.0)], seed=4)


def test_noalloc_rejects_unsupported_models(dcgpu_lib):
    # compartments with different species counts (padded device layout)
    gm = dcgpu_lib.Model(cases.FEATURES_3D_INI)
    with pytest.raises(dcgpu_lib.DcError) as ei:
        gm.residual_noalloc(gm.state(), 0.0, 1.0, 0.0)
    assert ei.value.status == 6
    gm.close()
    # more DOF than the staging array holds (2 x 741^2 > 2^20)
    ini, _ = cases.small_gray_scott(n=740)
    gm = dcgpu_lib.Model(ini)
    assert gm.ndof > 2 ** 20
    with pytest.raises(dcgpu_lib.DcError) as ei:
        gm.residual_noalloc(np.zeros(gm.ndof), 0.0, 1.0, 0.0)
    assert ei.value.status == 6
    gm.close()
