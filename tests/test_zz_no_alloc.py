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


def _device_free_bytes():
    """cudaMemGetInfo's free bytes on the current device, through the CUDA runtime that
    libdcgpu itself loaded."""
    import ctypes
    rt = ctypes.CDLL("libcudart.so.%d" % _cudart_major())
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def _cudart_major():
    import re
    maps = open("/proc/self/maps").read()
    m = re.search(r"libcudart\.so\.(\d+)", maps)
    assert m, "libcudart is not loaded"
    return int(m.group(1))


def test_noalloc_on_fresh_model_allocates_nothing(dcgpu_lib):
    # a model that never ran the regular entry point, so none of its on-demand buffers exist
    # to hide an allocation made by this call
    ini, _ = cases.small_gray_scott(n=20)
    gm = dcgpu_lib.Model(ini)
    rng = np.random.default_rng(7)
    x = gm.state() + 0.01 * rng.uniform(-1.0, 1.0, gm.ndof)
    out = np.empty(gm.ndof)
    gm.residual_noalloc(x, 0.0, 1.0, 0.5, out=out)  # warm-up call
    free0 = _device_free_bytes()
    first = out.copy()
    gm.residual_noalloc(x, 0.0, 1.0, 0.5, out=out)
    free1 = _device_free_bytes()
    assert free1 == free0
    assert np.array_equal(out, first)
    ref, _ = gm.assemble(x, 0.0, 1.0, 0.5, residual=True, jacobian=False)
    assert np.abs(out - ref).max() <= ASM_TOL * max(np.abs(ref).max(), 1e-300)
    gm.close()


def test_noalloc_wrapper_rejects_wrong_buffers(dcgpu_lib):
    ini, _ = cases.small_gray_scott(n=8)
    gm = dcgpu_lib.Model(ini)
    x = gm.state()
    with pytest.raises(ValueError):
        gm.residual_noalloc(x[:-1], 0.0, 1.0, 0.0)
    for bad in (np.empty(gm.ndof - 1), np.empty(gm.ndof, np.float32), np.empty(2 * gm.ndof)[::2]):
        with pytest.raises(ValueError):
            gm.residual_noalloc(x, 0.0, 1.0, 0.0, out=bad)
    gm.close()


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
