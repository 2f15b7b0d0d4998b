"""CPU tests of the C ABI library: it loads, exports every declared symbol, and its host
expression compiler agrees with the oracle's evaluator (no GPU compute calls)."""

import ctypes
import math
import os
import re

import numpy as np
import pytest

from oracle import expr as E
from oracle.ini import ParameterTree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "dcgpu.h")).read()
    return sorted(set(re.findall(r"\b(dc_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(dcgpu_lib):
    lib = ctypes.CDLL(dcgpu_lib.LIB_PATH)
    declared = _declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(dcgpu_lib.EXPORTED)


def test_model_create_without_gpu_fails_loudly(dcgpu_lib):
    """No CPU fallback: without a CUDA device model creation reports DC_ERR_CUDA."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(dcgpu_lib.DcError) as ei:
        dcgpu_lib.Model("[grid]\ncells = 2 2\n[compartments.d]\nexpression = 1\n"
                        "[model.scalar_field.u]\ncompartment = d\n")
    assert ei.value.status in (5, 7)


CONTEXT = """
[parser_context.F]
type = constant
value = 0.04
[parser_context.bump]
type = function
expression = x, y: 0.5*exp(-100*(x^2 + y^2))
[parser_context.tab]
type = interpolation
domain = -1 0 0.5 2
range = 3 1 4 -2
"""

EXPRESSIONS = [
    "u*v^2 + F*(1-u)", "-u*v^2 + F*(1-u)", "-v^2 - F", "2*u*v - (F+0.06)", "u^3 - v^-1",
    "u^2^0.5", "-u^2", "exp(-u)*sin(v) + cos(u*v)", "log(u) + ln(v) + log10(u) + log2(v)",
    "sqrt(u*u + v*v)", "abs(u - v) + sign(u - v)", "u < v ? u : v", "u > 0.5 && v < 0.5",
    "u >= 0.5 || v <= 0.5", "!(u > v)", "min(u, v, 0.3) + max(u, v, 0.3)", "sum(u, v, 1) / avg(u, v)",
    "pow(u, 2.5) + atan2(v, u) + hypot(u, v)", "bump(0.25 - u, 0.75 - v)", "tab(u) + tab(v - 1)",
    "u % 0.3", "floor(u*10) + ceil(v*10) + round(u*7) + trunc(-v*3)", "tanh(u) + sinh(v) + cosh(u)",
    "asin(u/2) + acos(v/2) + atan(u)", "1e-3*u + .5*v + 2.5e+1", "u == v", "u = u", "u <> v",
    "1 ? u : v", "0 ? u : v", "(u+v)*(u-v)/(u*v + 1)", "F*u^7", "u^-3", "erf(u) + erfc(v)",
    "u and v or 0", "not u", "u*v*u*v*u*v", "rint(u*4.5)",
]


@pytest.mark.parametrize("text", EXPRESSIONS)
def test_engine_compiler_matches_oracle(dcgpu_lib, text):
    ctx = E.Context(ParameterTree.from_text(CONTEXT).sub("parser_context"))
    ex = E.Expression(text, ctx)
    rng = np.random.default_rng(7)
    for _ in range(5):
        u, v = rng.uniform(0.05, 0.95, size=2)
        ref = float(ex({"u": u, "v": v}))
        got = dcgpu_lib.expr_eval(text, {"u": u, "v": v}, CONTEXT)
        if math.isnan(ref):
            assert math.isnan(got)
        else:
            assert got == pytest.approx(ref, rel=1e-13, abs=1e-13), text


@pytest.mark.parametrize("bad", ["1 +", "f(", "unknown_symbol + 1", "sin(1, 2)", "1 ? 2", "(1"])
def test_engine_compiler_rejects_bad_expressions(dcgpu_lib, bad):
    with pytest.raises(dcgpu_lib.DcError) as ei:
        dcgpu_lib.expr_eval(bad, {"u": 1.0})
    assert ei.value.status == 4


def test_nested_user_function_rejected(dcgpu_lib):
    ctx = "[parser_context.f]\ntype=function\nexpression=x: x\n[parser_context.g]\ntype=function\nexpression=x: f(x)\n"
    with pytest.raises(dcgpu_lib.DcError):
        dcgpu_lib.expr_eval("g(1)", {}, ctx)


# ------------------------------------------------------------------ parser-context extras

def _tiff_context(path, name="img"):
    return "[parser_context.%s]\ntype = tiff\npath = %s\n" % (name, path)


@pytest.mark.parametrize("bits,photometric,big_endian,compression,predictor", [
    (8, 1, False, "none", False), (16, 0, True, "lzw", True), (32, 1, True, "packbits", False),
    (16, 1, False, "lzw", False), (8, 0, False, "lzw", True)])
def test_engine_tiff_matches_oracle(dcgpu_lib, tmp_path, bits, photometric, big_endian, compression, predictor):
    """The engine's TIFF reader and position lookup against the oracle's, bit for bit, over
    positions inside, on the edges of and outside the image."""
    import tiff_files as TF
    from oracle.tiff import TiffImage
    path = str(tmp_path / "im.tif")
    v = TF.seeded_image(23, 37, bits, seed=bits)
    TF.write_tiff(path, v, bits=bits, photometric=photometric, big_endian=big_endian, compression=compression,
                  predictor=predictor, resolution=(37, 1), position=(1, 8), rows_per_strip=6)
    im = TiffImage(path)
    ctx = _tiff_context(path)
    rng = np.random.default_rng(bits)
    pts = list(rng.uniform(-0.3, 1.5, size=(60, 2))) + [(0.125, 0.125), (1.125, 0.75), (0.5, 1.0 / 37 + 0.125)]
    for x, y in pts:
        got = dcgpu_lib.expr_eval("img(x, y)", {"x": x, "y": y}, ctx)
        assert got == float(im(x, y)), (x, y)


def test_engine_tiff_errors(dcgpu_lib, tmp_path):
    import tiff_files as TF
    p4 = str(tmp_path / "four.tif")
    TF.write_tiff(p4, np.full((3, 4), 5, dtype=np.uint64), bits=4)
    rgb = str(tmp_path / "rgb.tif")
    TF.write_tiff(rgb, np.ones((3, 3), dtype=np.uint64), photometric=2)
    nores = str(tmp_path / "nores.tif")
    TF.write_tiff(nores, np.ones((3, 3), dtype=np.uint64), res_tags=False)
    for path, msg in [(p4, "Encoding with 4 bits not implemented"), (rgb, "must be in grayscale"),
                      (nores, "negative resolution"), (str(tmp_path / "none.tif"), "does not exists")]:
        with pytest.raises(dcgpu_lib.DcError) as ei:
            dcgpu_lib.expr_eval("img(0.5, 0.5)", {}, _tiff_context(path))
        assert ei.value.status == 4 and msg in str(ei.value)


TABULATED = """
[parser_context.k]
type = constant
value = 3
[parser_context.ramp]
type = interpolation
domain = 0 0.5 2
range = 1 2 0
[parser_context.f]
type = function
expression = s: k*sin(s) + ramp(s)
interpolate = true
interpolation.intervals = 37
interpolation.domain.s = -0.5 2
interpolation.out_of_bounds = %s
"""


@pytest.mark.parametrize("mode", ["clamp", "error"])
def test_engine_tabulated_function_matches_oracle(dcgpu_lib, mode):
    """interpolate = true: the grid values agree with the oracle's to rounding, and the
    lookup picks the same grid value (the reference's left-endpoint step) everywhere."""
    text = TABULATED % mode
    ctx = E.Context(ParameterTree.from_text(text).sub("parser_context"))
    f = ctx.functions["f"]
    xs = list(np.linspace(-0.5, 2.0, 38)) + list(np.random.default_rng(3).uniform(-1.0, 2.5, 80)) + [float("nan")]
    for x in xs:
        ref = float(E.Expression("f(x)", ctx)({"x": np.array(x)}))
        got = dcgpu_lib.expr_eval("f(x)", {"x": x}, text)
        if math.isnan(ref):
            assert math.isnan(got), x
        else:
            assert got == pytest.approx(ref, rel=1e-14, abs=1e-15), x
    assert f.n == 37


@pytest.mark.parametrize("edit,msg", [
    (("interpolation.intervals = 37", "interpolation.intervals = 100001"), "too big"),
    (("interpolation.intervals = 37", "interpolation.intervals = 0"), "At least one interval"),
    (("interpolation.domain.s = -0.5 2", "interpolation.domain.s = 2 -0.5"), "not ordered"),
    (("expression = s: k*sin(s) + ramp(s)", "expression = s, t: s*t"), "Cannot interpolate"),
])
def test_engine_tabulated_function_config_errors(dcgpu_lib, edit, msg):
    with pytest.raises(dcgpu_lib.DcError) as ei:
        dcgpu_lib.expr_eval("f(0.5)", {}, (TABULATED % "clamp").replace(*edit))
    assert ei.value.status == 4 and msg in str(ei.value)


def test_engine_interpolation_is_exact_lerp(dcgpu_lib):
    """Interpolation tables: std::lower_bound and std::lerp, the same bits as the oracle's
    restatement, at the nodes, between them, outside and for NaN."""
    text = "[parser_context.tab]\ntype = interpolation\ndomain = -1 0 0 0.5 2\nrange = 3 -1 2 4 -2\n"
    ctx = E.Context(ParameterTree.from_text(text).sub("parser_context"))
    for x in [-2.0, -1.0, -0.3, 0.0, 1e-17, 0.25, 0.5, 0.9999, 2.0, 7.0, float("nan")]:
        ref = float(ctx.functions["tab"](np.array(x)))
        got = dcgpu_lib.expr_eval("tab(x)", {"x": x}, text)
        assert got == ref, x


@pytest.mark.parametrize("typ,msg", [("random_field", "random fields"), ("cell_data", "cell data"),
                                     ("wavelet", "Unknown type")])
def test_engine_unsupported_context_types(dcgpu_lib, typ, msg):
    with pytest.raises(dcgpu_lib.DcError) as ei:
        dcgpu_lib.expr_eval("1", {}, "[parser_context.q]\ntype = %s\n" % typ)
    assert ei.value.status == 4 and msg in str(ei.value)


def test_run_time_compilation_selftest(dcgpu_lib):
    """NVRTC compiles the generated volume kernels of a synthetic compartment that covers
    every volume term kind, in 2D and 3D (no GPU needed)."""
    ok, msg = dcgpu_lib.jit_selftest()
    assert ok, msg


def test_server_entry_points_check_arguments(dcgpu_lib):
    """The batched-server entry points reject bad arguments before touching a device."""
    lib = ctypes.CDLL(dcgpu_lib.LIB_PATH)
    out = ctypes.c_void_p()
    # unknown flag bits
    assert lib.dc_server_create_ex(ctypes.c_int64(1 << 30), 4, 1 << 5, ctypes.byref(out)) == 6
    assert out.value is None
    # null handles and outputs
    stats = dcgpu_lib.BatchStats()
    assert lib.dc_server_batch_stats(None, ctypes.byref(stats)) == 6
    buf = ctypes.create_string_buffer(64)
    assert lib.dc_server_batch_tuning(None, buf, ctypes.c_size_t(len(buf))) == 6
    assert lib.dc_server_create_ex(ctypes.c_int64(1 << 30), 4, 0, None) == 6
