"""CPU tests of the oracle's parser-context extras against the reference's semantics:
grayscale TIFF images (src/dune/copasi/common/tiff_grayscale.cc, tiff_file.cc, and the
reference's test/dune/copasi/common/tiff_grayscale.cc cases), functions tabulated with
``interpolate = true`` and interpolation tables (src/dune/copasi/parser/context.cc)."""

import math
import os

import numpy as np
import pytest

from oracle import expr as E
from oracle.ini import ParameterTree
from oracle.tiff import TiffError, TiffImage

import tiff_files as TF


def _ctx(text):
    return E.Context(ParameterTree.from_text(text).sub("parser_context"))


# ------------------------------------------------------------------ TIFF reader


@pytest.mark.parametrize("bits", [8, 16, 32])
@pytest.mark.parametrize("photometric", [0, 1])
@pytest.mark.parametrize("big_endian", [False, True])
@pytest.mark.parametrize("compression,predictor", [("none", False), ("packbits", False), ("lzw", False),
                                                   ("lzw", True)])
def test_tiff_values_and_scaling(tmp_path, bits, photometric, big_endian, compression, predictor):
    """Samples come back exactly and are scaled as the reference scales them: v / 2^bits,
    and (2^bits - v) / 2^bits for WhiteIsZero images (tiff_grayscale.cc:46-52)."""
    v = TF.seeded_image(13, 17, bits, seed=bits + photometric)
    path = str(tmp_path / "im.tif")
    TF.write_tiff(path, v, bits=bits, photometric=photometric, big_endian=big_endian, compression=compression,
                  predictor=predictor, rows_per_strip=5)
    im = TiffImage(path)
    assert (im.rows, im.cols, im.bits) == (13, 17, bits)
    mx = float(1 << bits)
    expect = v.astype(float) / mx if photometric == 1 else (mx - v.astype(float)) / mx
    assert np.array_equal(im.px, expect)


def test_tiff_lzw_table_resets(tmp_path):
    """Enough distinct data for the LZW code table to fill and be cleared several times."""
    rng = np.random.default_rng(5)
    v = rng.integers(0, 1 << 16, size=(96, 96), dtype=np.uint64)
    path = str(tmp_path / "big.tif")
    TF.write_tiff(path, v, bits=16, compression="lzw")
    assert np.array_equal(TiffImage(path).px, v.astype(float) / 65536.0)


def test_tiff_64_bit_divisor(tmp_path):
    """64-bit samples: the reference's 1 << 64 shift count wraps to 0 in its x86-64 build,
    so the divisor is 1."""
    v = np.array([[1, 2], [3, 4]], dtype=np.uint64)
    path = str(tmp_path / "im64.tif")
    TF.write_tiff(path, v, bits=64)
    assert np.array_equal(TiffImage(path).px, v.astype(float))


def test_tiff_unsupported_encoding(tmp_path):
    """The reference's UnsupportedEncoding case: a 4-bit image is rejected."""
    path = str(tmp_path / "im4.tif")
    TF.write_tiff(path, np.full((4, 6), 7, dtype=np.uint64), bits=4)
    with pytest.raises(TiffError, match="Encoding with 4 bits not implemented"):
        TiffImage(path)


def test_tiff_rejections(tmp_path):
    v = np.ones((3, 3), dtype=np.uint64)
    p = str(tmp_path / "rgb.tif")
    TF.write_tiff(p, v, photometric=2)
    with pytest.raises(TiffError, match="must be in grayscale"):
        TiffImage(p)
    p = str(tmp_path / "nores.tif")
    TF.write_tiff(p, v, res_tags=False)
    with pytest.raises(TiffError, match="negative resolution"):
        TiffImage(p)
    p = str(tmp_path / "zero.tif")
    TF.write_tiff(p, v, resolution=(0, 1))
    with pytest.raises(TiffError, match="negative resolution"):
        TiffImage(p)
    with pytest.raises(TiffError, match="does not exists"):
        TiffImage(str(tmp_path / "missing.tif"))


def test_tiff_compare_16_vs_8_bits(tmp_path):
    """The reference's Compare16vs8Bits case: the same picture stored with 8 and 16 bits
    per sample agrees within 2/255 per pixel and per position lookup (72 pixels per unit)."""
    v8 = TF.seeded_image(20, 30, 8, seed=3)
    v16 = v8 * np.uint64(257)
    p8, p16 = str(tmp_path / "a8.tif"), str(tmp_path / "a16.tif")
    TF.write_tiff(p8, v8, bits=8, resolution=(72, 1))
    TF.write_tiff(p16, v16, bits=16, resolution=(72, 1))
    a, b = TiffImage(p8), TiffImage(p16)
    thr = 2.0 / 255.0
    assert (a.rows, a.cols) == (b.rows, b.cols)
    assert np.max(np.abs(a.px - b.px)) <= thr
    i, j = np.mgrid[0:a.rows, 0:a.cols]
    x, y = j / 72.0, i / 72.0
    assert np.max(np.abs(a(x, y) - b(x, y))) <= thr


def test_tiff_position_lookup(tmp_path):
    """tiff_grayscale.cc:94-108: column = trunc(x_res (x - x_off)), scanline = rows - 1 -
    trunc(y_res (y - y_off)) (unsigned), both clamped into the image; single precision."""
    rows, cols = 6, 9
    v = (np.arange(rows * cols, dtype=np.uint64).reshape(rows, cols) * 3) % 256
    p = str(tmp_path / "pos.tif")
    TF.write_tiff(p, v, bits=8, resolution=(4, 1), position=(1, 2))   # 4 px per unit, offset 0.5
    im = TiffImage(p)
    assert im.x_res == np.float32(4) and im.x_off == np.float32(0.5)
    px = v.astype(float) / 256.0
    # inside: x = 0.5 + (c + 0.5)/4, y = 0.5 + (k + 0.5)/4 -> column c, scanline rows-1-k
    for c in range(cols):
        for k in range(rows):
            x, y = 0.5 + (c + 0.5) / 4.0, 0.5 + (k + 0.5) / 4.0
            assert im(x, y) == px[rows - 1 - k, c]
    # past the right / top edge: clamped to the last column / (wrapped, then clamped) row
    assert im(100.0, 0.6) == px[rows - 1, cols - 1]
    assert im(0.6, 100.0) == px[rows - 1, 0]
    # just below the offset: truncation towards zero gives column / row index 0
    assert im(0.45, 0.45) == px[rows - 1, 0]
    # far below: the x86-64 conversion wraps to a huge unsigned value, clamped to the last column
    assert im(-10.0, 0.6) == px[rows - 1, cols - 1]


def test_tiff_function_in_expressions(tmp_path):
    v = TF.seeded_image(8, 8, 16, seed=9)
    p = str(tmp_path / "f.tif")
    TF.write_tiff(p, v, bits=16, resolution=(8, 1))
    ctx = _ctx("""
[parser_context.A]
type = tiff
path = %s
[parser_context.g]
type = function
expression = x, y: 2*A(x, y)
""" % p)
    im = TiffImage(p)
    xs, ys = np.array([0.1, 0.55, 0.99]), np.array([0.2, 0.7, 0.05])
    assert np.array_equal(E.Expression("1000*A(position_x, position_y)", ctx)({"position_x": xs, "position_y": ys}),
                          1000 * im(xs, ys))
    # a user function may call a context-independent function (an image)
    assert np.array_equal(E.Expression("g(position_x, position_y)", ctx)({"position_x": xs, "position_y": ys}),
                          2 * im(xs, ys))


# ------------------------------------------------------------------ tabulated functions


TAB = """
[parser_context.k]
type = constant
value = 3
[parser_context.f]
type = function
expression = s: k*s^2
interpolate = true
interpolation.intervals = 10
interpolation.domain.s = 0 2
interpolation.out_of_bounds = %s
"""


def test_tabulated_function_is_left_endpoint_step():
    """context.cc:251-266: the values g_i = f(d0 + i (d1 - d0)/N) and a lookup that returns
    g at the integer part of (x - d0) N / (d1 - d0)."""
    ctx = _ctx(TAB % "clamp")
    f = ctx.functions["f"]
    xs = np.linspace(0.0, 2.0, 11)
    assert np.array_equal(f.g, 3 * xs ** 2)
    ev = lambda x: float(E.Expression("f(u)", ctx)({"u": np.array(x)}))
    assert ev(0.0) == 0.0
    assert ev(0.35) == f.g[1]          # interval [0.2, 0.4): left end point
    assert ev(0.4) == f.g[2]
    assert ev(1.99) == f.g[9]
    assert ev(2.0) == f.g[10]
    # clamp: outside the domain the end values, NaN to the first
    assert ev(-5.0) == f.g[0] and ev(7.0) == f.g[10] and ev(float("nan")) == f.g[0]


def test_tabulated_function_error_mode():
    ctx = _ctx(TAB % "error")
    ev = lambda x: float(E.Expression("f(u)", ctx)({"u": np.array(x)}))
    assert ev(1.0) == 3.0
    assert math.isnan(ev(2.5)) and math.isnan(ev(-0.1)) and math.isnan(ev(float("nan")))


@pytest.mark.parametrize("edit,msg", [
    (("interpolation.intervals = 10", "interpolation.intervals = 100001"), "too big"),
    (("interpolation.intervals = 10", "interpolation.intervals = 0"), "At least one interval"),
    (("interpolation.domain.s = 0 2", "interpolation.domain.s = 2 2"), "not ordered"),
    (("out_of_bounds = clamp", "out_of_bounds = wrap"), "Not known"),
    (("expression = s: k*s^2", "expression = s, t: k*s^2*t"), "Cannot interpolate"),
])
def test_tabulated_function_config_errors(edit, msg):
    with pytest.raises(E.ExprError, match=msg):
        _ctx((TAB % "clamp").replace(*edit))


def test_tabulated_function_default_domain_and_intervals():
    ctx = _ctx("""
[parser_context.h]
type = function
expression = z: sin(z)
interpolate = true
interpolation.out_of_bounds = clamp
""")
    f = ctx.functions["h"]
    assert f.n == 1000 and (f.d0, f.d1) == (0.0, 1.0)
    assert f.g[500] == pytest.approx(math.sin(0.5), rel=0, abs=1e-15)


def test_user_function_may_not_call_a_tabulated_one():
    with pytest.raises(E.ExprError):
        _ctx((TAB % "clamp") + """
[parser_context.g]
type = function
expression = y: f(y)
""")


# ------------------------------------------------------------------ interpolation tables


def test_interpolation_table_lower_bound_and_lerp():
    """context.cc:77-90: std::lower_bound over the domain, the first range value up to and
    at the first domain point, the last one past the end, std::lerp in between."""
    ctx = _ctx("""
[parser_context.tab]
type = interpolation
domain = 0 1 1 2 4
range = -1 3 5 5 -7
""")
    tab = ctx.functions["tab"]
    x = np.array([-1.0, 0.0, 0.5, 1.0, 1.5, 3.0, 4.0, 9.0, float("nan")])
    got = tab(x)
    # at x = 1, lower_bound finds the first 1 (range 3); between the equal points there is none
    assert np.array_equal(got, [-1.0, -1.0, 1.0, 3.0, 5.0, -1.0, -7.0, -7.0, -1.0])


def test_lerp_is_exact_at_the_ends_and_monotonic():
    a = np.array([0.1, -2.0, 1e300, 3.0])
    b = np.array([0.7, 5.0, -1e300, 3.0])
    assert np.array_equal(E.lerp_exact(a, b, 1.0), b)
    assert np.array_equal(E.lerp_exact(a, b, 0.0), a)
    t = np.linspace(0, 1, 101)
    vals = E.lerp_exact(0.1, 0.7, t)
    assert np.all(np.diff(vals) >= 0) and vals[-1] == 0.7


@pytest.mark.parametrize("typ,msg", [("random_field", "random fields"), ("cell_data", "cell data"),
                                     ("wavelet", "Unknown type")])
def test_unsupported_context_types(typ, msg):
    with pytest.raises(E.ExprError, match=msg):
        _ctx("[parser_context.q]\ntype = %s\n" % typ)
