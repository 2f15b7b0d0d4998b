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
