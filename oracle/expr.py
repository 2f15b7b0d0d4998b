"""Math-expression parser and vectorised evaluator (oracle side, test infrastructure).

Restates the expression semantics the reference exposes through its parser backends
(src/dune/copasi/parser/mu.cc -- muParser is the default backend,
src/dune/copasi/parser/factory.cc:25-35 -- and src/dune/copasi/parser/exprtk.cc),
as documented in doc/docusaurus/docs/math_expr.mdx:
  * binary operators with muParser precedence, lowest first:
      ``? :`` < ``||``/``or`` < ``&&``/``and`` < comparisons < ``+ -`` (and prefix sign)
      < ``* / %`` < ``^`` (right associative);
  * comparisons and logic return 1.0 / 0.0; ``=`` is equality (ExprTk reading);
  * built-in functions of muParser (sin ... atanh, log2, log10, log = ln, exp, sqrt,
    sign, rint, abs, variadic min/max/sum/avg) plus the ExprTk ones the reference's
    examples use (pow, atan2, floor, ceil, round, trunc, hypot, erf, erfc, if, clamp);
  * user functions from ``parser_context.{tkn}.type=function``
    (src/dune/copasi/parser/context.cc:56-66,289-330): ``args: body`` with at most four
    arguments, which may not call other user functions;
  * 1-D ``interpolation`` tables (context.cc:68-92): linear, clamped to the end values.

Evaluation is vectorised with numpy: every free symbol maps to a scalar or an array.
"""

import math
import re

import numpy as np

from .tiff import TiffError, TiffImage


class ExprError(ValueError):
    pass


_TOKEN_RE = re.compile(
    r"\s*(?:"
    r"(?P<num>(?:\d+\.?\d*|\.\d+)(?:[eE][+\-]?\d+)?)"
    r"|(?P<id>[A-Za-z_][A-Za-z0-9_]*)"
    r"|(?P<op>\|\||&&|==|!=|<>|<=|>=|[-+*/%^<>=!?:(),])"
    r")")


def tokenize(text):
    pos = 0
    out = []
    text = text.strip()
    while pos < len(text):
        m = _TOKEN_RE.match(text, pos)
        if not m or m.end() == pos:
            raise ExprError("unexpected character at %d in %r" % (pos, text))
        if m.group("num") is not None:
            out.append(("num", float(m.group("num"))))
        elif m.group("id") is not None:
            out.append(("id", m.group("id")))
        else:
            out.append(("op", m.group("op")))
        pos = m.end()
        while pos < len(text) and text[pos].isspace():
            pos += 1
    out.append(("end", None))
    return out


# precedence levels (muParser: prLOR=1, prLAND=2, prCMP=5, prADD_SUB=6, prMUL_DIV=7, prPOW=8)
_BINARY = {
    "||": 1, "or": 1,
    "&&": 2, "and": 2,
    "==": 5, "=": 5, "!=": 5, "<>": 5, "<": 5, "<=": 5, ">": 5, ">=": 5,
    "+": 6, "-": 6,
    "*": 7, "/": 7, "%": 7,
    "^": 8,
}
_CANON = {"or": "||", "and": "&&", "=": "==", "<>": "!="}

FUNCTIONS = {
    # name: (min_args, max_args or None for variadic)
    "sin": (1, 1), "cos": (1, 1), "tan": (1, 1), "asin": (1, 1), "acos": (1, 1),
    "atan": (1, 1), "sinh": (1, 1), "cosh": (1, 1), "tanh": (1, 1), "asinh": (1, 1),
    "acosh": (1, 1), "atanh": (1, 1), "log2": (1, 1), "log10": (1, 1), "log": (1, 1),
    "ln": (1, 1), "exp": (1, 1), "sqrt": (1, 1), "sign": (1, 1), "rint": (1, 1),
    "abs": (1, 1), "floor": (1, 1), "ceil": (1, 1), "round": (1, 1), "trunc": (1, 1),
    "erf": (1, 1), "erfc": (1, 1),
    "pow": (2, 2), "atan2": (2, 2), "hypot": (2, 2),
    "min": (1, None), "max": (1, None), "sum": (1, None), "avg": (1, None),
    "if": (3, 3), "clamp": (3, 3),
}

BUILTIN_CONSTANTS = {"_pi": math.pi, "_e": math.e, "true": 1.0, "false": 0.0}


class Parser:
    """Recursive-descent parser producing a tuple AST.

    Node forms: ('num', v) | ('var', name) | ('neg', a) | ('not', a)
                | ('bin', op, a, b) | ('tern', c, a, b) | ('call', name, [args])
    """

    def __init__(self, text):
        self.toks = tokenize(text)
        self.i = 0
        self.text = text

    def peek(self):
        return self.toks[self.i]

    def take(self):
        t = self.toks[self.i]
        self.i += 1
        return t

    def expect(self, op):
        t = self.take()
        if t != ("op", op):
            raise ExprError("expected %r in %r" % (op, self.text))

    def parse(self):
        node = self.ternary()
        if self.peek()[0] != "end":
            raise ExprError("trailing input in %r" % self.text)
        return node

    def ternary(self):
        cond = self.binary(1)
        if self.peek() == ("op", "?"):
            self.take()
            a = self.ternary()
            self.expect(":")
            b = self.ternary()
            return ("tern", cond, a, b)
        return cond

    def _binop(self):
        t = self.peek()
        if t[0] == "op" and t[1] in _BINARY:
            return t[1]
        if t[0] == "id" and t[1] in ("and", "or"):
            return t[1]
        return None

    def binary(self, min_prec):
        lhs = self.unary()
        while True:
            op = self._binop()
            if op is None:
                return lhs
            prec = _BINARY[op]
            if prec < min_prec:
                return lhs
            self.take()
            if op == "^":
                rhs = self.binary_rhs_pow()
            else:
                rhs = self.binary(prec + 1)
            lhs = ("bin", _CANON.get(op, op), lhs, rhs)

    def binary_rhs_pow(self):
        # right associative: a^b^c = a^(b^c); the exponent may carry a prefix sign
        return self.binary(8)

    def unary(self):
        t = self.peek()
        if t == ("op", "-"):
            self.take()
            # prefix sign has the precedence of binary +/- (muParser prINFIX = 6)
            return ("neg", self.binary(7))
        if t == ("op", "+"):
            self.take()
            return self.binary(7)
        if t == ("op", "!") or t == ("id", "not"):
            self.take()
            return ("not", self.binary(7))
        return self.primary()

    def primary(self):
        t = self.take()
        if t[0] == "num":
            return ("num", t[1])
        if t == ("op", "("):
            node = self.ternary()
            self.expect(")")
            return node
        if t[0] == "id":
            name = t[1]
            if self.peek() == ("op", "("):
                self.take()
                args = []
                if self.peek() != ("op", ")"):
                    args.append(self.ternary())
                    while self.peek() == ("op", ","):
                        self.take()
                        args.append(self.ternary())
                self.expect(")")
                return ("call", name, args)
            return ("var", name)
        raise ExprError("unexpected token %r in %r" % (t, self.text))


def parse(text):
    return Parser(text).parse()


def free_symbols(node, out=None):
    if out is None:
        out = set()
    kind = node[0]
    if kind == "var":
        out.add(node[1])
    elif kind in ("neg", "not"):
        free_symbols(node[1], out)
    elif kind == "bin":
        free_symbols(node[2], out)
        free_symbols(node[3], out)
    elif kind == "tern":
        for c in node[1:]:
            free_symbols(c, out)
    elif kind == "call":
        for a in node[2]:
            free_symbols(a, out)
    return out


def called_functions(node, out=None):
    if out is None:
        out = set()
    kind = node[0]
    if kind in ("neg", "not"):
        called_functions(node[1], out)
    elif kind == "bin":
        called_functions(node[2], out)
        called_functions(node[3], out)
    elif kind == "tern":
        for c in node[1:]:
            called_functions(c, out)
    elif kind == "call":
        out.add(node[1])
        for a in node[2]:
            called_functions(a, out)
    return out


class UserFunction:
    def __init__(self, args, body):
        self.args = args
        self.body = body


def lerp_exact(a, b, t):
    """std::lerp, the algorithm of C++ proposal P0811R3: exact when a and b straddle zero,
    b at t == 1, monotonic and never past b."""
    a, b, t = np.broadcast_arrays(np.asarray(a, float), np.asarray(b, float), np.asarray(t, float))
    with np.errstate(invalid="ignore"):
        straddle = ((a <= 0) & (b >= 0)) | ((a >= 0) & (b <= 0))
        r1 = t * b + (1.0 - t) * a
        x = a + t * (b - a)
        r2 = np.where((t > 1) == (b > a), np.where(b < x, x, b), np.where(b > x, x, b))
        r2 = np.where(t == 1, b, r2)
    return np.where(straddle, r1, r2)


class Interpolation:
    def __init__(self, domain, rng):
        self.domain = np.asarray(domain, float)
        self.range = np.asarray(rng, float)

    def __call__(self, x):
        """context.cc:77-90: std::lower_bound over the domain; the first range value up to
        the first domain point (and for NaN), the last one past the end, std::lerp between."""
        X, Y = self.domain, self.range
        x = np.asarray(x, float)
        d = np.clip(np.searchsorted(X, np.where(np.isnan(x), X[0], x), side="left"), 1, len(X) - 1)
        with np.errstate(invalid="ignore", divide="ignore"):
            t = (x - X[d - 1]) / (X[d] - X[d - 1])
        mid = lerp_exact(Y[d - 1], Y[d], t)
        out = np.where(X[len(X) - 1] < x, Y[-1], mid)
        return np.where(~(X[0] < x), Y[0], out)


class FunctionTable:
    """A 1-argument parser-context function with ``interpolate = true`` (context.cc:237-280):
    its values g on intervals + 1 uniform points of the domain.  The reference's lookup
    blends g[i] with g[j] where both are the integer part of (x - d0) * intervals /
    (d1 - d0), so its result is g at that index exactly: a left-endpoint step function.
    out_of_bounds = clamp clamps x into the domain (NaN to d0); out_of_bounds = error
    raises MathError in the reference, and gives NaN here (the GPU path then fails the
    Newton step)."""

    def __init__(self, name, fn, intervals, d0, d1, clamp, constants, indep):
        self.name = name
        self.d0, self.d1, self.clamp = float(d0), float(d1), bool(clamp)
        self.n = int(intervals)
        nf = float(self.n)
        width = (self.d1 - self.d0) / nf
        self.ctn = nf / (self.d1 - self.d0)
        xs = self.d0 + np.arange(self.n + 1, dtype=float) * width
        env = dict(constants)
        env[fn.args[0]] = xs
        self.g = np.broadcast_to(np.asarray(evaluate(fn.body, env, indep), float), xs.shape).copy()

    def __call__(self, x):
        x = np.asarray(x, float)
        if self.clamp:
            x = np.where(x > self.d0, x, self.d0)
            x = np.where(self.d1 < x, self.d1, x)
            bad = np.zeros(x.shape, bool)
        else:
            bad = ~((x >= self.d0) & (x <= self.d1))
            x = np.where(bad, self.d0, x)
        i = np.minimum(((x - self.d0) * self.ctn).astype(np.int64), self.n)
        return np.where(bad, np.nan, self.g[i])


def _independent(functions):
    return {k: v for k, v in (functions or {}).items() if isinstance(v, (Interpolation, TiffImage))}


def parse_function_definition(text):
    """Split ``a, b: body`` (context.cc parse_function_expression) into (args, body AST)."""
    colon = text.find(":")
    if colon < 0:
        raise ExprError("function definition needs 'args: expression': %r" % text)
    head = text[:colon].strip()
    args = [a.strip() for a in head.split(",")] if head else []
    if len(args) > 4:
        raise ExprError("user functions take at most 4 arguments")
    return UserFunction(args, parse(text[colon + 1:]))


def _as_bool(x):
    return np.asarray(x) != 0.0


def evaluate(node, env, functions=None):
    """Evaluate AST ``node`` with numpy broadcasting.

    ``env`` maps symbol names to scalars/arrays; ``functions`` maps user function
    names to UserFunction / Interpolation objects.
    """
    functions = functions or {}
    kind = node[0]
    if kind == "num":
        return node[1]
    if kind == "var":
        name = node[1]
        if name in env:
            return env[name]
        if name in BUILTIN_CONSTANTS:
            return BUILTIN_CONSTANTS[name]
        raise ExprError("unknown symbol %r" % name)
    if kind == "neg":
        return -np.asarray(evaluate(node[1], env, functions), dtype=float)
    if kind == "not":
        return np.where(_as_bool(evaluate(node[1], env, functions)), 0.0, 1.0)
    if kind == "tern":
        c = evaluate(node[1], env, functions)
        a = evaluate(node[2], env, functions)
        b = evaluate(node[3], env, functions)
        return np.where(_as_bool(c), a, b)
    if kind == "bin":
        op = node[1]
        a = np.asarray(evaluate(node[2], env, functions), dtype=float)
        b = np.asarray(evaluate(node[3], env, functions), dtype=float)
        if op == "+":
            return a + b
        if op == "-":
            return a - b
        if op == "*":
            return a * b
        if op == "/":
            return a / b
        if op == "%":
            return np.fmod(a, b)
        if op == "^":
            return np.power(a, b)
        if op == "==":
            return np.where(a == b, 1.0, 0.0)
        if op == "!=":
            return np.where(a != b, 1.0, 0.0)
        if op == "<":
            return np.where(a < b, 1.0, 0.0)
        if op == "<=":
            return np.where(a <= b, 1.0, 0.0)
        if op == ">":
            return np.where(a > b, 1.0, 0.0)
        if op == ">=":
            return np.where(a >= b, 1.0, 0.0)
        if op == "&&":
            return np.where(_as_bool(a) & _as_bool(b), 1.0, 0.0)
        if op == "||":
            return np.where(_as_bool(a) | _as_bool(b), 1.0, 0.0)
        raise ExprError("unknown operator %r" % op)
    if kind == "call":
        name = node[1]
        args = [np.asarray(evaluate(a, env, functions), dtype=float) for a in node[2]]
        if name in functions:
            f = functions[name]
            if isinstance(f, (Interpolation, FunctionTable)):
                if len(args) != 1:
                    raise ExprError("interpolation %r takes one argument" % name)
                return f(args[0])
            if isinstance(f, TiffImage):
                if len(args) != 2:
                    raise ExprError("tiff function %r takes two arguments" % name)
                return f(args[0], args[1])
            if len(args) != len(f.args):
                raise ExprError("function %r takes %d arguments" % (name, len(f.args)))
            inner = dict(env)
            for an, av in zip(f.args, args):
                inner[an] = av
            # a user function's body sees the context-independent functions (interpolation
            # tables, images) but no other expression function (context.cc:283-330,
            # math_expr.mdx:325-347)
            return evaluate(f.body, inner, _independent(functions))
        if name not in FUNCTIONS:
            raise ExprError("unknown function %r" % name)
        lo, hi = FUNCTIONS[name]
        if len(args) < lo or (hi is not None and len(args) > hi):
            raise ExprError("wrong argument count for %r" % name)
        return _builtin(name, args)
    raise ExprError("bad node %r" % (node,))


def _builtin(name, a):
    x = a[0]
    simple = {
        "sin": np.sin, "cos": np.cos, "tan": np.tan, "asin": np.arcsin, "acos": np.arccos,
        "atan": np.arctan, "sinh": np.sinh, "cosh": np.cosh, "tanh": np.tanh,
        "asinh": np.arcsinh, "acosh": np.arccosh, "atanh": np.arctanh, "log2": np.log2,
        "log10": np.log10, "log": np.log, "ln": np.log, "exp": np.exp, "sqrt": np.sqrt,
        "sign": np.sign, "rint": np.rint, "abs": np.abs, "floor": np.floor, "ceil": np.ceil,
        "trunc": np.trunc,
    }
    if name in simple:
        return simple[name](x)
    if name == "round":
        # ExprTk round: half away from zero
        return np.where(x >= 0, np.floor(x + 0.5), np.ceil(x - 0.5))
    if name == "erf":
        return np.vectorize(math.erf, otypes=[float])(x)
    if name == "erfc":
        return np.vectorize(math.erfc, otypes=[float])(x)
    if name == "pow":
        return np.power(x, a[1])
    if name == "atan2":
        return np.arctan2(x, a[1])
    if name == "hypot":
        return np.hypot(x, a[1])
    if name == "min":
        r = x
        for y in a[1:]:
            r = np.minimum(r, y)
        return r
    if name == "max":
        r = x
        for y in a[1:]:
            r = np.maximum(r, y)
        return r
    if name == "sum":
        r = x
        for y in a[1:]:
            r = r + y
        return r
    if name == "avg":
        r = x
        for y in a[1:]:
            r = r + y
        return r / len(a)
    if name == "if":
        return np.where(_as_bool(a[0]), a[1], a[2])
    if name == "clamp":
        return np.minimum(np.maximum(a[1], a[0]), a[2])
    raise ExprError(name)


_ZERO_RE = re.compile(r"-?([0]+)?([\.]?)([0]+)?")
_FLOAT_RE = re.compile(r"-?([0-9]+)?([\.]?)([0-9]+)?")


def is_zero_literal(text):
    """functor_factory_parser.impl.hh:121-124: empty or all-zero expression => no functor."""
    return text == "" or _ZERO_RE.fullmatch(text) is not None


def constant_literal(text):
    """functor_factory_parser.impl.hh:125-128: a bare float literal bypasses the parser."""
    if _FLOAT_RE.fullmatch(text) is not None:
        return float(text)
    return None


class Context:
    """The ``parser_context`` section: constants, user functions and interpolation tables."""

    def __init__(self, cfg=None):
        self.constants = {}
        self.functions = {}
        if cfg is None:
            return
        tabulate = []
        for name in cfg.sub_keys():
            sub = cfg.sub(name)
            typ = sub.get("type")
            if typ == "constant":
                self.constants[name] = float(sub["value"])
            elif typ == "tiff":
                try:
                    self.functions[name] = TiffImage(sub["path"])
                except TiffError as e:
                    raise ExprError(str(e))
            elif typ == "random_field":
                # context.cc:93-160 needs the optional parafields library
                raise ExprError("Library was compiled without random fields support")
            elif typ == "cell_data":
                raise ExprError("cell data is not implemented")
            elif typ == "function":
                if sub.get_bool("interpolate", False):
                    tabulate.append((name, sub))
                    continue
                self.functions[name] = parse_function_definition(sub["expression"])
            elif typ == "interpolation":
                dom = sub.get_floats("domain")
                rng = sub.get_floats("range")
                if dom != sorted(dom):
                    raise ExprError("The interpolation domain must be sorted")
                if len(dom) < 2 or len(dom) != len(rng):
                    raise ExprError("Interpolation range and domain must match (>= 2 points)")
                self.functions[name] = Interpolation(dom, rng)
            else:
                raise ExprError("Unknown type %s" % typ)
        # context.cc:237-280: 1-argument functions replaced by their values on a grid; the
        # bodies see constants, interpolation tables and images only
        indep = _independent(self.functions)
        made = {}
        for name, sub in tabulate:
            fn = parse_function_definition(sub["expression"])
            if len(fn.args) != 1:
                raise ExprError("Cannot interpolate '%s' function with %d arguments" % (name, len(fn.args)))
            nested = called_functions(fn.body) & (set(self.functions) - set(indep))
            if nested:
                raise ExprError("user functions may not call user functions: %s" % nested)
            intervals = int(sub.get("interpolation.intervals", "1000"))
            if intervals > 100000:
                raise ExprError("Number of interpolation intervals is too big!")
            if intervals < 1:
                raise ExprError("At least one interval is required in function %s" % name)
            dom = sub.get_floats("interpolation.domain." + fn.args[0]) if sub.has_key(
                "interpolation.domain." + fn.args[0]) else [0.0, 1.0]
            if dom[0] >= dom[1]:
                raise ExprError("Domain arguments (%g, %g) of function %s are not ordered" % (dom[0], dom[1], name))
            ooo = sub.get("interpolation.out_of_bounds", "error")
            if ooo not in ("clamp", "error"):
                raise ExprError("Not known '%s.interpolation.out_of_bounds = %s'" % (name, ooo))
            made[name] = FunctionTable(name, fn, intervals, dom[0], dom[1], ooo == "clamp", self.constants, indep)
        self.functions.update(made)
        # user function bodies see the constants and the context-independent functions
        for f in self.functions.values():
            if isinstance(f, UserFunction):
                nested = called_functions(f.body) & (set(self.functions) - set(indep))
                if nested:
                    raise ExprError("user functions may not call user functions: %s" % nested)

    def env(self):
        return dict(self.constants)


class Expression:
    """A compiled expression bound to a parser context."""

    def __init__(self, text, context=None):
        self.text = text.strip()
        self.context = context or Context()
        self.literal = constant_literal(self.text)
        self.ast = None if self.literal is not None else parse(self.text)

    def __call__(self, env):
        if self.literal is not None:
            return self.literal
        full = self.context.env()
        full.update(env)
        for k, f in self.context.functions.items():
            if isinstance(f, UserFunction):
                # bodies may reference constants; arguments shadow them
                pass
        return evaluate(self.ast, full, self.context.functions)

    def symbols(self):
        if self.ast is None:
            return set()
        s = free_symbols(self.ast)
        for fname in called_functions(self.ast):
            f = self.context.functions.get(fname)
            if isinstance(f, UserFunction):
                s |= free_symbols(f.body) - set(f.args)
        return s
