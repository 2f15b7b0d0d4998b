"""P1 residual / Jacobian assembly of the diffusion-reaction operator (oracle, test infrastructure).

Restates dune/copasi/model/diffusion_reaction/local_operator.hh for P1 simplices:
  * volume residual, localAssembleVolume                 local_operator.hh:417-491
  * analytic volume Jacobian                             local_operator.hh:541-707
  * numerical (finite difference) volume Jacobian        local_operator.hh:713-765
  * skeleton / boundary outflow residual                 local_operator.hh:777-971,1398-1415
  * analytic skeleton / boundary outflow Jacobian        local_operator.hh:973-1203,1417-1436
and the functor tree of dune/copasi/model/diffusion_reaction/local_equations.hh:617-700
built through dune/copasi/model/functor_factory_parser.impl.hh:25-182.

Quadrature: order 2*k = 2 for P1 (local_operator.hh:128-139).  Element rule: the
symmetric 3-point (triangle) / 4-point (tetrahedron) interior rules; face rule: 2-point
Gauss-Legendre on edges, the 3-point rule on triangles.  (The dune-geometry tables are
not vendored; these are the standard symmetric order-2 rules.)

Deliberate deviation (documented): on a compartment interface, values of species that
exist only on the other side are evaluated at the physical quadrature point through
the other element's own local coordinates.  The reference binds the other element's
basis with the inside projection (local_operator.hh:887-890,1104-1107), which depends
on the grid manager's local vertex numbering.
"""

import math

import numpy as np

from . import expr as E

AXES = ("x", "y", "z")


def element_rule(dim):
    if dim == 2:
        pts = np.array([[2.0 / 3.0, 1.0 / 6.0], [1.0 / 6.0, 2.0 / 3.0], [1.0 / 6.0, 1.0 / 6.0]])
        w = np.full(3, 1.0 / 6.0)
    else:
        a = 0.5854101966249685
        b = 0.1381966011250105
        pts = np.array([[b, b, b], [a, b, b], [b, a, b], [b, b, a]])
        w = np.full(4, 1.0 / 24.0)
    return pts, w


def reduce_rule(dim):
    """Rule of the reduce operators, which ask dune-geometry for order 4 (reduce.hh:179-180).

    dune-geometry's tables are not available here; these are symmetric rules whose orbit
    parameters solve the moment equations: triangles, 6 points (two (a, a, 1-2a) orbits),
    exact to degree 4; tetrahedra, 14 points (two (a, a, a, 1-3a) orbits and one
    (b, b, 1/2-b, 1/2-b) orbit), exact to degree 5.  Points are listed by barycentric
    coordinates (lambda_0..lambda_d); returns (reference points [nq, d], weights summing
    to the reference volume).
    """
    if dim == 2:
        a1, a2 = 0.4459484909159645, 0.09157621350977077
        w1, w2 = 0.11169079483900554, 0.05497587182766112
        bary = []
        for a in (a1, a2):
            bary += [[a, a, 1 - 2 * a], [a, 1 - 2 * a, a], [1 - 2 * a, a, a]]
        w = [w1] * 3 + [w2] * 3
    else:
        a1, a2, b = 0.0927352503108912, 0.3108859192633006, 0.0455037041256496
        w1, w2, w3 = 0.01224884051939366, 0.01878132095300264, 0.007091003462846911
        bary = []
        for a in (a1, a2):
            bary += [[a, a, a, 1 - 3 * a], [a, a, 1 - 3 * a, a], [a, 1 - 3 * a, a, a], [1 - 3 * a, a, a, a]]
        c = 0.5 - b
        bary += [[b, b, c, c], [b, c, b, c], [b, c, c, b], [c, b, b, c], [c, b, c, b], [c, c, b, b]]
        w = [w1] * 4 + [w2] * 4 + [w3] * 6
    bary = np.array(bary)
    return bary[:, 1:].copy(), np.array(w)


def face_rule(dim):
    """Rule on the reference face (dim-1 simplex)."""
    if dim == 2:
        g = 0.5 / math.sqrt(3.0)
        return np.array([[0.5 - g], [0.5 + g]]), np.array([0.5, 0.5])
    return element_rule(2)


def p1_values(xi):
    """P1 basis on the reference simplex at points xi[..., d] -> [..., d+1]."""
    return np.concatenate([1.0 - xi.sum(axis=-1, keepdims=True), xi], axis=-1)


def p1_ref_gradients(dim):
    g = np.zeros((dim + 1, dim))
    g[0, :] = -1.0
    for k in range(dim):
        g[k + 1, k] = 1.0
    return g


def geometry(coords, cells):
    """Affine geometry: (v0 [n,d], B [n,d,d] columns v_k - v0, det, physical P1 gradients [n,d+1,d])."""
    dim = coords.shape[1]
    v0 = coords[cells[:, 0]]
    B = np.stack([coords[cells[:, k]] - v0 for k in range(1, dim + 1)], axis=2)
    det = np.linalg.det(B)
    Binv = np.linalg.inv(B)
    G = np.einsum("ak,nkj->naj", p1_ref_gradients(dim), Binv)
    return v0, B, det, G


# ----------------------------------------------------------------------------------------
# functor tree (local_equations.hh + functor_factory_parser.impl.hh)
# ----------------------------------------------------------------------------------------

def _scalar(cfg, ctx):
    """parse_scalar_expression: None when the expression is empty or all zeros."""
    text = (cfg.get("expression", "") or "").strip()
    if E.is_zero_literal(text):
        return None
    return E.Expression(text, ctx)


class ScalarFn:
    def __init__(self, value, jac):
        self.value = value      # Expression
        self.jac = jac          # list of (species name, Expression)


class VectorFn:
    def __init__(self, comps, jac):
        self.comps = comps      # list of Expression-or-None, one per axis
        self.jac = jac          # list of (species name, [Expression-or-None]*dim)


class TensorFn:
    """make_tensor_apply: 'scalar' -> d*g ; 'tensor' -> T g (functor_factory_parser.impl.hh:65-112)."""

    def __init__(self, kind, data):
        self.kind = kind
        self.data = data        # Expression, or dim x dim list of Expression-or-None

    def apply(self, env, g):
        if self.kind == "scalar":
            return np.asarray(self.data(env), float)[..., None] * g
        dim = g.shape[-1]
        out = np.zeros(g.shape)
        for i in range(dim):
            acc = 0.0
            for j in range(dim):
                t = self.data[i][j]
                if t is not None:
                    acc = acc + np.asarray(t(env), float) * g[..., j]
            out[..., i] = acc
        return out


def _make_vector(cfg, ctx, dim):
    comps = []
    active = False
    for i in range(dim):
        c = _scalar(cfg.sub(AXES[i]), ctx)
        comps.append(c)
        active |= c is not None
    return comps if active else None


def _make_tensor(cfg, ctx, dim):
    typ = cfg.get("type", "scalar")
    if typ == "scalar":
        s = _scalar(cfg, ctx)
        return None if s is None else TensorFn("scalar", s)
    if typ == "tensor":
        data = [[None] * dim for _ in range(dim)]
        active = False
        for i in range(dim):
            for j in range(dim):
                key = AXES[i] + AXES[j]
                if cfg.has_sub(key):
                    data[i][j] = _scalar(cfg.sub(key), ctx)
                    active |= data[i][j] is not None
        return TensorFn("tensor", data) if active else None
    raise ValueError("unknown diffusion type %r" % typ)


class SpeciesEq:
    def __init__(self, name, comp, local):
        self.name = name
        self.comp = comp
        self.local = local
        self.storage = None
        self.reaction = None
        self.velocity = None
        self.cross_diffusion = []   # list of (wrt name, TensorFn, [(v name, TensorFn)])
        self.outflow = {}           # compartment index -> ScalarFn


def build_equations(sf_cfg, species, comp_names, ctx, dim):
    """Functor tree per species (local_equations.hh:617-700)."""
    all_names = [s.name for s in species]
    eqs = []
    for sp in species:
        eq = SpeciesEq(sp.name, sp.comp, sp.local)
        cfg = sf_cfg.sub(sp.name)

        def scalar_fn(c):
            v = _scalar(c, ctx)
            jac = []
            jc = c.sub("jacobian")
            for w in all_names:
                if jc.has_sub(w):
                    j = _scalar(jc.sub(w), ctx)
                    if j is not None:
                        jac.append((w, j))
            # a differentiable function exists when its value functor exists
            return None if v is None else ScalarFn(v, jac)

        if cfg.has_sub("cross_diffusion"):
            cd = cfg.sub("cross_diffusion")
            for w in all_names:
                if cd.has_sub(w):
                    dc = cd.sub(w)
                    t = _make_tensor(dc, ctx, dim)
                    if t is None:
                        continue
                    jac = []
                    jc = dc.sub("jacobian")
                    for v in all_names:
                        if jc.has_sub(v):
                            jt = _make_tensor(jc.sub(v), ctx, dim)
                            if jt is not None:
                                jac.append((v, jt))
                    eq.cross_diffusion.append((w, t, jac))
        if cfg.has_sub("reaction"):
            eq.reaction = scalar_fn(cfg.sub("reaction"))
        if cfg.has_sub("velocity"):
            vc = cfg.sub("velocity")
            comps = _make_vector(vc, ctx, dim)
            if comps is not None:
                jac = []
                jc = vc.sub("jacobian")
                for w in all_names:
                    if jc.has_sub(w):
                        jv = _make_vector(jc.sub(w), ctx, dim)
                        if jv is not None:
                            jac.append((w, jv))
                eq.velocity = VectorFn(comps, jac)
        if cfg.has_sub("storage"):
            eq.storage = scalar_fn(cfg.sub("storage"))
        if cfg.has_sub("outflow"):
            oc = cfg.sub("outflow")
            for ci, cname in enumerate(comp_names):
                if oc.has_sub(cname):
                    f = scalar_fn(oc.sub(cname))
                    if f is not None:
                        eq.outflow[ci] = f
        eqs.append(eq)
    return eqs


def _ev(ex, env, shape):
    return np.broadcast_to(np.asarray(ex(env), float), shape)
