"""Seeded synthetic DuneCopasi models (configuration text + optional initial state).

The benchmark configurations of this engine are synthetic: no public dataset is
involved.  Each generator returns ``(ini_text, init)`` where ``init`` is either None
(initial conditions come from ``initial.expression``) or a callable
``init(species_name, vertex_coords) -> values`` that gives seeded nodal values; the
caller writes them through the state-setting entry point.

  heat(n)            2D unit square, n x n cells, one species, D = 1e-2,
                     u0 = exp(-|x-(0.5,0.5)|^2/0.01), implicit Euler dt = 0.01
  gray_scott(n)      2D unit square, n x n cells, Gray-Scott (F=0.04, k=0.06,
                     D_u=2e-5, D_v=1e-5), u=1, v=0 + seeded U[0,0.1] in the central
                     0.1 x 0.1 patch, Alexander2 dt = 1
  two_compartment(n) inner disk r = 0.3 and outer annulus, 5 species each, 10 seeded
                     mass-action reactions per compartment (rates log-U[1e-2,1e1]),
                     D log-U[1e-4,1e-2], transmission 0.5 (u_in - u_out), U[0,1]
                     initial values, implicit Euler dt = 0.05
  cross_diffusion_3d(n)  unit cube, n^3 cubes x 6 tetrahedra, 3 species,
                     Michaelis-Menten reactions (Vmax 1, Km 0.5), full 3x3 scalar
                     cross-diffusion (diag 1e-2, off-diag +-1e-3 seeded signs), sum of
                     8 seeded Gaussians sigma = 0.05, Alexander2 dt = 0.01
"""

import numpy as np

SEED = 20261203


def _tso(scheme, dt, t_end, newton_rel=None, linear="UMFPack", extra="", dt_min=None):
    s = ["[model.time_step_operator]",
         "type = %s" % scheme,
         "time_begin = 0",
         "time_end = %r" % t_end,
         "time_step_initial = %r" % dt,
         "time_step_max = %r" % dt]
    if dt_min is not None:
        s.append("time_step_min = %r" % dt_min)
    s.append("[model.time_step_operator.linear_solver]")
    s.append("type = %s" % linear)
    if newton_rel is not None:
        s.append("[model.time_step_operator.nonlinear_solver]")
        s.append("convergence_condition.relative_tolerance = %r" % newton_rel)
    return "\n".join(s) + "\n" + extra


def heat(n=128, steps=100, dt=0.01, newton_rel=1e-10):
    ini = """
[grid]
dimension = 2
cells = {n} {n}

[compartments.domain]
expression = 1

[model.scalar_field.u]
compartment = domain
initial.expression = exp(-((position_x-0.5)^2 + (position_y-0.5)^2)/0.01)
storage.expression = 1
cross_diffusion.u.expression = 1e-2
""".format(n=n)
    ini += _tso("ImplicitEuler", dt, dt * steps, newton_rel)
    return ini, None


def gray_scott(n=512, steps=2000, dt=1.0, newton_rel=1e-10, seed=SEED, linear="UMFPack"):
    ini = """
[grid]
dimension = 2
cells = {n} {n}

[compartments.domain]
expression = 1

[parser_context.F]
type = constant
value = 0.04

[parser_context.k]
type = constant
value = 0.06

[model.scalar_field.u]
compartment = domain
initial.expression = 1
storage.expression = 1
reaction.expression = -u*v^2 + F*(1-u)
reaction.jacobian.u.expression = -v^2 - F
reaction.jacobian.v.expression = -2*u*v
cross_diffusion.u.expression = 2e-5

[model.scalar_field.v]
compartment = domain
storage.expression = 1
reaction.expression = u*v^2 - (F+k)*v
reaction.jacobian.u.expression = v^2
reaction.jacobian.v.expression = 2*u*v - (F+k)
cross_diffusion.v.expression = 1e-5
""".format(n=n)
    ini += _tso("Alexander2", dt, dt * steps, newton_rel, linear)

    def init(name, coords):
        if name == "u":
            return np.ones(coords.shape[0])
        rng = np.random.default_rng(seed)
        noise = rng.uniform(0.0, 0.1, size=coords.shape[0])
        patch = (np.abs(coords[:, 0] - 0.5) <= 0.05) & (np.abs(coords[:, 1] - 0.5) <= 0.05)
        return np.where(patch, noise, 0.0)

    return ini, init


def _mass_action(names, n_reactions, rng, dissipative=False):
    """Random mass-action network: returns {species: (rate expr, {wrt: jac expr})}.

    Reactions have one or two reactants and one or two products. With ``dissipative``
    a reaction has no more products than reactants and none of them is a reactant, so the
    total amount never grows (no autocatalysis, no finite-time blow-up).
    """
    terms = {s: [] for s in names}
    jac = {s: {} for s in names}
    for _ in range(n_reactions):
        if dissipative:
            nre = int(rng.integers(1, 3)) if len(names) > 1 else 1
            re = list(rng.choice(len(names), size=nre, replace=True))
            others = [i for i in range(len(names)) if i not in re]
            npr = min(int(rng.integers(0, nre + 1)), len(others))
            pr = list(rng.choice(others, size=npr, replace=True)) if npr else []
        else:
            nre = int(rng.integers(1, 3))
            npr = int(rng.integers(1, 3))
            re = list(rng.choice(len(names), size=nre, replace=True))
            pr = list(rng.choice(len(names), size=npr, replace=True))
        k = float(10.0 ** rng.uniform(-2.0, 1.0))
        kk = "%.17g" % k
        # rate = k * prod(reactants)
        rate = kk + "".join("*" + names[i] for i in re)
        # d rate / d species
        drate = {}
        for i in set(re):
            cnt = re.count(i)
            others = [names[j] for j in re if j != i]
            if cnt == 2:
                d = "%s*2*%s" % (kk, names[i])
            else:
                d = kk
            for o in others:
                d += "*" + o
            drate[names[i]] = d
        stoich = {}
        for i in re:
            stoich[names[i]] = stoich.get(names[i], 0) - 1
        for i in pr:
            stoich[names[i]] = stoich.get(names[i], 0) + 1
        for s, c in stoich.items():
            if c == 0:
                continue
            terms[s].append("%d*%s" % (c, rate))
            for w, d in drate.items():
                jac[s].setdefault(w, []).append("%d*%s" % (c, d))
    out = {}
    for s in names:
        r = " + ".join(terms[s]) if terms[s] else "0"
        js = {w: " + ".join(v) for w, v in jac[s].items()}
        out[s] = (r, js)
    return out


def two_compartment(n=1024, steps=200, dt=0.05, newton_rel=1e-10, seed=SEED, kt=0.5, ns=5,
                    n_reactions=10, linear="UMFPack"):
    rng = np.random.default_rng(seed)
    inner = ["a%d" % i for i in range(ns)]
    outer = ["b%d" % i for i in range(ns)]
    lines = ["[grid]", "dimension = 2", "cells = %d %d" % (n, n), "",
             "[compartments]",
             "inner.expression = ((position_x-0.5)^2 + (position_y-0.5)^2) < 0.09",
             "outer.expression = ((position_x-0.5)^2 + (position_y-0.5)^2) >= 0.09", ""]
    for comp, names, other in (("inner", inner, outer), ("outer", outer, inner)):
        net = _mass_action(names, n_reactions, rng)
        for i, s in enumerate(names):
            D = 10.0 ** rng.uniform(-4.0, -2.0)
            lines.append("[model.scalar_field.%s]" % s)
            lines.append("compartment = %s" % comp)
            lines.append("storage.expression = 1")
            lines.append("cross_diffusion.%s.expression = %.17g" % (s, D))
            r, js = net[s]
            if r != "0":
                lines.append("reaction.expression = %s" % r)
                for w, d in js.items():
                    lines.append("reaction.jacobian.%s.expression = %s" % (w, d))
            tgt = "outer" if comp == "inner" else "inner"
            o = other[i]
            lines.append("outflow.%s.expression = %r*(%s - %s)" % (tgt, kt, s, o))
            lines.append("outflow.%s.jacobian.%s.expression = %r" % (tgt, s, kt))
            lines.append("outflow.%s.jacobian.%s.expression = %r" % (tgt, o, -kt))
            lines.append("")
    ini = "\n".join(lines) + "\n" + _tso("ImplicitEuler", dt, dt * steps, newton_rel, linear)

    def init(name, coords):
        idx = (inner + outer).index(name)
        r = np.random.default_rng(seed + 1 + idx)
        return r.uniform(0.0, 1.0, size=coords.shape[0])

    return ini, init


def cross_diffusion_3d(n=128, steps=100, dt=0.01, newton_rel=1e-10, seed=SEED, linear="UMFPack"):
    rng = np.random.default_rng(seed)
    names = ["s0", "s1", "s2"]
    sign = rng.choice([-1.0, 1.0], size=(3, 3))
    centers = rng.uniform(0.2, 0.8, size=(8, 3))
    g = " + ".join("exp(-((position_x-%.17g)^2 + (position_y-%.17g)^2 + (position_z-%.17g)^2)/(2*0.05^2))"
                   % tuple(c) for c in centers)
    lines = ["[grid]", "dimension = 3", "cells = %d %d %d" % (n, n, n), "",
             "[compartments.domain]", "expression = 1", "",
             "[parser_context.Vmax]", "type = constant", "value = 1", "",
             "[parser_context.Km]", "type = constant", "value = 0.5", ""]
    # Michaelis-Menten chain s0 -> s1 -> s2 -> s0
    for i, s in enumerate(names):
        prev = names[(i - 1) % 3]
        lines.append("[model.scalar_field.%s]" % s)
        lines.append("compartment = domain")
        lines.append("storage.expression = 1")
        lines.append("initial.expression = %s" % (g if i == 0 else "0.5*(%s)" % g if i == 1 else "0.1"))
        lines.append("reaction.expression = Vmax*%s/(Km+%s) - Vmax*%s/(Km+%s)" % (prev, prev, s, s))
        lines.append("reaction.jacobian.%s.expression = Vmax*Km/(Km+%s)^2" % (prev, prev))
        lines.append("reaction.jacobian.%s.expression = -Vmax*Km/(Km+%s)^2" % (s, s))
        for j, w in enumerate(names):
            D = 1e-2 if i == j else 1e-3 * sign[i, j]
            lines.append("cross_diffusion.%s.expression = %.17g" % (w, D))
        lines.append("")
    ini = "\n".join(lines) + "\n" + _tso("Alexander2", dt, dt * steps, newton_rel, linear)
    return ini, None


def random_request(rng, n2d=(32, 256), n3d=(16, 40), steps=(10, 100), dt=0.05):
    """One serving request: 2D (N^2 cells) or 3D (N^3 cubes), one or two compartments,
    1-8 species per compartment, a seeded mass-action network, implicit Euler."""
    three_d = bool(rng.integers(0, 2))
    lo, hi = n3d if three_d else n2d
    n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
    two = bool(rng.integers(0, 2))
    ns = int(rng.integers(1, 9))
    nsteps = int(rng.integers(steps[0], steps[1] + 1))
    dim = 3 if three_d else 2
    lines = ["[grid]", "dimension = %d" % dim, "cells = " + " ".join([str(n)] * dim), ""]
    r2 = " + ".join("(position_%s-0.5)^2" % a for a in "xyz"[:dim])
    if two:
        lines += ["[compartments]", "inner.expression = (%s) < 0.09" % r2, "outer.expression = (%s) >= 0.09" % r2, ""]
        comps = [("inner", "a"), ("outer", "b")]
    else:
        lines += ["[compartments.domain]", "expression = 1", ""]
        comps = [("domain", "a")]
    for comp, prefix in comps:
        names = ["%s%d" % (prefix, i) for i in range(ns)]
        net = _mass_action(names, max(1, 2 * ns), rng, dissipative=True)
        for i, s in enumerate(names):
            lines.append("[model.scalar_field.%s]" % s)
            lines.append("compartment = %s" % comp)
            lines.append("storage.expression = 1")
            lines.append("initial.expression = %.6g" % rng.uniform(0.0, 1.0))
            lines.append("cross_diffusion.%s.expression = %.17g" % (s, 10.0 ** rng.uniform(-4.0, -2.0)))
            r, js = net[s]
            if r != "0":
                lines.append("reaction.expression = %s" % r)
                for w, d in js.items():
                    lines.append("reaction.jacobian.%s.expression = %s" % (w, d))
            if two:
                other = ("b" if prefix == "a" else "a") + str(i)
                tgt = "outer" if comp == "inner" else "inner"
                lines.append("outflow.%s.expression = 0.5*(%s - %s)" % (tgt, s, other))
                lines.append("outflow.%s.jacobian.%s.expression = 0.5" % (tgt, s))
                lines.append("outflow.%s.jacobian.%s.expression = -0.5" % (tgt, other))
            lines.append("")
    ini = "\n".join(lines) + "\n" + _tso("ImplicitEuler", dt, dt * nsteps, 1e-10, dt_min=dt * 1e-3)
    return ini


def serving_stream(n_requests=512, lam=50.0, seed=SEED, **kw):
    """Poisson arrivals (rate lam per second) of random requests: [(arrival_s, ini)]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n_requests):
        t += rng.exponential(1.0 / lam)
        out.append((t, random_request(rng, **kw)))
    return out


def apply_init(model_like, init, coords_of, setter):
    """Helper: evaluate ``init`` per species on its vertices and hand the values to ``setter``."""
    if init is None:
        return
    for name in model_like:
        setter(name, init(name, coords_of(name)))
