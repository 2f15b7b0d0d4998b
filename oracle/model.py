"""Model, assembly driver, Newton, Runge-Kutta and stepper (oracle, test infrastructure).

Restates, on top of oracle.fem:
  * DOF layout (dune/copasi/model/diffusion_reaction/model_multi_compartment_traits.hh:16-23,
    model_single_compartment_traits.hh:18-30): compartment-major; inside a compartment
    vertex-major with the species of that compartment interleaved;
  * initial condition: nodal interpolation of ``initial.expression`` at time_begin
    (dune/copasi/model/make_initial.hh:24-90, interpolate.hh:21-78);
  * the Runge-Kutta stage residual  sum_j a_ij M(u_j, t+d_j dt) + b_ij dt A(u_j, t+d_j dt)
    with M the mass (storage) form and A the stiffness form
    (dune/copasi/model/make_step_operator.hh:408-443, PDELab one-step parameters);
  * Newton with the reference's settings (make_step_operator.hh:246-288): relative tolerance
    1e-4 on the SQUARED l2 norm by default, iteration range {0, 40}, adaptive linear
    tolerance, optional absolute tolerance; the linear branch (make_step_operator.hh:210-245)
    for ``is_linear`` models is one defect-correction solve per stage;
  * SimpleAdaptiveStepper::do_step, TimeStepper::evolve and snap_to_time
    (dune/copasi/common/stepper.hh:95-239,337-368) with the CLI defaults of
    src/dune_copasi.cc:384-402 (decrease 0.5, increase 1.1).
The linear solve is direct (scipy SuperLU), standing in for the reference's default
UMFPack (dune/copasi/solver/istl/factory/direct.hh:9-12).  For meshes whose factorisation
does not fit in memory (3D and 1024^2 multi-species systems) ``linear="iterative"`` replaces
it with BiCGSTAB + Jacobi inside iterative refinement to a relative true residual of 1e-13,
or of the rounding floor of the fp64 residual r - J z where that lies above (accepted up to
1e-10; the direct solve's role in Newton: an essentially exact correction).  Assembly runs over at
most ``chunk`` cells at a time, so the element arrays of large meshes stay bounded.
"""

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import expr as E
from . import fem as F
from .ini import ParameterTree
from .mesh import Mesh, mark_compartments

AXES = ("x", "y", "z")


# --------------------------------------------------------------------------------------
# time-stepping schemes (PDELab one-step parameter form: rows i=1..s over stages j=0..s)
# --------------------------------------------------------------------------------------

def rk_scheme(name):
    if name == "ImplicitEuler":
        return [[-1.0, 1.0]], [[0.0, 1.0]], [0.0, 1.0]
    if name == "ExplicitEuler":
        return [[-1.0, 1.0]], [[1.0, 0.0]], [0.0, 1.0]
    if name == "Alexander2":
        a = 1.0 - 0.5 * math.sqrt(2.0)
        return ([[-1.0, 1.0, 0.0], [-1.0, 0.0, 1.0]],
                [[0.0, a, 0.0], [0.0, 1.0 - a, a]],
                [0.0, a, 1.0])
    if name == "Heun":
        return ([[-1.0, 1.0, 0.0], [-0.5, -0.5, 1.0]],
                [[1.0, 0.0, 0.0], [0.0, 0.5, 0.0]],
                [0.0, 1.0, 1.0])
    if name == "Shu3":
        return ([[-1.0, 1.0, 0.0, 0.0], [-0.75, -0.25, 1.0, 0.0], [-1.0 / 3.0, 0.0, -2.0 / 3.0, 1.0]],
                [[1.0, 0.0, 0.0, 0.0], [0.0, 0.25, 0.0, 0.0], [0.0, 0.0, 2.0 / 3.0, 0.0]],
                [0.0, 1.0, 0.5, 1.0])
    if name == "RungeKutta4":
        return ([[-1.0, 1.0, 0.0, 0.0, 0.0], [-1.0, 0.0, 1.0, 0.0, 0.0],
                 [-1.0, 0.0, 0.0, 1.0, 0.0], [-1.0, 0.0, 0.0, 0.0, 1.0]],
                [[0.5, 0.0, 0.0, 0.0, 0.0], [0.0, 0.5, 0.0, 0.0, 0.0],
                 [0.0, 0.0, 1.0, 0.0, 0.0], [1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0.0]],
                [0.0, 0.5, 0.5, 1.0, 1.0])
    if name == "FractionalStepTheta":
        th = 1.0 - 0.5 * math.sqrt(2.0)
        thp = 1.0 - 2.0 * th
        al = 2.0 - math.sqrt(2.0)
        be = 1.0 - al
        return ([[-1.0, 1.0, 0.0, 0.0], [0.0, -1.0, 1.0, 0.0], [0.0, 0.0, -1.0, 1.0]],
                [[th * be, th * al, 0.0, 0.0], [0.0, thp * al, thp * be, 0.0],
                 [0.0, 0.0, th * be, th * al]],
                [0.0, th, 1.0 - th, 1.0])
    if name == "Alexander3":
        al = 0.4358665215084590
        tau2 = (1.0 + al) / 2.0
        b1 = -(6.0 * al * al - 16.0 * al + 1.0) / 4.0
        b2 = (6.0 * al * al - 20.0 * al + 5.0) / 4.0
        return ([[-1.0, 1.0, 0.0, 0.0], [-1.0, 0.0, 1.0, 0.0], [-1.0, 0.0, 0.0, 1.0]],
                [[0.0, al, 0.0, 0.0], [0.0, tau2 - al, al, 0.0], [0.0, b1, b2, al]],
                [0.0, al, tau2, 1.0])
    raise ValueError("Not known time stepping type %r" % name)


# --------------------------------------------------------------------------------------
# dune FloatCmp (relativeWeak, epsilon = 8 * DBL_EPSILON)
# --------------------------------------------------------------------------------------

_EPS = 8.0 * np.finfo(float).eps


def f_eq(a, b):
    return abs(a - b) <= _EPS * max(abs(a), abs(b))


def f_le(a, b):
    return a < b or f_eq(a, b)


def f_lt(a, b):
    return a < b and not f_eq(a, b)


def f_gt(a, b):
    return a > b and not f_eq(a, b)


class Species:
    def __init__(self, name, comp, local):
        self.name = name
        self.comp = comp
        self.local = local


class StepFailed(Exception):
    pass


class OracleModel:
    """Everything between an ini text and a time-evolved state, on the CPU."""

    #: cells assembled at once (bounds the memory of the element arrays on big meshes)
    chunk = 1 << 19
    #: matrix entries collected before they are summed into the global matrix
    flush_entries = 1 << 26
    #: relative true-residual target of the iterative solve, and the largest relative residual
    #: it accepts once refinement sweeps stop reducing it (the rounding floor of r - J z)
    iterative_rtol = 1e-13
    iterative_floor = 1e-10

    def __init__(self, ini_text, overrides=None, linear="direct"):
        if linear not in ("direct", "iterative"):
            raise ValueError("linear must be 'direct' or 'iterative'")
        self.linear = linear
        self.cfg = ParameterTree.from_text(ini_text, overrides)
        cfg = self.cfg
        self.ctx = E.Context(cfg.sub("parser_context") if cfg.has_sub("parser_context") else None)
        self.mesh = Mesh.from_config(cfg.sub("grid"))
        self.dim = self.mesh.dim
        self.comp_names, self.comp_mask = mark_compartments(self.mesh, cfg.sub("compartments"), self.ctx)
        mcfg = cfg.sub("model")
        self.mcfg = mcfg
        sf = mcfg.sub("scalar_field")
        # species per compartment in configuration order
        self.species = []
        per_comp = [[] for _ in self.comp_names]
        for name in sf.sub_keys():
            cname = sf.sub(name).get("compartment")
            if cname is None or cname == "":
                continue
            if cname not in self.comp_names:
                raise ValueError("species %r refers to unknown compartment %r" % (name, cname))
            ci = self.comp_names.index(cname)
            per_comp[ci].append(name)
        for ci, names in enumerate(per_comp):
            for k, n in enumerate(names):
                self.species.append(Species(n, ci, k))
        if not self.species:
            raise ValueError("Basis has dimension 0")
        self.per_comp = per_comp
        self.ns = [len(p) for p in per_comp]
        self.is_linear = mcfg.get_bool("is_linear", False)
        jt = mcfg.get("jacobian.type", "analytical")
        if jt not in ("analytical", "numerical"):
            raise ValueError("model.jacobian.type must be analytical or numerical")
        self.numerical_jacobian = (jt == "numerical") and not self.is_linear
        self.fd_eps = mcfg.get_float("jacobian.epsilon", 1e-7)
        self.eqs = F.build_equations(sf, self.species, self.comp_names, self.ctx, self.dim)
        self.eq_by_name = {e.name: e for e in self.eqs}
        self.has_outflow = any(e.outflow for e in self.eqs)
        self._setup_dofs()
        self._setup_geometry()
        self._setup_faces()
        self._setup_constraints()
        self._pattern_cache = {}
        tso = mcfg.sub("time_step_operator")
        self.tso = tso

    # ---------------------------------------------------------------- layout
    def _setup_dofs(self):
        m = self.mesh
        self.comp_vertices = []
        self.comp_vloc = []
        self.comp_offset = []
        off = 0
        for ci in range(len(self.comp_names)):
            els = np.nonzero(self.comp_mask[ci])[0]
            verts = np.unique(m.cells[els].ravel()) if self.ns[ci] else np.zeros(0, np.int64)
            vloc = np.full(m.nv, -1, np.int64)
            vloc[verts] = np.arange(verts.shape[0])
            self.comp_vertices.append(verts)
            self.comp_vloc.append(vloc)
            self.comp_offset.append(off)
            off += verts.shape[0] * self.ns[ci]
        self.ndof = off

    def dof(self, sp_, vertices):
        ci = sp_.comp
        return self.comp_offset[ci] + self.comp_vloc[ci][vertices] * self.ns[ci] + sp_.local

    def _setup_geometry(self):
        m = self.mesh
        self.v0, self.B, self.det, self.G = F.geometry(m.coords, m.cells)
        self.qpts, self.qw = F.element_rule(self.dim)
        self.phi = F.p1_values(self.qpts)                       # [nq, d+1]
        self.xq = self.v0[:, None, :] + np.einsum("nij,qj->nqi", self.B, self.qpts)
        self.factor = np.abs(self.det)[:, None] * self.qw[None, :]
        self.vol = np.abs(self.det) / math.factorial(self.dim)
        # group elements by their compartment signature
        sig = np.zeros(m.ne, np.int64)
        for ci in range(len(self.comp_names)):
            sig |= self.comp_mask[ci].astype(np.int64) << ci
        self.elem_sig = sig
        self.groups = []
        for s in np.unique(sig):
            if s == 0:
                continue
            els = np.nonzero(sig == s)[0]
            comps = [ci for ci in range(len(self.comp_names)) if (s >> ci) & 1]
            sps = [sp_ for sp_ in self.species if sp_.comp in comps]
            if sps:
                self.groups.append((els, sps))

    def _setup_faces(self):
        m = self.mesh
        fv, e0, l0, e1, l1 = m.faces()
        sig = self.elem_sig
        interior = e1 >= 0
        inter = interior & (sig[e0] != sig[np.where(interior, e1, 0)])
        bnd = ~interior
        keep = inter | (bnd if self.has_outflow else np.zeros_like(bnd))
        self.face_vertices = fv[keep]
        self.face_e0 = e0[keep]
        self.face_l0 = l0[keep]
        self.face_e1 = e1[keep]
        self.face_l1 = l1[keep]

    def _setup_constraints(self):
        """Dirichlet (translation) constraints, model/constraints.hh:51-199.

        constrain.boundary / constrain.skeleton expressions of a species are evaluated once
        (time = NaN) at the P1 vertices of the faces of the species' compartment: a face with
        no neighbour cell in the compartment is a boundary face (in_boundary = 1, normal
        pointing out of the compartment cell); a face with the compartment on both sides is a
        skeleton face (in_skeleton = 1, evaluated from both cells, normal out of each) and
        constrains only vertices that lie on no boundary face (constraints.hh:178).  A value
        of no_value (DBL_MAX) leaves the vertex free.  When several faces give a vertex a
        value, the first in (sorted vertex ids, inside before outside) order wins.
        P1 has no cell-interior DOFs, so constrain.volume never applies (constraints.hh:104).
        Result: self.cons_dofs (sorted), self.cons_vals.
        """
        m = self.mesh
        d = self.dim
        sf = self.mcfg.sub("scalar_field")
        todo = []
        for sp_ in self.species:
            c = sf.sub(sp_.name)
            for kind in ("boundary", "skeleton"):
                key = "constrain." + kind
                if c.has_sub(key):
                    ex = F._scalar(c.sub(key), self.ctx)
                    if ex is not None:
                        todo.append((sp_, kind, ex))
        self.cons_dofs = np.zeros(0, np.int64)
        self.cons_vals = np.zeros(0)
        if not todo:
            return
        fv, e0, _l0, e1, _l1 = m.faces()
        has1 = e1 >= 0
        e1s = np.where(has1, e1, 0)
        dofs, vals = [], []
        for sp_, kind, ex in todo:
            mask = self.comp_mask[sp_.comp]
            in0 = mask[e0]
            in1 = has1 & mask[e1s]
            bnd = in0 ^ in1
            bverts = np.zeros(m.nv, bool)
            bverts[fv[bnd].ravel()] = True
            if kind == "boundary":
                sel = np.nonzero(bnd)[0]
                sides = [(sel, np.where(in0[sel], e0[sel], e1s[sel]))]
                flags = (1.0, 0.0)
            else:
                sel = np.nonzero(in0 & in1)[0]
                sides = [(sel, e0[sel]), (sel, e1s[sel])]
                flags = (0.0, 1.0)
            # candidate (face order, side, vertex) triples
            cand_v, cand_pos, cand_n, cand_vol, cand_key = [], [], [], [], []
            for side, (fs, cells) in enumerate(sides):
                fvc = m.coords[fv[fs]]                       # [k, d, d]
                f0 = fvc[:, 0, :]
                T = np.stack([fvc[:, j, :] - f0 for j in range(1, d)], axis=2)
                if d == 2:
                    nrm = np.stack([T[:, 1, 0], -T[:, 0, 0]], axis=1)
                    meas = np.linalg.norm(T[:, :, 0], axis=1)
                else:
                    nrm = np.cross(T[:, :, 0], T[:, :, 1])
                    meas = 0.5 * np.linalg.norm(nrm, axis=1)
                nrm = nrm / np.linalg.norm(nrm, axis=1)[:, None]
                ctr = m.coords[m.cells[cells]].mean(axis=1)
                flip = np.einsum("ni,ni->n", nrm, f0 - ctr) < 0
                nrm[flip] *= -1.0
                for j in range(d):
                    v = fv[fs, j]
                    cand_v.append(v)
                    cand_pos.append(m.coords[v])
                    cand_n.append(nrm)
                    cand_vol.append(meas)
                    cand_key.append(fs * 2 + side)
            v = np.concatenate(cand_v)
            pos = np.concatenate(cand_pos)
            nr = np.concatenate(cand_n)
            fvol = np.concatenate(cand_vol)
            key = np.concatenate(cand_key)
            if kind == "skeleton":
                keep = ~bverts[v]
                v, pos, nr, fvol, key = v[keep], pos[keep], nr[keep], fvol[keep], key[keep]
            if v.size == 0:
                continue
            env = {"time": float("nan"), "integration_factor": 0.0, "in_volume": 0.0,
                   "in_boundary": flags[0], "in_skeleton": flags[1], "no_value": np.finfo(float).max,
                   "entity_volume": fvol}
            for j in range(3):
                env["position_" + AXES[j]] = pos[:, j] if j < d else 0.0
                env["normal_" + AXES[j]] = nr[:, j] if j < d else 0.0
            val = np.broadcast_to(np.asarray(ex(env), float), v.shape).copy()
            ok = val != np.finfo(float).max
            v, val, key = v[ok], val[ok], key[ok]
            order = np.lexsort((key, v))                     # by vertex, then face order
            v, val = v[order], val[order]
            first = np.ones(v.shape[0], bool)
            first[1:] = v[1:] != v[:-1]
            dofs.append(self.dof(sp_, v[first]))
            vals.append(val[first])
        if dofs:
            dd = np.concatenate(dofs)
            vv = np.concatenate(vals)
            # a species may carry both kinds: the boundary entry comes first and wins
            order = np.argsort(dd, kind="stable")
            dd, vv = dd[order], vv[order]
            first = np.ones(dd.shape[0], bool)
            first[1:] = dd[1:] != dd[:-1]
            self.cons_dofs = dd[first]
            self.cons_vals = vv[first]

    def apply_constraints(self, x):
        """x with the constrained entries set to their values (a copy)."""
        if self.cons_dofs.size == 0:
            return x
        x = x.copy()
        x[self.cons_dofs] = self.cons_vals
        return x

    def _constrain_residual(self, r):
        if self.cons_dofs.size:
            r[self.cons_dofs] = 0.0
        return r

    def _constrain_jacobian(self, J):
        """Constrained rows become unit rows."""
        if self.cons_dofs.size == 0:
            return J
        J = J.tocsr(copy=True)
        mask = np.zeros(self.ndof, bool)
        mask[self.cons_dofs] = True
        rows = np.repeat(np.arange(self.ndof), np.diff(J.indptr))
        J.data[mask[rows]] = 0.0
        J = J + sp.csr_matrix((np.ones(self.cons_dofs.size), (self.cons_dofs, self.cons_dofs)),
                              shape=J.shape)
        return J

    # ---------------------------------------------------------------- state helpers
    def initial_state(self):
        t0 = self.tso.get_float("time_begin", 0.0)
        x = np.zeros(self.ndof)
        sf = self.mcfg.sub("scalar_field")
        for sp_ in self.species:
            c = sf.sub(sp_.name)
            if not c.has_sub("initial"):
                continue
            ex = F._scalar(c.sub("initial"), self.ctx)
            if ex is None:
                continue
            verts = self.comp_vertices[sp_.comp]
            pos = self.mesh.coords[verts]
            env = {"time": t0}
            for d in range(3):
                env["position_" + AXES[d]] = pos[:, d] if d < self.dim else 0.0
            val = np.broadcast_to(np.asarray(ex(env), float), (verts.shape[0],))
            x[self.dof(sp_, verts)] = val
        return x

    def reduce(self, x, t, cfg=None):
        """Transform/reduce operators, model/diffusion_reaction/reduce.hh:40-285.

        For every key of the [model.reduce] section (or `cfg`): value = initial.value
        (default 0); then, over every cell in grid order and every point of the order-4 rule
        (F.reduce_rule), value = reduction(evaluation, value) with reduction the user
        function `init, val: ...` (default: +).  The per-thread value is then combined with
        initial.value once more (reduce.hh:237-241, one thread), transformation `arg: ...`
        is applied, and error `arg: ...` / warn `arg: ...` flag the key when non-zero.
        Variables: species values and gradients (0 for species whose compartment does not
        contain the cell), position_*, integration_factor = weight x |det J|, time,
        entity_volume = cell volume, in_volume = 1.
        Returns ({key: value}, [error keys], [warning keys]).
        """
        if cfg is None:
            if not self.mcfg.has_sub("reduce"):
                return {}, [], []
            cfg = self.mcfg.sub("reduce")
        keys = cfg.sub_keys()
        if not keys:
            return {}, [], []
        m = self.mesh
        d = self.dim
        qp, qw = F.reduce_rule(d)
        phi = F.p1_values(qp)                                     # [nq, nl]
        nq = qw.shape[0]
        xq = self.v0[:, None, :] + np.einsum("nij,qj->nqi", self.B, qp)
        env = {"time": t, "integration_factor": np.abs(self.det)[:, None] * qw[None, :],
               "entity_volume": np.repeat(self.vol[:, None], nq, axis=1), "in_volume": 1.0,
               "in_boundary": 0.0, "in_skeleton": 0.0, "no_value": np.finfo(float).max}
        for j in range(3):
            env["position_" + AXES[j]] = xq[:, :, j] if j < d else 0.0
        for sp_ in self.species:
            inside = self.comp_mask[sp_.comp]
            vloc = self.comp_vloc[sp_.comp]
            cells = m.cells
            ok = inside & np.all(vloc[cells] >= 0, axis=1)
            c = np.zeros(cells.shape)
            c[ok] = x[self.comp_offset[sp_.comp] + vloc[cells[ok]] * self.ns[sp_.comp] + sp_.local]
            env[sp_.name] = c @ phi.T                               # [ne, nq]
            g = np.einsum("na,naj->nj", c, self.G)                  # [ne, d]
            for j in range(3):
                env["grad_%s_%s" % (sp_.name, AXES[j])] = (
                    np.repeat(g[:, j:j + 1], nq, axis=1) if j < d else 0.0)
        values, errors, warns = {}, [], []
        for key in keys:
            sub = cfg.sub(key)
            init = sub.get_float("initial.value", 0.0)
            ev = F._scalar(sub.sub("evaluation"), self.ctx) if sub.has_sub("evaluation") else None
            vals = (np.zeros((m.ne, nq)) if ev is None
                    else np.broadcast_to(np.asarray(ev(env), float), (m.ne, nq))).ravel()
            red = sub.get("reduction.expression") if sub.has_sub("reduction") else None
            acc = self._fold(red, vals, init)
            acc = self._fold(red, np.array([acc]), init)             # thread combine
            for part in ("transformation",):
                if sub.has_sub(part):
                    acc = float(self._call1(sub.get(part + ".expression"), acc))
            if sub.has_sub("error") and self._call1(sub.get("error.expression"), acc) != 0.0:
                errors.append(key)
            elif sub.has_sub("warn") and self._call1(sub.get("warn.expression"), acc) != 0.0:
                warns.append(key)
            values[key] = acc
        return values, errors, warns

    def _call1(self, text, arg):
        f = E.parse_function_definition(text)
        if len(f.args) != 1:
            raise ValueError("function must have exactly 1 argument: %r" % text)
        env = self.ctx.env()
        env[f.args[0]] = arg
        return float(E.evaluate(f.body, env, self.ctx.functions))

    def _fold(self, text, vals, init):
        """acc = f(v, acc) over vals in order, starting from init (f = + by default)."""
        if text is None:
            return float(np.cumsum(np.concatenate([[init], vals]))[-1])
        f = E.parse_function_definition(text)
        if len(f.args) != 2:
            raise ValueError("Reduction arguments must be exactly 2")
        a, b = f.args
        body = text[text.find(":") + 1:].replace(" ", "")
        if body in ("%s+%s" % (a, b), "%s+%s" % (b, a)):
            return float(np.cumsum(np.concatenate([[init], vals]))[-1])
        for fn, op in (("max", np.max), ("min", np.min)):
            if body in ("%s(%s,%s)" % (fn, a, b), "%s(%s,%s)" % (fn, b, a)):
                return float(op(np.concatenate([[init], vals])))
        acc = init
        env = self.ctx.env()
        for v in vals:
            env[a] = float(v)
            env[b] = acc
            acc = float(E.evaluate(f.body, env, self.ctx.functions))
        return acc

    def species_values(self, x, name):
        sp_ = next(s for s in self.species if s.name == name)
        return x[self.dof(sp_, self.comp_vertices[sp_.comp])]

    # ---------------------------------------------------------------- volume terms
    def _volume_env(self, els, sps, x, t, perturb=None):
        """Quadrature-point values of every symbol on elements ``els``.

        ``perturb`` = (species name, local dof, delta[n]) adds delta to one local
        coefficient of every element (element-local finite differences).
        """
        n = els.shape[0]
        nq = self.qw.shape[0]
        cells = self.mesh.cells[els]
        env = {"time": t, "integration_factor": 0.0, "in_volume": 1.0, "in_boundary": 0.0,
               "in_skeleton": 0.0, "no_value": np.finfo(float).max}
        env["entity_volume"] = np.repeat(self.vol[els][:, None], nq, axis=1)
        for d in range(3):
            env["position_" + AXES[d]] = self.xq[els, :, d] if d < self.dim else 0.0
        zeros = np.zeros((n, nq))
        for s in self.species:
            env[s.name] = zeros
            for d in range(3):
                env["grad_%s_%s" % (s.name, AXES[d])] = zeros
        grad = {}
        G = self.G[els]
        for s in sps:
            c = x[self.dof(s, cells)]                                  # [n, d+1]
            if perturb is not None and perturb[0] == s.name:
                c = c.copy()
                c[:, perturb[1]] += perturb[2]
            u = c @ self.phi.T                                         # [n, nq]
            g = np.einsum("na,naj->nj", c, G)                          # [n, d]
            env[s.name] = u
            grad[s.name] = np.repeat(g[:, None, :], nq, axis=1)
            for d in range(3):
                env["grad_%s_%s" % (s.name, AXES[d])] = grad[s.name][..., d] if d < self.dim else 0.0
        return env, grad, cells

    def _local_volume_residual(self, x, t, form, els, sps, perturb):
        env, grad, cells = self._volume_env(els, sps, x, t, perturb)
        n = els.shape[0]
        nq = self.qw.shape[0]
        G = self.G[els]
        fac = self.factor[els]
        shape = (n, nq)
        out = {}
        for s in sps:
            eq = self.eq_by_name[s.name]
            scalar = np.zeros(shape)
            flux = np.zeros(shape + (self.dim,))
            if form == "stiffness":
                if eq.reaction is not None:
                    scalar = scalar - F._ev(eq.reaction.value, env, shape)
                if eq.velocity is not None:
                    v = np.stack([F._ev(c, env, shape) if c is not None else np.zeros(shape)
                                  for c in eq.velocity.comps], axis=-1)
                    flux = flux + v * env[s.name][..., None]
                for (w, D, _jac) in eq.cross_diffusion:
                    gw = grad.get(w)
                    if gw is None:
                        continue
                    flux = flux - D.apply(env, gw)
            else:
                if eq.storage is not None:
                    scalar = scalar + env[s.name] * F._ev(eq.storage.value, env, shape)
            out[s.name] = (np.einsum("nq,qa->na", scalar * fac, self.phi)
                           - np.einsum("nqj,naj->na", flux * fac[..., None], G))
        return out, cells

    def _volume_residual(self, x, t, form, els, sps, r):
        loc, cells = self._local_volume_residual(x, t, form, els, sps, None)
        for s in sps:
            np.add.at(r, self.dof(s, cells), loc[s.name])

    def _volume_jacobian(self, x, t, form, els, sps, rows, cols, vals):
        env, grad, cells = self._volume_env(els, sps, x, t)
        n = els.shape[0]
        nq = self.qw.shape[0]
        G = self.G[els]
        fac = self.factor[els]
        shape = (n, nq)
        phi = self.phi
        names = {s.name: s for s in sps}
        # mass-like kernel  K[n,a,b] = sum_q c[n,q] phi_a phi_b fac
        def mass(c):
            return np.einsum("nq,qa,qb->nab", c * fac, phi, phi)

        def add(test, trial, loc):
            ri = self.dof(test, cells)          # [n, d+1]
            ci = self.dof(trial, cells)
            rows.append(np.repeat(ri[:, :, None], ci.shape[1], axis=2).ravel())
            cols.append(np.repeat(ci[:, None, :], ri.shape[1], axis=1).ravel())
            vals.append(loc.ravel())

        for s in sps:
            eq = self.eq_by_name[s.name]
            if form == "stiffness":
                if eq.reaction is not None:
                    for (w, jex) in eq.reaction.jac:
                        if w in names:
                            add(s, names[w], -mass(F._ev(jex, env, shape)))
                if eq.velocity is not None:
                    v = np.stack([F._ev(c, env, shape) if c is not None else np.zeros(shape)
                                  for c in eq.velocity.comps], axis=-1)
                    # -phi_a (v . grad psi_b)  (test/trial as assembled by the reference)
                    loc = -np.einsum("nqj,qa,nbj->nab", v * fac[..., None], phi, G)
                    add(s, s, loc)
                    for (w, jv) in eq.velocity.jac:
                        if w in names:
                            af = np.stack([F._ev(c, env, shape) if c is not None else np.zeros(shape)
                                           for c in jv], axis=-1) * env[s.name][..., None]
                            loc = -np.einsum("nqj,qa,nbj->nab", af * fac[..., None], phi, G)
                            add(s, names[w], loc)
                for (w, D, jac) in eq.cross_diffusion:
                    if w not in names:
                        continue
                    # D(grad phi_a) . grad psi_b
                    loc = np.zeros((n, self.dim + 1, self.dim + 1))
                    for a in range(self.dim + 1):
                        ga = np.repeat(G[:, a, None, :], nq, axis=1)          # [n,nq,d]
                        da = D.apply(env, ga)                                  # [n,nq,d]
                        loc[:, a, :] = np.einsum("nqj,nbj->nb", da * fac[..., None], G)
                    add(s, names[w], loc)
                    for (v, JD) in jac:
                        if v not in names:
                            continue
                        dfl = JD.apply(env, grad[v])                           # [n,nq,d]
                        loc = np.einsum("nqj,qa,nbj->nab", dfl * fac[..., None], phi, G)
                        add(s, names[v], loc)
            else:
                if eq.storage is not None:
                    add(s, s, mass(F._ev(eq.storage.value, env, shape)))
                    for (w, jex) in eq.storage.jac:
                        if w in names:
                            add(s, names[w], mass(F._ev(jex, env, shape) * env[s.name]))

    # ---------------------------------------------------------------- skeleton terms
    def _face_geometry(self):
        """Face quadrature points, weights*|face| and normals, plus local coordinates in both cells."""
        if hasattr(self, "_fgeo"):
            return self._fgeo
        m = self.mesh
        d = self.dim
        fq, fw = F.face_rule(d)
        fvc = m.coords[self.face_vertices]                 # [nf, d, d]
        # face parametrisation x = f0 + sum_k s_k (f_k - f0)
        f0 = fvc[:, 0, :]
        T = np.stack([fvc[:, k, :] - f0 for k in range(1, d)], axis=2)   # [nf, d, d-1]
        xq = f0[:, None, :] + np.einsum("nik,qk->nqi", T, fq)
        if d == 2:
            meas = np.linalg.norm(T[:, :, 0], axis=1)
        else:
            meas = np.linalg.norm(np.cross(T[:, :, 0], T[:, :, 1]), axis=1)
        fac = meas[:, None] * fw[None, :]
        # outward normal of e0
        if d == 2:
            t = T[:, :, 0]
            nrm = np.stack([t[:, 1], -t[:, 0]], axis=1)
        else:
            nrm = np.cross(T[:, :, 0], T[:, :, 1])
        nrm /= np.linalg.norm(nrm, axis=1)[:, None]
        ctr0 = m.coords[m.cells[self.face_e0]].mean(axis=1)
        flip = np.einsum("ni,ni->n", nrm, f0 - ctr0) < 0
        nrm[flip] *= -1.0
        self._fgeo = (xq, fac, nrm, meas * (1.0 if d == 2 else 0.5))
        return self._fgeo

    def _local_coords(self, els, xq):
        """Reference coordinates of physical points xq[nf, nq, d] in cells els."""
        v0 = self.v0[els]
        Binv = np.linalg.inv(self.B[els])
        return np.einsum("nij,nqj->nqi", Binv, xq - v0[:, None, :])

    def _skeleton(self, x, t, residual, rows, cols, vals, perturb=None, local=None):
        """Skeleton / boundary outflow terms (local_operator.hh:777-1203, 1398-1436).

        ``perturb`` = (cell role 0 | 1 (the face's first / second cell), species name, cell-local
        vertex, delta[nf]) adds delta to one local coefficient of that cell on every face
        (face-local finite differences); ``local`` (a dict) receives the residual contributions
        per face instead of summing them into ``residual``: local[(role, species)] = [nf, d+1]
        over the test functions of the cell with that role.
        """
        if self.face_e0.shape[0] == 0:
            return
        m = self.mesh
        xq, fac, nrm, fvol = self._face_geometry()
        nf, nq = fac.shape
        sig = self.elem_sig
        e0 = self.face_e0
        e1 = self.face_e1
        has_nb = e1 >= 0
        e1s = np.where(has_nb, e1, e0)
        xi0 = self._local_coords(e0, xq)
        xi1 = self._local_coords(e1s, xq)
        phi0 = F.p1_values(xi0)                         # [nf, nq, d+1]
        phi1 = F.p1_values(xi1)
        cells0 = m.cells[e0]
        cells1 = m.cells[e1s]
        ncomp = len(self.comp_names)

        def exists(sp_, sigs):
            return ((sigs >> sp_.comp) & 1).astype(bool)

        for side in (0, 1):
            if side == 0:
                ein, eout, phin, phout, cin, cout, nr = e0, e1s, phi0, phi1, cells0, cells1, nrm
            else:
                ein, eout, phin, phout, cin, cout, nr = e1s, e0, phi1, phi0, cells1, cells0, -nrm
            sig_in = sig[ein]
            sig_out = sig[eout]
            active_side = has_nb if side == 1 else np.ones(nf, bool)
            # species values: own side first, else the other side (local_operator.hh:879-896)
            env = {"time": t, "integration_factor": 0.0, "in_volume": 0.0,
                   "no_value": np.finfo(float).max}
            env["in_boundary"] = np.repeat((~has_nb).astype(float)[:, None], nq, axis=1)
            env["in_skeleton"] = np.repeat(has_nb.astype(float)[:, None], nq, axis=1)
            env["entity_volume"] = np.repeat(fvol[:, None], nq, axis=1)
            for d in range(3):
                env["position_" + AXES[d]] = xq[..., d] if d < self.dim else 0.0
                env["normal_" + AXES[d]] = np.repeat(nr[:, None, d], nq, axis=1) if d < self.dim else 0.0
            src_in = {}
            for s in self.species:
                ex_in = exists(s, sig_in)
                ex_out = exists(s, sig_out) & has_nb
                use_in = ex_in
                use_out = (~ex_in) & ex_out
                u = np.zeros((nf, nq))
                g = np.zeros((nf, nq, self.dim))
                if use_in.any():
                    idx = np.nonzero(use_in)[0]
                    c = x[self.dof(s, cin[idx])]
                    if perturb is not None and perturb[1] == s.name and perturb[0] == side:
                        c = c.copy()
                        c[:, perturb[2]] += perturb[3][idx]
                    u[idx] = np.einsum("na,nqa->nq", c, phin[idx])
                    g[idx] = np.einsum("na,naj->nj", c, self.G[ein[idx]])[:, None, :]
                if use_out.any():
                    idx = np.nonzero(use_out)[0]
                    c = x[self.dof(s, cout[idx])]
                    if perturb is not None and perturb[1] == s.name and perturb[0] == 1 - side:
                        c = c.copy()
                        c[:, perturb[2]] += perturb[3][idx]
                    u[idx] = np.einsum("na,nqa->nq", c, phout[idx])
                    g[idx] = np.einsum("na,naj->nj", c, self.G[eout[idx]])[:, None, :]
                env[s.name] = u
                for d in range(3):
                    env["grad_%s_%s" % (s.name, AXES[d])] = g[..., d] if d < self.dim else 0.0
                src_in[s.name] = (ex_in, ex_out)
            for s in self.species:
                eq = self.eq_by_name[s.name]
                if not eq.outflow:
                    continue
                ci = s.comp
                ex_in = exists(s, sig_in) & active_side
                for co, fn in eq.outflow.items():
                    # interior: species absent outside, co != ci present on either side;
                    # boundary: co == ci   (local_operator.hh:836-853)
                    interior_ok = has_nb & ~exists(s, sig_out) & (co != ci) & \
                        ((((sig_out >> co) & 1) | ((sig_in >> co) & 1)).astype(bool))
                    boundary_ok = (~has_nb) & (co == ci)
                    sel = ex_in & (interior_ok | boundary_ok)
                    if not sel.any():
                        continue
                    idx = np.nonzero(sel)[0]
                    sub = {k: (v[idx] if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == nf else v)
                           for k, v in env.items()}
                    shape = (idx.shape[0], nq)
                    fq_ = fac[idx]
                    rows_test = self.dof(s, cin[idx])                          # [k, d+1]
                    if residual is not None or local is not None:
                        T = F._ev(fn.value, sub, shape)
                        loc = np.einsum("kq,kqa->ka", T * fq_, phin[idx])
                        if local is not None:
                            acc = local.setdefault((side, s.name), np.zeros((nf, self.dim + 1)))
                            np.add.at(acc, idx, loc)
                        else:
                            np.add.at(residual, rows_test, loc)
                    if rows is not None:
                        for (w, jex) in fn.jac:
                            sw = next(sp_ for sp_ in self.species if sp_.name == w)
                            J = F._ev(jex, sub, shape)
                            w_out = exists(sw, sig_out[idx]) & has_nb[idx]
                            w_in = exists(sw, sig_in[idx])
                            # do_self_basis when w has no basis outside (local_operator.hh:1099-1101)
                            for use_out_b in (False, True):
                                pick = (w_out if use_out_b else (~w_out & w_in))
                                if not pick.any():
                                    continue
                                k = np.nonzero(pick)[0]
                                ph_tr = (phout if use_out_b else phin)[idx[k]]
                                ctr = (cout if use_out_b else cin)[idx[k]]
                                loc = np.einsum("kq,kqa,kqb->kab", J[k] * fq_[k], phin[idx[k]], ph_tr)
                                ri = rows_test[k]
                                cj = self.dof(sw, ctr)
                                rows.append(np.repeat(ri[:, :, None], cj.shape[1], axis=2).ravel())
                                cols.append(np.repeat(cj[:, None, :], ri.shape[1], axis=1).ravel())
                                vals.append(loc.ravel())

    # ---------------------------------------------------------------- global operators
    def _chunks(self, els):
        for i in range(0, els.shape[0], self.chunk):
            yield els[i:i + self.chunk]

    def residual(self, x, t, form):
        r = np.zeros(self.ndof)
        for els, sps in self.groups:
            for part in self._chunks(els):
                self._volume_residual(x, t, form, part, sps, r)
        if form == "stiffness" and self.has_outflow:
            self._skeleton(x, t, r, None, None, None)
        return r

    def jacobian(self, x, t, form):
        if self.numerical_jacobian:
            return self._numerical_jacobian(x, t, form)
        rows, cols, vals = [], [], []
        J = None

        def flush(J):
            part = self._to_csr(rows, cols, vals)
            rows.clear()
            cols.clear()
            vals.clear()
            return part if J is None else J + part

        for els, sps in self.groups:
            for part in self._chunks(els):
                self._volume_jacobian(x, t, form, part, sps, rows, cols, vals)
                if sum(v.size for v in vals) >= self.flush_entries:
                    J = flush(J)
        if form == "stiffness" and self.has_outflow:
            self._skeleton(x, t, None, rows, cols, vals)
        return flush(J) if (rows or J is None) else J

    def _to_csr(self, rows, cols, vals):
        n = self.ndof
        if not rows:
            return sp.csr_matrix((n, n))
        r = np.concatenate(rows)
        c = np.concatenate(cols)
        v = np.concatenate(vals)
        return sp.csr_matrix((v, (r, c)), shape=(n, n))

    def _numerical_skeleton_jacobian(self, x, t, rows, cols, vals):
        """Face-local forward differences of the outflow terms (local_operator.hh:1205-1344):
        every local coefficient of the face's first cell, then of its second cell, is moved by
        delta and the change of both cells' face residuals divided by it.  The reference sizes
        the delta of a second-cell coefficient from the first cell's container at the same node
        and index (line 1305), which on an interface between compartments names a coefficient
        the first cell does not carry; here delta = eps (1 + |c|) of the coefficient moved."""
        nf = self.face_e0.shape[0]
        if nf == 0:
            return
        m = self.mesh
        e0 = self.face_e0
        has_nb = self.face_e1 >= 0
        e1s = np.where(has_nb, self.face_e1, e0)
        role_cells = (m.cells[e0], m.cells[e1s])
        role_elems = (e0, e1s)
        role_valid = (np.ones(nf, bool), has_nb)
        sig = self.elem_sig
        down = {}
        self._skeleton(x, t, None, None, None, None, local=down)
        for role in (0, 1):
            for sw in self.species:
                ex_w = ((sig[role_elems[role]] >> sw.comp) & 1).astype(bool) & role_valid[role]
                if not ex_w.any():
                    continue
                for b in range(self.dim + 1):
                    vtx = np.where(ex_w, role_cells[role][:, b], self.comp_vertices[sw.comp][0])
                    delta = np.where(ex_w, self.fd_eps * (1.0 + np.abs(x[self.dof(sw, vtx)])), 0.0)
                    up = {}
                    self._skeleton(x, t, None, None, None, None, perturb=(role, sw.name, b, delta), local=up)
                    for (rho, sname), arr in up.items():
                        sp_t = next(sp_ for sp_ in self.species if sp_.name == sname)
                        ex_s = ((sig[role_elems[rho]] >> sp_t.comp) & 1).astype(bool) & role_valid[rho]
                        sel = ex_w & ex_s
                        if not sel.any():
                            continue
                        dn = down.get((rho, sname), np.zeros_like(arr))
                        d = (arr[sel] - dn[sel]) / delta[sel][:, None]               # [k, d+1]
                        rr = self.dof(sp_t, role_cells[rho][sel])
                        cc = np.repeat(self.dof(sw, role_cells[role][sel, b])[:, None], self.dim + 1, axis=1)
                        rows.append(rr.ravel())
                        cols.append(cc.ravel())
                        vals.append(d.ravel())

    def _numerical_jacobian(self, x, t, form):
        """Element-local forward differences, delta = eps (1 + |c|) (local_operator.hh:713-765),
        and face-local ones for the outflow terms of the stiffness form."""
        rows, cols, vals = [], [], []
        cells_all = self.mesh.cells
        nl = self.dim + 1
        for els, sps in self.groups:
            cells = cells_all[els]
            down, _ = self._local_volume_residual(x, t, form, els, sps, None)
            for s_tr in sps:
                for b in range(nl):
                    dofs_b = self.dof(s_tr, cells[:, b])
                    delta = self.fd_eps * (1.0 + np.abs(x[dofs_b]))
                    up, _ = self._local_volume_residual(x, t, form, els, sps, (s_tr.name, b, delta))
                    for s_te in sps:
                        col = (up[s_te.name] - down[s_te.name]) / delta[:, None]     # [n, nl]
                        rows.append(self.dof(s_te, cells).ravel())
                        cols.append(np.repeat(dofs_b[:, None], nl, axis=1).ravel())
                        vals.append(col.ravel())
        if form == "stiffness" and self.has_outflow:
            self._numerical_skeleton_jacobian(x, t, rows, cols, vals)
        return self._to_csr(rows, cols, vals)

    # ---------------------------------------------------------------- time stepping
    def one_step(self, x0, t, dt, stats=None):
        """PDELab RungeKutta + Newton (or linear defect correction) for one step.

        Stage i solves  sum_{j<i} [a_ij M(u_j) + b_ij dt A(u_j)] + a_ii M(u_i) + b_ii dt A(u_i) = 0,
        each operator evaluated at t + d_j dt; the stage's initial guess is u_{i-1}.
        """
        A, B, D = rk_scheme(self.tso.get("type", "Alexander2"))
        s = len(A)
        ts = [t + D[j] * dt for j in range(s + 1)]
        us = [x0]
        x = x0.copy()
        for i in range(1, s + 1):
            a = A[i - 1]
            b = B[i - 1]
            const = np.zeros(self.ndof)
            for j in range(i):
                if a[j] != 0.0:
                    const += a[j] * self.residual(us[j], ts[j], "mass")
                if b[j] != 0.0:
                    const += (b[j] * dt) * self.residual(us[j], ts[j], "stiffness")
            ai, bi, ti = a[i], b[i] * dt, ts[i]

            def res(y, const=const, ai=ai, bi=bi, ti=ti):
                r = const.copy()
                if ai != 0.0:
                    r += ai * self.residual(y, ti, "mass")
                if bi != 0.0:
                    r += bi * self.residual(y, ti, "stiffness")
                return self._constrain_residual(r)

            def jac(y, ai=ai, bi=bi, ti=ti):
                J = sp.csr_matrix((self.ndof, self.ndof))
                if ai != 0.0:
                    J = J + ai * self.jacobian(y, ti, "mass")
                if bi != 0.0:
                    J = J + bi * self.jacobian(y, ti, "stiffness")
                return self._constrain_jacobian(J)

            # constrained entries take their values before the stage solve; their residual
            # rows are zero and their Jacobian rows unit rows, so the solve keeps them
            x = self.apply_constraints(x)
            if self.is_linear:
                x = self._linear_solve_step(res, jac, x, stats)
            else:
                x = self._newton(res, jac, x, stats)
            us.append(x.copy())
        return x

    def _solve(self, J, r):
        if J.nnz == 0:
            raise StepFailed("singular stage Jacobian")
        if self.linear == "iterative":
            return self._solve_iterative(J, r)
        # minimum-degree ordering on A^T + A: the matrix pattern is structurally symmetric
        lu = spla.splu(J.tocsc(), permc_spec="MMD_AT_PLUS_A")
        z = lu.solve(r)
        if not np.all(np.isfinite(z)):
            raise StepFailed("linear solve produced non-finite values")
        return z

    def _solve_iterative(self, J, r):
        """BiCGSTAB + Jacobi (scipy) inside iterative refinement: corrections are added
        until the true residual |r - J z| is below iterative_rtol |r|."""
        J = J.tocsr()
        d = J.diagonal()
        if np.any(d == 0.0):
            raise StepFailed("zero diagonal entry in the stage Jacobian")
        dinv = 1.0 / d
        M = spla.LinearOperator(J.shape, matvec=lambda v: dinv * v, dtype=float)
        bn = float(np.linalg.norm(r))
        z = np.zeros_like(r)
        if bn == 0.0:
            return z
        res = r.copy()
        rn = float(np.linalg.norm(res))
        for _sweep in range(8):
            if rn <= self.iterative_rtol * bn:
                return z
            # the correction equation scaled to a unit right-hand side: scipy's breakdown test
            # on rho = <rhat, r> is absolute (eps^2), and rho scales with |r|^2, so Newton's
            # small late right-hand sides would otherwise break down before any progress
            dz, info = spla.bicgstab(J, res / rn, rtol=max(1e-10, 0.1 * self.iterative_rtol * bn / rn), atol=0.0,
                                     maxiter=20000, M=M)
            dz *= rn
            if not np.all(np.isfinite(dz)):
                raise StepFailed("iterative linear solve produced non-finite values")
            z_new = z + dz
            res_new = r - J @ z_new
            rn_new = float(np.linalg.norm(res_new))
            if rn_new > 0.5 * rn and rn <= self.iterative_floor * bn:
                # no longer reduced: the fp64 evaluation of r - J z has reached its rounding
                # floor (a small right-hand side against an operator of large norm), as a
                # direct solve's backward error would
                return z if rn <= rn_new else z_new
            z, res, rn = z_new, res_new, rn_new
        if rn > self.iterative_floor * bn:
            raise StepFailed("iterative linear solve did not reach %g" % self.iterative_floor)
        return z

    def _linear_solve_step(self, res, jac, x, stats):
        b = res(x)
        J = jac(x)
        z = self._solve(J, b)
        if stats is not None:
            stats["linear_solves"] = stats.get("linear_solves", 0) + 1
        return x - z

    def _newton(self, res, jac, x, stats):
        ns = self.tso.sub("nonlinear_solver")
        rel = ns.get_float("convergence_condition.relative_tolerance", 1e-4)
        it_range = [int(v) for v in ns.get_floats("convergence_condition.iteration_range", [0, 40])]
        abs_tol = ns.get_float("convergence_condition.absolute_tolerance", 0.0)
        norm = ns.get("norm", "l_2")
        thr = ns.get_float("linearization_threshold", 0.0)

        def nrm(v):
            if norm == "l_2":
                return float(np.dot(v, v))
            if norm == "l_inf":
                return float(np.max(np.abs(v))) if v.size else 0.0
            if norm == "l_1":
                return float(np.sum(np.abs(v)))
            raise ValueError("Not known nonlinear norm %r" % norm)

        r = res(x)
        defect = nrm(r)
        first = defect
        prev = defect
        it = 0
        J = None
        while True:
            if not math.isfinite(defect):
                raise StepFailed("Newton defect is not finite")
            if it >= it_range[0] and (defect <= abs_tol or defect < first * rel or defect == 0.0):
                break
            if it >= it_range[1]:
                raise StepFailed("Newton did not converge in %d iterations" % it_range[1])
            if J is None or thr <= 0.0 or not (prev > 0 and defect / prev < thr):
                J = jac(x)
            z = self._solve(J, r)
            x = x - z
            prev = defect
            r = res(x)
            defect = nrm(r)
            it += 1
        if stats is not None:
            stats["newton_iterations"] = stats.get("newton_iterations", 0) + it
            stats.setdefault("newton_per_stage", []).append(it)
        return x

    # ---------------------------------------------------------------- stepper
    def stepper_params(self):
        tso = self.tso
        dec = tso.get_float("time_step_decrease_factor", 0.5)
        inc = tso.get_float("time_step_increase_factor", 1.1)
        t0 = tso.get_float("time_begin", 0.0)
        t1 = tso.get_float("time_end", 1.0)
        mn = tso.get_float("time_step_min") if tso.has_key("time_step_min") else None
        mx = tso.get_float("time_step_max") if tso.has_key("time_step_max") else None
        dt0 = tso.get_float("time_step_initial", mx if mx is not None else 0.1)
        return dec, inc, t0, t1, mn, mx, dt0

    def do_step(self, x, t, dt, stats=None):
        """SimpleAdaptiveStepper::do_step: returns (x_new, t_new, dt_next, dt_used)."""
        dec, inc, _t0, _t1, mn, mx, _dt0 = self.stepper_params()

        def check(d):
            if mn is not None and f_lt(abs(d), abs(mn)):
                return False
            if mx is not None and f_gt(abs(d), abs(mx)):
                return False
            return True

        if not check(dt):
            raise StepFailed("time step outside [min, max]")
        while True:
            try:
                xn = self.one_step(x, t, dt, stats)
                break
            except StepFailed:
                if stats is not None:
                    stats["failed_steps"] = stats.get("failed_steps", 0) + 1
                dt = dt * dec
                if not check(dt):
                    raise
        used = dt
        nd = dt * inc
        if mx is not None:
            nd = min(max(nd, -abs(mx)), abs(mx))
        return xn, t + used, nd, used

    def evolve(self, x, t, dt, t_end, callback=None, stats=None):
        """TimeStepper::evolve with snap_to_end_time = true."""
        while f_le(t + 2.0 * dt, t_end):
            x, t, dt, _ = self.do_step(x, t, dt, stats)
            if callback:
                callback(x, t)
        # snap_to_time
        snap = 0
        while f_lt(t, t_end):
            k = int(math.ceil((t_end - t) / dt))
            if k <= 0:
                raise StepFailed("Timestep doesn't make advances towards snap step")
            dt = (t_end - t) / k
            try:
                x, t, dt, _ = self.do_step(x, t, dt, stats)
                if callback:
                    callback(x, t)
            except StepFailed:
                if snap == 100:
                    raise
                snap += 1
                dt *= 0.5
        return x, t, dt

    def run(self, callback=None, stats=None):
        _dec, _inc, t0, t1, _mn, _mx, dt0 = self.stepper_params()
        x = self.initial_state()
        return self.evolve(x, t0, dt0, t1, callback, stats)
