"""CPU tests of the oracle against the reference's own known answers.

The reference's system tests pin this path only through analytic-error thresholds
(test/exp.ini, test/gauss.ini); their configuration text is restated below (it is data,
not code).  Closed-form P1 identities on the Kuhn grid pin the assembly.
"""

import math

import numpy as np
import pytest

from oracle import expr as E
from oracle.ini import ParameterTree
from oracle.mesh import Mesh, structured_simplex
from oracle.model import OracleModel, f_le, rk_scheme

EXP_INI = """
[grid]
dimension = 2
refinement_level = 1

[compartments.domain]
type = expression
expression = 1

[parser_context.grow_rate]
type = constant
value = -2.

[model.scalar_field.u]
compartment = domain
initial.expression = 1
storage.expression = 1
reaction.expression = grow_rate*u
reaction.jacobian.u.expression = grow_rate

[model.time_step_operator]
time_step_max = 0.1
time_end = 10
"""

GAUSS_INI = """
[grid]
extensions = 2 2
origin = -1 -1
refinement_level = 5

[compartments.domain]
type = expression
expression = 1

[parser_context.diffusion]
type = constant
value = 0.005

[parser_context.gauss]
type = function
expression = x, y, z, t: exp(-(x^2+y^2+z^2)/(4*t*diffusion)) / (4*3.14159265359*t*diffusion)

[model]
is_linear = true

[model.scalar_field.u]
compartment = domain

[model.scalar_field.u.cross_diffusion.u]
expression = diffusion

[model.scalar_field.u.initial]
expression = gauss(position_x, position_y, position_z, time)

[model.scalar_field.u.storage]
expression = 1

[model.time_step_operator]
time_begin = 1
time_end = 1.2
"""


def _l2_error(m, x, t, exact):
    env, _g, _c = m._volume_env(np.arange(m.mesh.ne), m.species, x, t)
    xq = m.xq
    ex = exact(xq[..., 0], xq[..., 1], t)
    return math.sqrt(float(((env["u"] - ex) ** 2 * m.factor).sum()))


def test_exp_ini_known_answer():
    """test/exp.ini: ||u - exp(-2t)||_L2 <= 5e-3 at every step (test/exp.ini:32-35)."""
    m = OracleModel(EXP_INI)
    errs = []
    m.run(callback=lambda x, t: errs.append(_l2_error(m, x, t, lambda X, Y, T: np.exp(-2.0 * T) + 0 * X)))
    assert len(errs) >= 100
    assert max(errs) <= 5e-3


@pytest.mark.parametrize("dim", [2, 3])
def test_exp_ini_dimensions(dim):
    """exp-{dim}D runs of test/CMakeLists.txt:111-116 (grid.dimension override)."""
    ini = EXP_INI.replace("time_end = 10", "time_end = 1")
    m = OracleModel(ini, {"grid.dimension": dim})
    x, t, _ = m.run()
    assert abs(t - 1.0) < 1e-12
    assert np.all(np.abs(x - math.exp(-2.0)) < 5e-3)


def test_gauss_ini_known_answer():
    """test/gauss.ini: L2 error <= 0.5, max <= 1/(4 pi D), min >= -1e-2 (gauss.ini:38-55)."""
    m = OracleModel(GAUSS_INI)
    D = 0.005

    def gauss(X, Y, T):
        return np.exp(-(X ** 2 + Y ** 2) / (4 * T * D)) / (4 * 3.14159265359 * T * D)

    rec = []
    m.run(callback=lambda x, t: rec.append((_l2_error(m, x, t, gauss), x.max(), x.min())))
    assert rec
    for err, mx, mn in rec:
        assert err <= 0.5
        assert mx <= 1.0 / (4 * 3.14159265359 * D)
        assert mn >= -1e-2


def test_p1_stiffness_is_five_point_stencil():
    """On the Kuhn triangulation the P1 Laplacian is the 5-point stencil (h-independent in 2D)."""
    n = 6
    ini = """
[grid]
cells = {n} {n}
[compartments.domain]
expression = 1
[model.scalar_field.u]
compartment = domain
cross_diffusion.u.expression = 1
""".format(n=n)
    m = OracleModel(ini)
    K = m.jacobian(np.zeros(m.ndof), 0.0, "stiffness").toarray()
    # interior vertex (i, j) = (3, 3)
    v = 3 + 3 * (n + 1)
    row = K[v]
    assert row[v] == pytest.approx(4.0)
    for nb in (v - 1, v + 1, v - (n + 1), v + (n + 1)):
        assert row[nb] == pytest.approx(-1.0)
    assert abs(row.sum()) < 1e-12
    assert np.count_nonzero(np.abs(row) > 1e-14) == 5
    assert np.allclose(K, K.T)


def test_p1_mass_matrix_known_answer():
    """Consistent P1 mass matrix: total mass = area, diagonal at an interior vertex = h^2/2."""
    n = 8
    ini = """
[grid]
cells = {n} {n}
[compartments.domain]
expression = 1
[model.scalar_field.u]
compartment = domain
storage.expression = 1
""".format(n=n)
    m = OracleModel(ini)
    M = m.jacobian(np.zeros(m.ndof), 0.0, "mass").toarray()
    assert M.sum() == pytest.approx(1.0)
    h = 1.0 / n
    v = 4 + 4 * (n + 1)
    # six triangles of area h^2/2 around an interior vertex, each contributing area/6
    assert M[v, v] == pytest.approx(6 * (h * h / 2) / 6.0)
    r = m.residual(np.ones(m.ndof), 0.0, "mass")
    assert r.sum() == pytest.approx(1.0)


def test_kuhn_grid_3d_volume_and_orientation():
    coords, cells = structured_simplex(3, [2, 3, 4], [0, 0, 0], [1, 2, 3])
    mesh = Mesh(coords, cells)
    assert mesh.ne == 2 * 3 * 4 * 6
    assert mesh.volumes().sum() == pytest.approx(6.0)
    # each cube splits into 6 tets sharing the main diagonal
    assert np.all(mesh.volumes() > 0)


def test_refinement_level_doubles_cells():
    cfg = ParameterTree.from_text("[grid]\ncells = 3 2\nrefinement_level = 2\n")
    m = Mesh.from_config(cfg.sub("grid"))
    assert m.ne == 2 * (3 * 4) * (2 * 4)


@pytest.mark.parametrize("text,val", [
    ("2^3^2", 512.0), ("-2^2", -4.0), ("2*-3", -6.0), ("1+2*3", 7.0), ("(1+2)*3", 9.0),
    ("1 < 2", 1.0), ("2 <= 1", 0.0), ("1 == 1", 1.0), ("1 = 1", 1.0), ("1 != 1", 0.0),
    ("1 && 0", 0.0), ("1 || 0", 1.0), ("1 and 1", 1.0), ("0 or 0", 0.0), ("!0", 1.0),
    ("1 ? 2 : 3", 2.0), ("0 ? 2 : 0 ? 4 : 5", 5.0), ("min(3, 1, 2)", 1.0), ("max(3, 1, 2)", 3.0),
    ("sum(1,2,3)", 6.0), ("avg(1,2,3)", 2.0), ("log(_e)", 1.0), ("ln(1)", 0.0), ("log10(100)", 2.0),
    ("log2(8)", 3.0), ("sqrt(16)", 4.0), ("abs(-3)", 3.0), ("sign(-2)", -1.0), ("rint(2.5)", 2.0),
    ("pow(2, 10)", 1024.0), ("atan2(0, -1)", math.pi), ("7 % 3", 1.0), ("1e-2*100", 1.0),
    (".5 + .5", 1.0), ("floor(-1.5)", -2.0), ("ceil(1.2)", 2.0), ("round(2.5)", 3.0),
])
def test_expression_semantics(text, val):
    assert float(E.evaluate(E.parse(text), {})) == pytest.approx(val)


def test_zero_expression_elision():
    """functor_factory_parser.impl.hh:121-124: empty / all-zero expressions are no functor."""
    for t in ("", "0", "0.0", "-0", "000", ".0"):
        assert E.is_zero_literal(t)
    for t in ("1", "0.1", "u", "0*u"):
        assert not E.is_zero_literal(t)


def test_user_function_and_interpolation():
    ctx = E.Context(ParameterTree.from_text("""
[parser_context.f]
type = function
expression = a, b: a*b + c
[parser_context.c]
type = constant
value = 2
[parser_context.tab]
type = interpolation
domain = 0 1 2
range = 0 10 30
""").sub("parser_context"))
    assert E.Expression("f(3, 4)", ctx)({}) == pytest.approx(14.0)
    assert E.Expression("tab(1.5)", ctx)({}) == pytest.approx(20.0)
    assert E.Expression("tab(-1)", ctx)({}) == pytest.approx(0.0)
    assert E.Expression("tab(5)", ctx)({}) == pytest.approx(30.0)


def test_nested_user_function_rejected():
    cfg = ParameterTree.from_text("""
[parser_context.f]
type = function
expression = x: x
[parser_context.g]
type = function
expression = x: f(x)
""")
    with pytest.raises(E.ExprError):
        E.Context(cfg.sub("parser_context"))


def test_alexander2_is_second_order():
    """Alexander2 on u' = -u: global error ~ dt^2 (PDELab Alexander2Parameter)."""
    ini = EXP_INI.replace("value = -2.", "value = -1.").replace("time_end = 10", "time_end = 1")
    errs = []
    for dt in (0.1, 0.05):
        m = OracleModel(ini, {"model.time_step_operator.time_step_max": dt,
                              "grid.refinement_level": 0})
        x, t, _ = m.run()
        errs.append(abs(x[0] - math.exp(-1.0)))
    assert 3.5 < errs[0] / errs[1] < 4.5


def test_rk_tables_are_consistent():
    for name in ("ImplicitEuler", "Alexander2", "Heun", "Shu3", "RungeKutta4", "FractionalStepTheta",
                 "Alexander3", "ExplicitEuler"):
        A, B, D = rk_scheme(name)
        for row in A:
            assert abs(sum(row)) < 1e-14


def test_snap_to_time_step_count():
    """time_snap behaviour: evolve stops 2 dt before the end and snaps in equal steps."""
    m = OracleModel(EXP_INI.replace("time_end = 10", "time_end = 1"),
                    {"model.time_step_operator.time_step_max": "0.3"})
    times = []
    m.run(callback=lambda x, t: times.append(t))
    assert times[-1] == pytest.approx(1.0)
    assert all(f_le(a, b) for a, b in zip(times, times[1:]))


def test_two_compartment_outflow_conserves_mass():
    """Interface transmission T = k (a - b) moves mass between compartments without loss."""
    ini = """
[grid]
cells = 8 8
[compartments]
left.expression = position_x < 0.5
right.expression = position_x >= 0.5
[model.scalar_field.a]
compartment = left
storage.expression = 1
initial.expression = 1
cross_diffusion.a.expression = 0.1
outflow.right.expression = 0.5*(a - b)
outflow.right.jacobian.a.expression = 0.5
outflow.right.jacobian.b.expression = -0.5
[model.scalar_field.b]
compartment = right
storage.expression = 1
initial.expression = 0
cross_diffusion.b.expression = 0.1
outflow.left.expression = 0.5*(b - a)
outflow.left.jacobian.b.expression = 0.5
outflow.left.jacobian.a.expression = -0.5
[model.time_step_operator]
type = ImplicitEuler
time_end = 0.5
time_step_max = 0.1
[model.time_step_operator.nonlinear_solver]
convergence_condition.relative_tolerance = 1e-20
"""
    m = OracleModel(ini)
    x0 = m.initial_state()
    M = m.jacobian(x0, 0.0, "mass")
    mass0 = M @ x0
    x, t, _ = m.run()
    mass1 = M @ x
    assert abs(mass1.sum() - mass0.sum()) < 1e-10
    a = m.species_values(x, "a")
    b = m.species_values(x, "b")
    assert a.max() < 1.0 and b.max() > 0.0


def test_poisson_constraints_nodally_exact():
    """constrain.boundary holds |x|^2 on the boundary of -lap u = -4; P1 on the Kuhn split
    reproduces the quadratic at the vertices (the reference's poisson test checks the L2
    error only, against a loose threshold)."""
    import cases
    om = OracleModel(cases.POISSON_INI)
    assert om.cons_dofs.size == 4 * 12
    x, t, *_ = om.run()
    c = om.mesh.coords
    assert t == pytest.approx(0.1)
    assert np.abs(x - (c[:, 0] ** 2 + c[:, 1] ** 2)).max() < 1e-12


def test_constraint_selection_rules():
    """Boundary faces of a compartment include its interface; skeleton constraints skip
    vertices on any boundary face; the zero literal is no constraint; constrained values
    are held through the time steps."""
    import cases
    om = OracleModel(cases.CONSTRAINED_INI)
    counts = {}
    for sp_ in om.species:
        d = om.dof(sp_, om.comp_vertices[sp_.comp])
        counts[sp_.name] = int(np.isin(d, om.cons_dofs).sum())
    assert counts == {"a": 11, "b": 5, "c": 0, "d": 5}
    sp_a = next(s for s in om.species if s.name == "a")
    va = om.comp_vertices[sp_a.comp]
    da = om.dof(sp_a, va)
    held = np.isin(da, om.cons_dofs)
    assert np.allclose(om.mesh.coords[va[held], 0], 0.0)
    x, t, *_ = om.run()
    assert np.array_equal(x[om.cons_dofs], om.cons_vals)


@pytest.mark.parametrize("dim,degree", [(2, 4), (3, 5)])
def test_reduce_rule_exactness(dim, degree):
    """The reduce operators' rule integrates every monomial of the stated degree exactly."""
    import itertools
    from oracle import fem as F
    pts, w = F.reduce_rule(dim)
    lam = F.p1_values(pts)
    for alpha in itertools.product(range(degree + 1), repeat=dim + 1):
        if sum(alpha) > degree:
            continue
        exact = (math.prod(math.factorial(a) for a in alpha) * math.factorial(dim)
                 / math.factorial(sum(alpha) + dim) / math.factorial(dim))
        got = float(np.dot(w, np.prod(lam ** np.array(alpha), axis=1)))
        assert got == pytest.approx(exact, rel=1e-13, abs=1e-16), alpha


def test_reduce_operators():
    """Integral, max with initial value, L2 error with transformation/error, warn flag and a
    general reduction function folded in grid order."""
    import cases
    om = OracleModel(cases.DECAY_INI)
    x0 = om.initial_state()
    vals, errs, warns = om.reduce(x0, 0.0)
    c = om.mesh.coords
    assert vals["area"] == pytest.approx(1.2, rel=1e-14)
    # integral of the P1 interpolant of 1 + 0.01 x y over [0, 1.2] x [0, 1]
    assert vals["mass"] == pytest.approx(1.2 + 0.01 * (1.2 ** 2 / 2) * 0.5, rel=1e-4)
    # the max runs over quadrature points, inside the cells
    assert 1.011 < vals["umax"] < 1 + 0.01 * 1.2
    assert errs == [] and warns == ["area"]
    x, t, *_ = om.run()
    vals, errs, warns = om.reduce(x, t)
    assert t == pytest.approx(0.5)
    # implicit Euler with dt = 0.1 against exp(-2t): the L2 error check trips
    assert vals["err"] > 5e-3 and errs == ["err"]
    # general fold: acc = acc + 0.5 v over all points, then combined with the initial value
    # (0) once more: 0 + 0.5 acc
    om2 = OracleModel(cases.DECAY_INI)
    v2, _, _ = om2.reduce(x, t)
    assert v2["mixed"] == vals["mixed"]
    assert np.isfinite(vals["mixed"])


@pytest.mark.parametrize("dim", [2, 3])
def test_gmsh_grid_and_physical_compartments(tmp_path, dim):
    """grid.path: MSH 2.2 ASCII nodes and elements in file order, lower-dimensional elements
    skipped, node ids remapped, gmsh_id (first tag) usable in compartment expressions."""
    import cases
    path = tmp_path / "grid.msh"
    coords, cells, phys = cases.write_gmsh(str(path), dim=dim, n=4)
    om = OracleModel(cases.gmsh_ini(str(path), dim))
    assert np.array_equal(om.mesh.coords, coords)
    assert np.array_equal(om.mesh.cells, cells)
    assert np.array_equal(om.comp_mask[0], phys == 1) and np.array_equal(om.comp_mask[1], phys == 2)
    x, t, *_ = om.run()
    assert t == pytest.approx(0.2) and np.all(np.isfinite(x))


@pytest.mark.parametrize("scale", [1.0, 1e-10, 1e-14])
def test_iterative_solve_scale_invariant(scale):
    """The oracle's iterative stand-in for the direct solve reaches a relative residual of
    1e-13 whatever the size of the right-hand side: Newton's late right-hand sides are tiny,
    and an unscaled solve broke down in scipy's absolute test on rho = <rhat, r>."""
    import scipy.sparse as sp
    ini = ("[grid]\ncells = 4 4\n[compartments.d]\nexpression = 1\n"
           "[model.scalar_field.u]\ncompartment = d\ncross_diffusion.u.expression = 0.01\n")
    om = OracleModel(ini, linear="iterative")
    rng = np.random.default_rng(7)
    n = 400
    A = sp.random(n, n, density=0.02, random_state=11, format="csr")
    J = (A + A.T) * 0.1 + sp.diags(2.0 + rng.random(n))
    r = rng.standard_normal(n) * scale
    z = om._solve_iterative(J.tocsr(), r)
    assert np.linalg.norm(r - J @ z) <= 1e-13 * np.linalg.norm(r)
    assert np.allclose(z / scale, om._solve_iterative(J.tocsr(), r / scale), rtol=1e-10, atol=1e-14)
