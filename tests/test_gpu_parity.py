"""GPU parity tests: the CUDA engine (through the C ABI) against the CPU oracle.

Tolerances: assembly (residual and Jacobian) relative 1e-12 of the operator's scale;
time stepping: per-species relative L2 <= 1e-8 after every step, Newton iteration
counts equal to within +-1 per stage.
"""

import numpy as np
import pytest

import cases
from oracle.model import OracleModel

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-8
ASM_TOL = 1e-12


def _init_state(om, init):
    x = om.initial_state()
    if init is not None:
        for sp in om.species:
            verts = om.comp_vertices[sp.comp]
            x[om.dof(sp, verts)] = init(sp.name, om.mesh.coords[verts])
    return x


def _rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _species_errors(om, gm, xo, xg):
    out = {}
    for sp in om.species:
        out[sp.name] = _rel(gm_species(gm, om, xg, sp), xo[om.dof(sp, om.comp_vertices[sp.comp])])
    return out


def gm_species(gm, om, xg, sp):
    return xg[om.dof(sp, om.comp_vertices[sp.comp])]


ALL_CASES = {
    "heat": cases.small_heat,
    "gray_scott": cases.small_gray_scott,
    "two_compartment": cases.small_two_compartment,
    "cross_diffusion_3d": cases.small_3d,
    "features_2d": lambda: (cases.FEATURES_INI, None),
    "features_3d_padded": lambda: (cases.FEATURES_3D_INI, None),
    "poisson_constrained": lambda: (cases.POISSON_INI, None),
    "two_compartment_constrained": lambda: (cases.CONSTRAINED_INI, None),
}


@pytest.mark.parametrize("case", ["poisson_constrained", "two_compartment_constrained", "gray_scott"])
def test_constraints_match_oracle(dcgpu_lib, case):
    """Same constrained DOFs (exactly) and values (to rounding) as the oracle's reading of
    constrain.{boundary,skeleton}.expression."""
    ini, _ = ALL_CASES[case]()
    om = OracleModel(ini)
    gm = dcgpu_lib.Model(ini)
    dofs, vals = gm.constraints()
    assert np.array_equal(dofs, om.cons_dofs)
    assert np.allclose(vals, om.cons_vals, rtol=1e-14, atol=1e-15)
    gm.close()


def test_poisson_constrained_is_nodally_exact(dcgpu_lib):
    ini, _ = ALL_CASES["poisson_constrained"]()
    gm = dcgpu_lib.Model(ini)
    gm.evolve(0.1, 0.1)
    x = gm.state()
    c = gm.vertex_coords()
    assert np.abs(x - (c[:, 0] ** 2 + c[:, 1] ** 2)).max() < 1e-9
    gm.close()


@pytest.mark.parametrize("case", sorted(ALL_CASES))
def test_layout_matches_oracle(dcgpu_lib, case):
    ini, _ = ALL_CASES[case]()
    om = OracleModel(ini)
    gm = dcgpu_lib.Model(ini)
    assert gm.ndof == om.ndof
    assert gm.species == [s.name for s in om.species]
    for sp in om.species:
        assert np.array_equal(gm.species_vertices(sp.name), om.comp_vertices[sp.comp])
    np.testing.assert_allclose(gm.state(), om.initial_state(), rtol=1e-14, atol=1e-14)
    gm.close()


# model.assembly.jit: "false" runs the bytecode-interpreter volume kernels, "true" the
# kernels compiled at set-up for each model's programs (NVRTC)
JIT = ["false", "true"]


@pytest.mark.parametrize("jit", JIT)
@pytest.mark.parametrize("case", sorted(ALL_CASES))
@pytest.mark.parametrize("form", ["mass", "stiffness"])
def test_assembly_matches_oracle(dcgpu_lib, case, form, jit):
    ini, init = ALL_CASES[case]()
    om = OracleModel(ini)
    rng = np.random.default_rng(11)
    x = _init_state(om, init) + 0.05 * rng.uniform(-1, 1, om.ndof)
    t = 0.0375
    gm = dcgpu_lib.Model(ini, {"model.assembly.jit": jit})
    assert gm.jit_status() == ("compiled" if jit == "true" else "off")
    cm, ca = (1.0, 0.0) if form == "mass" else (0.0, 1.0)
    r, J = gm.assemble(x, t, cm, ca)
    r_ref = om.residual(x, t, form)
    scale = max(np.abs(r_ref).max(), 1e-300)
    assert np.abs(r - r_ref).max() <= ASM_TOL * scale + 1e-300, case
    Jg = gm.jacobian_csr(J)
    Jo = om.jacobian(x, t, form)
    D = (Jg - Jo).tocoo()
    jscale = max(abs(Jo).max(), 1e-300)
    assert (np.abs(D.data).max() if D.nnz else 0.0) <= ASM_TOL * jscale, case
    # combined stage operator: cm M + ca A in one pass
    r2, J2 = gm.assemble(x, t, 0.7, -1.3)
    r2_ref = 0.7 * om.residual(x, t, "mass") - 1.3 * om.residual(x, t, "stiffness")
    assert np.abs(r2 - r2_ref).max() <= 1e-11 * max(np.abs(r2_ref).max(), 1e-300)
    gm.close()


def assert_newton_per_stage(oracle_counts, engine_counts, where):
    """The same stage solves, and per stage Newton iteration counts equal within +-1."""
    assert len(oracle_counts) == len(engine_counts), (where, oracle_counts, engine_counts)
    for a, b in zip(oracle_counts, engine_counts):
        assert abs(a - b) <= 1, (where, oracle_counts, engine_counts)


def _run_both(dcgpu_lib, ini, init, mixed=False, overrides=None):
    om = OracleModel(ini, overrides)
    gm = dcgpu_lib.Model(ini, overrides)
    if mixed:
        gm.set_mixed_precision(True)
    x = _init_state(om, init)
    _dec, _inc, t0, t1, _mn, _mx, dt0 = om.stepper_params()
    gm.set_state(x, t0)
    dt_o = dt0
    dt_g = dt0
    t = t0
    records = []
    while t < t1 - 1e-12:
        st = {}
        x, t_new, dt_o, used_o = om.do_step(x, t, dt_o, st)
        info = gm.step(dt_g)
        dt_g = info["dt_next"]
        assert info["time"] == pytest.approx(t_new, rel=0, abs=1e-14)
        assert info["dt_used"] == pytest.approx(used_o, rel=0, abs=1e-15)
        xg = gm.state()
        errs = {sp.name: _rel(xg[om.dof(sp, om.comp_vertices[sp.comp])],
                              x[om.dof(sp, om.comp_vertices[sp.comp])]) for sp in om.species}
        records.append((t_new, errs, list(st.get("newton_per_stage", [])), info["newton_per_stage"]))
        t = t_new
    gm.close()
    return records


@pytest.mark.parametrize("jit", JIT)
@pytest.mark.parametrize("case", sorted(ALL_CASES))
def test_time_stepping_matches_oracle(dcgpu_lib, case, jit):
    ini, init = ALL_CASES[case]()
    records = _run_both(dcgpu_lib, ini, init, overrides={"model.assembly.jit": jit})
    assert records
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, t, name, e)
        assert_newton_per_stage(n_o, n_g, (case, t))


@pytest.mark.parametrize("case", ["gray_scott", "two_compartment", "cross_diffusion_3d", "features_3d_padded"])
@pytest.mark.parametrize("fmt,jit", [("auto", "false"), ("bsr", "false"), ("sell", "false"), ("auto", "true")])
def test_mixed_precision_matches_oracle(dcgpu_lib, case, fmt, jit):
    """fp32 BiCGSTAB inside fp64 iterative refinement, with the fp32 operator in BSR or
    SELL-32 layout or the tuner's choice: same tolerance against the fp64 oracle (and with
    the run-time compiled volume kernels, whose fp32 Jacobian-only pass this exercises)."""
    ini, init = ALL_CASES[case]()
    ov = {"model.time_step_operator.linear_solver.spmv": fmt, "model.assembly.jit": jit}
    records = _run_both(dcgpu_lib, ini, init, mixed=True, overrides=ov)
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, t, name, e)
        assert_newton_per_stage(n_o, n_g, (case, t))


def test_spmv_tuner_reports_choice(dcgpu_lib):
    """linear_solver.spmv = auto: both layouts are timed on the first fp32 operator and the
    faster one is kept; forced layouts are reported as given and not timed."""
    ini, init = cases.small_gray_scott()
    gm = dcgpu_lib.Model(ini)
    assert gm.spmv_format()["format"] == "auto"
    gm.set_mixed_precision(True)
    # the seeded state: the configuration's own initial state (u = 1, v = 0) is the exact
    # stage solution, whose rounding-level defect no relative Newton criterion can reduce
    gm.set_state(gm.seeded_state(init), 0.0)
    gm.step(1.0)
    f = gm.spmv_format()
    assert f["format"] in ("bsr", "sell")
    assert f["bsr_us"] > 0 and f["sell_us"] > 0
    assert (f["format"] == "sell") == (f["sell_us"] < f["bsr_us"])
    gm.close()
    gm = dcgpu_lib.Model(ini, {"model.time_step_operator.linear_solver.spmv": "sell"})
    gm.set_mixed_precision(True)
    gm.set_state(gm.seeded_state(init), 0.0)
    gm.step(1.0)
    f = gm.spmv_format()
    assert f["format"] == "sell" and f["bsr_us"] == 0 and f["sell_us"] == 0
    gm.close()
    with pytest.raises(dcgpu_lib.DcError):
        dcgpu_lib.Model(ini, {"model.time_step_operator.linear_solver.spmv": "csr"})


@pytest.mark.parametrize("case", ["gray_scott", "two_compartment", "cross_diffusion_3d", "features_3d_padded"])
@pytest.mark.parametrize("mixed", [False, True])
def test_multigrid_preconditioner_matches_oracle(dcgpu_lib, case, mixed):
    """Aggregation multigrid V-cycle as the BiCGSTAB preconditioner (fp64, and fp32 inside
    fp64 refinement): same 1e-8 tolerance against the oracle's direct solves."""
    ini, init = ALL_CASES[case]()
    ov = {"model.time_step_operator.linear_solver.preconditioner.type": "AMG",
          "model.time_step_operator.linear_solver.preconditioner.coarsen_target": "16"}
    records = _run_both(dcgpu_lib, ini, init, mixed=mixed, overrides=ov)
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, t, name, e)
        assert_newton_per_stage(n_o, n_g, (case, t))


@pytest.mark.parametrize("case", ["gray_scott", "cross_diffusion_3d", "two_compartment"])
def test_numerical_jacobian_matches_oracle(dcgpu_lib, case):
    """model.jacobian.type = numerical: element-local forward differences with
    delta = eps (1 + |c|) (local_operator.hh:713-765) on both sides, and face-local ones for
    the interface outflow terms of the two-compartment case (local_operator.hh:1205-1344)."""
    ini, init = ALL_CASES[case]()
    ov = {"model.jacobian.type": "numerical",
          "model.time_step_operator.nonlinear_solver.convergence_condition.relative_tolerance": "1e-20"}
    records = _run_both(dcgpu_lib, ini, init, overrides=ov)
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, t, name, e)
        assert_newton_per_stage(n_o, n_g, (case, t))


def test_linear_model_defect_correction(dcgpu_lib):
    """is_linear = true: one defect-correction solve per stage (make_step_operator.hh:210-245)."""
    import test_oracle as T
    ini = T.GAUSS_INI.replace("refinement_level = 5", "refinement_level = 3")
    records = _run_both(dcgpu_lib, ini, None)
    assert records
    for t, errs, *_ in records:
        assert errs["u"] <= STEP_TOL


def test_iterative_solver_configuration(dcgpu_lib):
    """linear_solver.type = BiCGSTAB with the adaptive Newton linear tolerance still converges
    to the oracle's solution within the Newton tolerance."""
    ini, init = cases.small_gray_scott()
    ov = {"model.time_step_operator.linear_solver.type": "BiCGSTAB",
          "model.time_step_operator.nonlinear_solver.convergence_condition.relative_tolerance": "1e-24"}
    records = _run_both(dcgpu_lib, ini, init, overrides=ov)
    for t, errs, n_o, n_g in records:
        for e in errs.values():
            assert e <= STEP_TOL


def test_deterministic_bitwise(dcgpu_lib):
    ini, init = cases.small_two_compartment(steps=2)
    om = OracleModel(ini)
    x0 = _init_state(om, init)
    outs = []
    for _ in range(2):
        gm = dcgpu_lib.Model(ini)
        gm.set_state(x0, 0.0)
        dt = 0.05
        for _s in range(2):
            dt = gm.step(dt)["dt_next"]
        outs.append(gm.state())
        gm.close()
    assert np.array_equal(outs[0], outs[1])


def test_evolve_matches_oracle_times(dcgpu_lib):
    ini, _ = cases.small_heat(n=12, steps=5)
    ini = ini.replace("time_end = 0.05", "time_end = 0.047")
    om = OracleModel(ini)
    times_o = []
    om.run(callback=lambda x, t: times_o.append(t))
    gm = dcgpu_lib.Model(ini)
    times_g = []
    gm.evolve(0.047, 0.01, callback=lambda t: times_g.append(t))
    assert len(times_g) == len(times_o)
    np.testing.assert_allclose(times_g, times_o, rtol=0, atol=1e-15)
    gm.close()


def test_step_failure_halves_dt_and_reports_dt_min(dcgpu_lib):
    """A stage whose expressions go non-finite fails; the stepper halves dt down to
    time_step_min and reports DC_ERR_DT_MIN, leaving the state untouched (stepper.hh:337-382)."""
    ini = """
[grid]
cells = 4 4
[compartments.domain]
expression = 1
[model.scalar_field.u]
compartment = domain
initial.expression = 1
storage.expression = 1
reaction.expression = log(u - 2)
reaction.jacobian.u.expression = 1/(u - 2)
cross_diffusion.u.expression = 0.1
[model.time_step_operator]
type = ImplicitEuler
time_end = 1
time_step_initial = 0.1
time_step_min = 0.02
time_step_max = 0.1
"""
    gm = dcgpu_lib.Model(ini)
    before = gm.state()
    with pytest.raises(dcgpu_lib.DcError) as ei:
        gm.step(0.1)
    assert ei.value.status == 2
    assert np.array_equal(gm.state(), before)
    assert gm.time() == 0.0
    assert gm.stats()["failed_steps"] >= 3
    gm.close()


def test_config_errors_are_reported(dcgpu_lib):
    with pytest.raises(dcgpu_lib.DcError) as ei:
        dcgpu_lib.Model("[grid]\ncells = 2 2\n[compartments.d]\nexpression = 1\n"
                        "[model.scalar_field.u]\ncompartment = d\nreaction.expression = u +\n")
    assert ei.value.status == 4
    with pytest.raises(dcgpu_lib.DcError) as ei:
        dcgpu_lib.Model("[grid]\ncells = 2 2\n[compartments.d]\nexpression = 1\n")
    assert ei.value.status == 4


def test_single_cell_and_empty_compartment(dcgpu_lib):
    """Edge cases: a one-cell grid, and a compartment that contains no cell."""
    ini = """
[grid]
cells = 1 1
[compartments]
a.expression = 1
b.expression = 0
[model.scalar_field.u]
compartment = a
initial.expression = position_x + 2*position_y
storage.expression = 1
cross_diffusion.u.expression = 1
reaction.expression = -u
reaction.jacobian.u.expression = -1
[model.scalar_field.v]
compartment = b
initial.expression = 1
[model.time_step_operator]
type = ImplicitEuler
time_end = 0.2
time_step_max = 0.1
"""
    records = _run_both(dcgpu_lib, ini, None)
    for t, errs, *_ in records:
        assert errs["u"] <= STEP_TOL


def test_reduce_matches_oracle(dcgpu_lib):
    """Transform/reduce operators on the initial state and after the run: sums to 1e-12,
    max exactly, the general fold and the error/warn flags as the oracle."""
    ini = cases.DECAY_INI
    om = OracleModel(ini)
    gm = dcgpu_lib.Model(ini)
    for when in ("initial", "final"):
        if when == "final":
            # both reduce the same state (the two runs agree to the stepping tolerance only)
            x, t, *_ = om.run()
            gm.evolve(0.5, 0.1)
            assert np.abs(gm.state() - x).max() <= STEP_TOL * np.abs(x).max()
            gm.set_state(x, t)
        else:
            x, t = om.initial_state(), 0.0
        vo, eo, wo = om.reduce(x, t)
        vg, eg, wg = gm.reduce()
        assert set(vg) == set(vo)
        for k in vo:
            assert vg[k] == pytest.approx(vo[k], rel=1e-10, abs=1e-14), (when, k)
        assert sorted(eg) == sorted(eo) and sorted(wg) == sorted(wo)
    # an explicit reduce section on a two-compartment 3D model (gradients, per-compartment species)
    sec = """
[model.reduce]
pmass.evaluation.expression = p*integration_factor
qgrad.evaluation.expression = (grad_q_x + 2*grad_q_z)*integration_factor
rmin.evaluation.expression = r + position_y
rmin.reduction.expression = a, b: min(b, a)
rmin.initial.value = 1e100
vol.evaluation.expression = entity_volume*integration_factor
"""
    om = OracleModel(cases.FEATURES_3D_INI)
    gm = dcgpu_lib.Model(cases.FEATURES_3D_INI)
    from oracle.ini import ParameterTree
    vo, _, _ = om.reduce(om.initial_state(), 0.0, ParameterTree.from_text(sec).sub("model.reduce"))
    vg, _, _ = gm.reduce(sec)
    for k in vo:
        assert vg[k] == pytest.approx(vo[k], rel=1e-10, abs=1e-14), k
    gm.close()


def test_vtk_output_round_trip(dcgpu_lib, tmp_path):
    """Per compartment a .vtu piece with the compartment's cells and one vertex field per
    species, and a .pvd time series that lists every written step."""
    import xml.etree.ElementTree as ET
    ini, init = ALL_CASES["two_compartment_constrained"]()
    gm = dcgpu_lib.Model(ini)
    out = tmp_path / "run"
    gm.write_vtk(out, append=False)
    gm.step(0.05)
    gm.write_vtk(out)
    x = gm.state()
    coords = gm.vertex_coords()
    off = 0
    for comp, names in (("left", ["a", "b"]), ("right", ["c", "d"])):
        verts = gm.species_vertices(names[0])
        pvd = ET.parse(out / ("run-%s.pvd" % comp)).getroot()
        files = [d.get("file") for d in pvd.iter("DataSet")]
        times = [float(d.get("timestep")) for d in pvd.iter("DataSet")]
        assert files == ["run-%s-00000.vtu" % comp, "run-%s-00001.vtu" % comp]
        assert times == [0.0, pytest.approx(0.05)]
        piece = ET.parse(out / files[1]).getroot().find("UnstructuredGrid/Piece")
        assert int(piece.get("NumberOfPoints")) == len(verts)
        arrays = {a.get("Name"): np.array(a.text.split(), float) for a in piece.find("PointData")}
        for k, nm in enumerate(names):
            np.testing.assert_array_equal(arrays[nm], x[off + k: off + len(names) * len(verts): len(names)])
        pts = np.array(piece.find("Points/DataArray").text.split(), float).reshape(-1, 3)
        np.testing.assert_array_equal(pts[:, :2], coords[verts])
        off += len(names) * len(verts)
    gm.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_gmsh_grid_matches_oracle(dcgpu_lib, tmp_path, dim):
    """An unstructured (perturbed) Gmsh grid with compartments chosen by physical entity:
    same layout and the same time steps as the oracle."""
    path = tmp_path / "grid.msh"
    cases.write_gmsh(str(path), dim=dim, n=6 if dim == 2 else 3)
    ini = cases.gmsh_ini(str(path), dim)
    om = OracleModel(ini)
    gm = dcgpu_lib.Model(ini)
    np.testing.assert_array_equal(gm.vertex_coords(), om.mesh.coords)
    for sp in om.species:
        assert np.array_equal(gm.species_vertices(sp.name), om.comp_vertices[sp.comp])
    gm.close()
    records = _run_both(dcgpu_lib, ini, None)
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (dim, t, name, e)
        assert_newton_per_stage(n_o, n_g, (t,))


MF = {"model.time_step_operator.linear_solver.matrix_free": "true",
      "model.time_step_operator.linear_solver.type": "BiCGSTAB",
      "model.time_step_operator.linear_solver.preconditioner.type": "Richardson",
      "model.time_step_operator.linear_solver.convergence_condition.relative_tolerance": "1e-12",
      "model.time_step_operator.nonlinear_solver.convergence_condition.relative_tolerance": "1e-24"}


@pytest.mark.parametrize("case", ["features_2d", "two_compartment", "features_3d_padded", "gray_scott",
                                  "cross_diffusion_3d", "two_compartment_constrained"])
def test_jacobian_apply_matches_assembled_product(dcgpu_lib, case):
    """dc_jacobian_apply (per-element and per-face evaluation of the state-dependent terms,
    the constant terms from their matrices) equals the assembled Jacobian times v, on the
    rows that are not constrained (the assembled values carry no unit rows)."""
    ini, init = ALL_CASES[case]()
    gm = dcgpu_lib.Model(ini)
    x = gm.seeded_state(init) if init is not None else gm.state()
    rng = np.random.default_rng(11)
    x = x * (1.0 + 0.1 * rng.standard_normal(x.size))
    v = rng.standard_normal(x.size)
    for cm, ca in ((1.0, 0.0), (0.0, 1.0), (1.0, 0.37)):
        _r, J = gm.assemble(x, 0.25, cm, ca, residual=False)
        want = gm.jacobian_csr(J) @ v
        got = gm.jacobian_apply(x, 0.25, cm, ca, v)
        free = np.ones(x.size, bool)
        cons = gm.constraints()
        if cons is not None and len(cons[0]):
            free[np.asarray(cons[0])] = False
            assert np.array_equal(got[~free], v[~free])
        err = np.linalg.norm(got[free] - want[free]) / max(np.linalg.norm(want[free]), 1e-300)
        assert err <= 1e-13, (case, cm, ca, err)
    gm.close()


@pytest.mark.parametrize("case", ["features_2d", "two_compartment", "features_3d_padded", "poisson_constrained"])
def test_matrix_free_matches_oracle(dcgpu_lib, case):
    """linear_solver.matrix_free = true (make_step_operator.hh:289-293): no matrix; BiCGSTAB +
    Richardson with every product evaluated per element / face; the oracle's solution within
    the Newton tolerance."""
    ini, init = ALL_CASES[case]()
    records = _run_both(dcgpu_lib, ini, init, overrides=MF)
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, t, name, e)


@pytest.mark.parametrize("solver", ["CG", "RestartedGMRes"])
def test_matrix_free_other_krylov(dcgpu_lib, solver):
    ini, init = ALL_CASES["heat" if solver == "CG" else "features_2d"]()
    ov = dict(MF)
    ov["model.time_step_operator.linear_solver.type"] = solver
    records = _run_both(dcgpu_lib, ini, init, overrides=ov)
    for t, errs, n_o, n_g in records:
        for e in errs.values():
            assert e <= STEP_TOL, (solver, t, e)


def test_matrix_free_configuration(dcgpu_lib):
    """Matrix-free takes what the reference's matrix-free registries hold: iterative solvers
    and Richardson / InverseOperator; a direct solver, a matrix-based preconditioner or a
    non-boolean value is a configuration error."""
    ini, _init = ALL_CASES["features_2d"]()
    L = "model.time_step_operator.linear_solver."
    gm = dcgpu_lib.Model(ini, {L + "matrix_free": "true", L + "type": "BiCGSTAB"})
    assert gm.precond_info()["type"] == "Richardson"
    gm.close()
    for bad in ({L + "matrix_free": "maybe"},
                {L + "matrix_free": "true"},  # UMFPack: a direct solver needs the matrix
                {L + "matrix_free": "true", L + "type": "BiCGSTAB", L + "preconditioner.type": "SSOR"},
                {L + "matrix_free": "true", L + "type": "BiCGSTAB", L + "preconditioner.type": "AMG"}):
        with pytest.raises(dcgpu_lib.DcError):
            dcgpu_lib.Model(ini, bad)


@pytest.mark.parametrize("precond", ["Jacobi", "AMG"])
@pytest.mark.parametrize("mixed", [False, True])
def test_cg_matches_oracle(dcgpu_lib, precond, mixed):
    """linear_solver.type = CG (dune-istl CGSolver) on a symmetric model, block Jacobi or
    multigrid preconditioned, fp64 or fp32-in-fp64: the oracle's solution within the Newton
    tolerance."""
    ini, init = ALL_CASES["heat"]()
    ov = {"model.time_step_operator.linear_solver.type": "CG",
          "model.time_step_operator.linear_solver.preconditioner.type": precond,
          "model.time_step_operator.linear_solver.preconditioner.coarsen_target": "16",
          "model.time_step_operator.nonlinear_solver.convergence_condition.relative_tolerance": "1e-24"}
    records = _run_both(dcgpu_lib, ini, init, mixed=mixed, overrides=ov)
    for t, errs, n_o, n_g in records:
        for e in errs.values():
            assert e <= STEP_TOL, (precond, mixed, t, e)


def test_fp32_and_fp64_jacobian_in_mixed_precision(dcgpu_lib):
    """Mixed precision with the state-dependent Jacobian terms in fp32 (default) or fp64:
    both meet the oracle tolerance and reach the same state to well within it."""
    ini, init = ALL_CASES["features_2d"]()
    finals = []
    for jp in ("single", "double"):
        ov = {"model.time_step_operator.linear_solver.jacobian_precision": jp}
        records = _run_both(dcgpu_lib, ini, init, mixed=True, overrides=ov)
        for t, errs, n_o, n_g in records:
            for e in errs.values():
                assert e <= STEP_TOL, (jp, t, e)
        finals.append(records[-1][1])
    with pytest.raises(dcgpu_lib.DcError):
        dcgpu_lib.Model(ini, {"model.time_step_operator.linear_solver.jacobian_precision": "half"})
    with pytest.raises(dcgpu_lib.DcError):
        dcgpu_lib.Model(ini, {"model.time_step_operator.linear_solver.type": "QMR"})


@pytest.mark.parametrize("inner", ["1e-5", "1e-6"])
def test_mixed_inner_reduction(dcgpu_lib, inner):
    """linear_solver.inner_reduction: a deeper fp32 correction solve per refinement still
    meets the oracle tolerance on every step; values outside [1e-7, 1) are rejected."""
    ini, init = ALL_CASES["features_2d"]()
    ov = {"model.time_step_operator.linear_solver.inner_reduction": inner}
    records = _run_both(dcgpu_lib, ini, init, mixed=True, overrides=ov)
    for t, errs, n_o, n_g in records:
        for e in errs.values():
            assert e <= STEP_TOL, (inner, t, e)
    for bad in ("0", "1", "1e-9"):
        with pytest.raises(dcgpu_lib.DcError):
            dcgpu_lib.Model(ini, {"model.time_step_operator.linear_solver.inner_reduction": bad})


@pytest.mark.parametrize("restart,precond,mixed", [(40, "Jacobi", False), (5, "Jacobi", False),
                                                   (10, "AMG", False), (10, "Jacobi", True)])
def test_gmres_matches_oracle(dcgpu_lib, restart, precond, mixed):
    """linear_solver.type = RestartedGMRes (right-preconditioned, restart m) on a
    non-symmetric model (velocity and tensor diffusion): the oracle's solution within the
    Newton tolerance, also with short restarts, multigrid, and fp32 inside fp64 refinement."""
    ini, init = ALL_CASES["features_2d"]()
    ov = {"model.time_step_operator.linear_solver.type": "RestartedGMRes",
          "model.time_step_operator.linear_solver.restart": str(restart),
          "model.time_step_operator.linear_solver.preconditioner.type": precond,
          "model.time_step_operator.linear_solver.preconditioner.coarsen_target": "16",
          "model.time_step_operator.linear_solver.convergence_condition.relative_tolerance": "1e-12",
          "model.time_step_operator.nonlinear_solver.convergence_condition.relative_tolerance": "1e-24"}
    records = _run_both(dcgpu_lib, ini, init, mixed=mixed, overrides=ov)
    for t, errs, n_o, n_g in records:
        for e in errs.values():
            assert e <= STEP_TOL, (restart, precond, mixed, t, e)


@pytest.mark.parametrize("case,n", [("gray_scott", 24), ("gray_scott", 72), ("two_compartment", 40),
                                    ("cross_diffusion_3d", 9)])
@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("single", ["true", "false"])
def test_single_launch_bicgstab_matches_oracle(dcgpu_lib, case, n, mixed, single):
    """BiCGSTAB + block Jacobi as one cooperative launch per solve (single_launch = true,
    the default) and as graph-replayed per-phase launches: both within the step tolerance of
    the oracle.  The larger sizes run the single-launch kernel on many blocks (one block row
    per thread), so its grid barriers and the block-order partial sums are exercised."""
    builders = {"gray_scott": cases.small_gray_scott, "two_compartment": cases.small_two_compartment,
                "cross_diffusion_3d": cases.small_3d}
    ini, init = builders[case](n=n, steps=2)
    ov = {"model.time_step_operator.linear_solver.single_launch": single}
    records = _run_both(dcgpu_lib, ini, init, mixed=mixed, overrides=ov)
    assert records
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, n, t, name, e)
        assert_newton_per_stage(n_o, n_g, (t,))


@pytest.mark.parametrize("mixed", [False, True])
def test_single_launch_path_is_taken(dcgpu_lib, mixed):
    """With single_launch on, the Krylov iterations run inside the cooperative kernel (the
    per-phase SpMV timer sees no launch); with it off, no single-launch solve runs."""
    ini, init = cases.small_gray_scott(n=48, steps=1)
    om = OracleModel(ini)
    x0 = _init_state(om, init)
    seen = {}
    for single in ("true", "false"):
        gm = dcgpu_lib.Model(ini, {"model.time_step_operator.linear_solver.single_launch": single})
        if mixed:
            gm.set_mixed_precision(True)
        gm.set_state(x0, 0.0)
        gm.profile(True)
        info = gm.step(1.0)
        kt = gm.kernel_times()
        gm.close()
        seen[single] = (kt, info)
    kt, info = seen["true"]
    assert kt["krylov_iteration"][1] == info["linear_iterations"] > 0
    assert kt["spmv"][1] == 0
    kt, info = seen["false"]
    assert kt["krylov_iteration"][1] == 0 and kt["spmv"][1] > 0


def test_single_launch_matches_graph_path_at_full_size(dcgpu_lib):
    """Gray-Scott 512^2 (526,338 DOF, more block rows than the cooperative grid has threads):
    one mixed-precision Alexander2 step through the single-launch solve and through the
    per-phase launches agree to far below the step tolerance, with the same Newton counts."""
    import workloads as W
    ini, init = W.gray_scott(n=512, steps=1, dt=1.0)
    out = {}
    for single in ("true", "false"):
        gm = dcgpu_lib.Model(ini, {"model.time_step_operator.linear_solver.single_launch": single})
        gm.set_mixed_precision(True)
        gm.set_state(gm.seeded_state(init), 0.0)
        info = gm.step(1.0)
        out[single] = (gm.state(), info["newton_iterations"])
        gm.close()
    (xa, na), (xb, nb) = out["true"], out["false"]
    assert na == nb
    assert _rel(xa, xb) <= 1e-10


@pytest.mark.parametrize("case", ["gray_scott", "two_compartment", "cross_diffusion_3d"])
@pytest.mark.parametrize("mixed", [False, True])
def test_unsplit_stage_residual_matches_oracle(dcgpu_lib, case, mixed):
    """model.assembly.split_residual = false: every stage residual is one combined pass over
    the static and state-dependent terms (the default keeps the state-dependent part of the
    last evaluated state and reuses it at stage boundaries); both meet the oracle tolerance."""
    ini, init = ALL_CASES[case]()
    records = _run_both(dcgpu_lib, ini, init, mixed=mixed, overrides={"model.assembly.split_residual": "false"})
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, t, name, e)
        assert_newton_per_stage(n_o, n_g, (case, t))


def test_split_residual_saves_assembly_passes(dcgpu_lib):
    """With the split stage residual an Alexander2 step of a model with a static mass form
    runs fewer assembly passes than the combined form, for the same state."""
    ini, init = ALL_CASES["cross_diffusion_3d"]()
    out = {}
    for split in ("true", "false"):
        gm = dcgpu_lib.Model(ini, {"model.assembly.split_residual": split})
        for _ in range(3):
            gm.step(0.01)
        out[split] = (gm.stats()["assemblies"], gm.state())
        gm.close()
    assert out["true"][0] < out["false"][0]
    x1, x0 = out["true"][1], out["false"][1]
    assert np.linalg.norm(x1 - x0) <= 1e-12 * np.linalg.norm(x0)


@pytest.mark.parametrize("scheme", ["ExplicitEuler", "ImplicitEuler", "Heun", "Shu3", "RungeKutta4", "Alexander2",
                                    "FractionalStepTheta", "Alexander3"])
def test_runge_kutta_schemes_match_oracle(dcgpu_lib, scheme):
    """Every one-step scheme of the reference's registry (make_step_operator.hh:408-443) on the
    engine against the oracle: the stage states after each step and the Newton iterations of
    every stage (explicit schemes solve their mass-form stage systems by Newton too)."""
    ini, init = cases.small_gray_scott(n=20, steps=3)
    records = _run_both(dcgpu_lib, ini, init, overrides={"model.time_step_operator.type": scheme})
    assert len(records) == 3
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (scheme, t, name, e)
        assert_newton_per_stage(n_o, n_g, (scheme, t))


@pytest.mark.parametrize("case", ["two_compartment", "features_2d"])
def test_numerical_skeleton_jacobian_matches_oracle(dcgpu_lib, case):
    """The numerical Jacobian of a model with outflow terms: the engine's forward differences of
    the face residuals against the oracle's (same delta rule), and, where the configured
    jacobian expressions are the exact derivatives (the two-compartment case), close to the
    analytic Jacobian (forward-difference truncation, delta ~ 1e-7)."""
    ini, init = ALL_CASES[case]()
    ov = {"model.jacobian.type": "numerical"}
    om = OracleModel(ini, ov)
    om_a = OracleModel(ini)
    rng = np.random.default_rng(5)
    x = _init_state(om, init) + 0.05 * rng.uniform(0, 1, om.ndof)
    gm = dcgpu_lib.Model(ini, ov)
    _r, J = gm.assemble(x, 0.0125, 0.0, 1.0)
    Jg = gm.jacobian_csr(J)
    Jo = om.jacobian(x, 0.0125, "stiffness")
    Ja = om_a.jacobian(x, 0.0125, "stiffness")
    jscale = abs(Ja).max()
    # forward differences divide the residuals' rounding (~1e-16 relative) by delta ~ 1e-7
    assert abs(Jg - Jo).max() <= 1e-7 * jscale
    if case == "two_compartment":
        assert abs(Jg - Ja).max() <= 1e-6 * jscale
    gm.close()
