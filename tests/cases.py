"""Small model configurations shared by the parity tests (seeded, CPU-oracle sized)."""

import numpy as np

import workloads as W


def small_heat(n=24, steps=6):
    return W.heat(n=n, steps=steps, dt=0.01)


def small_gray_scott(n=24, steps=4):
    return W.gray_scott(n=n, steps=steps, dt=1.0)


def small_two_compartment(n=24, steps=4):
    return W.two_compartment(n=n, steps=steps, dt=0.05)


def small_3d(n=5, steps=3):
    return W.cross_diffusion_3d(n=n, steps=steps, dt=0.01)


FEATURES_INI = """
[grid]
dimension = 2
cells = 10 8
extensions = 1.5 1
origin = -0.25 0

[compartments.domain]
expression = 1

[parser_context.rate]
type = constant
value = 0.7

[parser_context.pulse]
type = function
expression = t, x: exp(-t) * (1 + 0.5*sin(3*x))

[parser_context.profile]
type = interpolation
domain = -1 0 1 2
range = 0.5 1 2 1

[model.scalar_field.u]
compartment = domain
initial.expression = 0.5 + 0.25*cos(2*position_x)*sin(3*position_y)
storage.expression = 1 + 0.1*u
storage.jacobian.u.expression = 0.1
reaction.expression = -rate*u*w + pulse(time, position_x)
reaction.jacobian.u.expression = -rate*w
reaction.jacobian.w.expression = -rate*u
velocity.x.expression = 0.3*profile(position_y)
velocity.y.expression = -0.2
cross_diffusion.u.type = tensor
cross_diffusion.u.xx.expression = 0.02*(1 + u^2)
cross_diffusion.u.xy.expression = 0.005
cross_diffusion.u.yx.expression = 0.002
cross_diffusion.u.yy.expression = 0.01
cross_diffusion.u.jacobian.u.type = tensor
cross_diffusion.u.jacobian.u.xx.expression = 0.04*u
cross_diffusion.w.expression = 0.003
outflow.domain.expression = 0.2*u*(position_x > 0.5 ? 1 : 0.5) + 0.1*normal_x
outflow.domain.jacobian.u.expression = 0.2*(position_x > 0.5 ? 1 : 0.5)

[model.scalar_field.w]
compartment = domain
initial.expression = 0.3 + 0.1*position_x*position_y
storage.expression = 1
reaction.expression = rate*u*w - 0.1*w + entity_volume*0
reaction.jacobian.u.expression = rate*w
reaction.jacobian.w.expression = rate*u - 0.1
cross_diffusion.w.expression = 0.01 + 0.002*(time > 0.05)
velocity.x.expression = 0.1*w
velocity.jacobian.w.x.expression = 0.1

[model.time_step_operator]
type = Alexander2
time_begin = 0
time_end = 0.1
time_step_initial = 0.02
time_step_max = 0.02

[model.time_step_operator.nonlinear_solver]
convergence_condition.relative_tolerance = 1e-16
"""

FEATURES_3D_INI = """
[grid]
dimension = 3
cells = 3 4 3

[compartments]
lower.expression = position_z < 0.5
upper.expression = position_z >= 0.5

[model.scalar_field.p]
compartment = lower
initial.expression = 1 + position_x
storage.expression = 1
cross_diffusion.p.expression = 0.05
reaction.expression = -0.3*p^2
reaction.jacobian.p.expression = -0.6*p
outflow.upper.expression = 0.4*(p - q) + 0.05*normal_z
outflow.upper.jacobian.p.expression = 0.4
outflow.upper.jacobian.q.expression = -0.4

[model.scalar_field.q]
compartment = upper
initial.expression = 0.2*position_y
storage.expression = 1
cross_diffusion.q.type = tensor
cross_diffusion.q.xx.expression = 0.02
cross_diffusion.q.yy.expression = 0.03
cross_diffusion.q.zz.expression = 0.04
cross_diffusion.q.xz.expression = 0.005
outflow.lower.expression = 0.4*(q - p)
outflow.lower.jacobian.q.expression = 0.4
outflow.lower.jacobian.p.expression = -0.4

[model.scalar_field.r]
compartment = upper
initial.expression = 0.5
storage.expression = 1
reaction.expression = 0.1*q - 0.2*r
reaction.jacobian.q.expression = 0.1
reaction.jacobian.r.expression = -0.2
cross_diffusion.r.expression = 0.01

[model.time_step_operator]
type = ImplicitEuler
time_end = 0.3
time_step_max = 0.1

[model.time_step_operator.nonlinear_solver]
convergence_condition.relative_tolerance = 1e-16
"""

# Poisson problem with a quadratic exact solution: -div(grad u) = -2 dim, u = |x|^2 on the
# boundary (constrain.boundary), linear model, one implicit Euler step; P1 on the Kuhn
# split is nodally exact for it.
POISSON_INI = """
[grid]
dimension = 2
cells = 12 12

[compartments.domain]
expression = 1

[parser_context.dim]
type = constant
value = 2

[model]
is_linear = true

[model.scalar_field.u]
compartment = domain
initial.expression = 0
cross_diffusion.u.expression = 1
reaction.expression = -2*dim
constrain.boundary.expression = in_boundary ? position_x^2 + position_y^2 + position_z^2 : no_value

[model.time_step_operator]
type = ImplicitEuler
time_end = 0.1
time_step_initial = 0.1
time_step_max = 0.1
"""

# Two compartments, two species each: the left part of the outer boundary held by a
# constrain.boundary expression that also reads normal and face measure, interior vertices
# of a strip held by constrain.skeleton, one species whose constraint is the zero literal
# (no constraint at all), a transient nonlinear model stepped with Alexander2.
CONSTRAINED_INI = """
[grid]
dimension = 2
cells = 10 10

[compartments]
left.expression = position_x < 0.6
right.expression = position_x >= 0.6

[model.scalar_field.a]
compartment = left
initial.expression = 0.2 + position_y
storage.expression = 1
cross_diffusion.a.expression = 0.05
reaction.expression = -a*b
reaction.jacobian.a.expression = -b
reaction.jacobian.b.expression = -a
constrain.boundary.expression = position_x < 1e-12 ? 1 + position_y + 0*normal_x + 0*entity_volume : no_value
outflow.right.expression = 0.3*(a - c)
outflow.right.jacobian.a.expression = 0.3
outflow.right.jacobian.c.expression = -0.3

[model.scalar_field.b]
compartment = left
initial.expression = 0.5
storage.expression = 1
cross_diffusion.b.expression = 0.02
reaction.expression = -a*b
reaction.jacobian.a.expression = -b
reaction.jacobian.b.expression = -a
constrain.skeleton.expression = position_y > 0.45 and position_y < 0.55 ? 0.9 : no_value

[model.scalar_field.c]
compartment = right
initial.expression = 0.1
storage.expression = 1
cross_diffusion.c.expression = 0.04
constrain.boundary.expression = 0
outflow.left.expression = 0.3*(c - a)
outflow.left.jacobian.c.expression = 0.3
outflow.left.jacobian.a.expression = -0.3

[model.scalar_field.d]
compartment = right
initial.expression = 0.3
storage.expression = 1
cross_diffusion.d.expression = 0.01
reaction.expression = 0.2*c - 0.1*d
reaction.jacobian.c.expression = 0.2
reaction.jacobian.d.expression = -0.1
constrain.boundary.expression = normal_y > 0.5 ? 0.25 + 0*entity_volume : no_value

[model.time_step_operator]
type = Alexander2
time_end = 0.2
time_step_initial = 0.05
time_step_max = 0.05

[model.time_step_operator.nonlinear_solver]
convergence_condition.relative_tolerance = 1e-16
"""

# transform/reduce operators of the exponential-decay model: an integral, a max with an
# explicit reduction and initial value, an L2 error with transformation and error check,
# and a reduction function outside the sum/max/min forms (folded in cell order)
REDUCE_SECTION = """
[model.reduce]
mass.evaluation.expression = u*integration_factor
umax.evaluation.expression = u
umax.reduction.expression = acc, val: max(acc, val)
umax.initial.value = -1e100
err.evaluation.expression = (u - exp(grow_rate*time))^2 * integration_factor
err.transformation.expression = e: sqrt(e)
err.error.expression = e: e > 5e-3
area.evaluation.expression = integration_factor
area.warn.expression = a: a > 0.5
mixed.evaluation.expression = u*position_x + grad_u_x
mixed.reduction.expression = p, q: q + 0.5*p
"""

DECAY_INI = """
[grid]
dimension = 2
cells = 6 5
extensions = 1.2 1

[compartments.domain]
expression = 1

[parser_context.grow_rate]
type = constant
value = -2

[model.scalar_field.u]
compartment = domain
initial.expression = 1 + 0.01*position_x*position_y
storage.expression = 1
reaction.expression = grow_rate*u
reaction.jacobian.u.expression = grow_rate

[model.time_step_operator]
type = ImplicitEuler
time_end = 0.5
time_step_initial = 0.1
time_step_max = 0.1
""" + REDUCE_SECTION


def write_gmsh(path, dim=2, n=8, seed=5):
    """A Gmsh MSH 2.2 ASCII file of the Kuhn-split unit square / cube with interior vertices
    displaced by up to 0.2 h (an unstructured-looking grid), node ids offset and with a gap,
    physical entity 1 for cells whose centre has x < 0.5 and 2 otherwise, and boundary
    line / point elements that the reader must skip."""
    from oracle.mesh import structured_simplex
    coords, cells = structured_simplex(dim, [n] * dim, [0.0] * dim, [1.0] * dim)
    rng = np.random.default_rng(seed)
    interior = np.all((coords > 1e-12) & (coords < 1 - 1e-12), axis=1)
    coords = coords.copy()
    coords[interior] += rng.uniform(-0.2, 0.2, (interior.sum(), dim)) / n
    ids = np.arange(coords.shape[0]) + 10
    ids[coords.shape[0] // 2:] += 7                      # a gap in the node ids
    ctr = coords[cells].mean(axis=1)
    phys = np.where(ctr[:, 0] < 0.5, 1, 2)
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(coords.shape[0])]
    for k in range(coords.shape[0]):
        xyz = list(coords[k]) + [0.0] * (3 - dim)
        lines.append("%d %.17g %.17g %.17g" % (ids[k], *xyz))
    lines += ["$EndNodes", "$Elements"]
    elems = ["1 15 2 9 9 %d" % ids[0], "2 1 2 7 7 %d %d" % (ids[0], ids[1])]
    typ = 2 if dim == 2 else 4
    for e in range(cells.shape[0]):
        elems.append("%d %d 2 %d %d " % (e + 3, typ, phys[e], 100 + phys[e]) + " ".join(str(ids[v]) for v in cells[e]))
    lines += [str(len(elems))] + elems + ["$EndElements"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return coords, cells, phys


def gmsh_ini(path, dim=2):
    """Two compartments selected by the Gmsh physical entity, one species each coupled
    through an outflow term, Alexander2 steps."""
    return """
[grid]
dimension = %d
path = %s

[compartments]
left.expression = gmsh_id == 1
right.expression = gmsh_id == 2

[model.scalar_field.u]
compartment = left
initial.expression = 1 + position_x*position_y
storage.expression = 1
cross_diffusion.u.expression = 0.05
reaction.expression = -0.5*u^2
reaction.jacobian.u.expression = -u
outflow.right.expression = 0.3*(u - v)
outflow.right.jacobian.u.expression = 0.3
outflow.right.jacobian.v.expression = -0.3

[model.scalar_field.v]
compartment = right
initial.expression = 0.2
storage.expression = 1
cross_diffusion.v.expression = 0.02
outflow.left.expression = 0.3*(v - u)
outflow.left.jacobian.v.expression = 0.3
outflow.left.jacobian.u.expression = -0.3

[model.time_step_operator]
type = Alexander2
time_end = 0.2
time_step_initial = 0.05
time_step_max = 0.05

[model.time_step_operator.nonlinear_solver]
convergence_condition.relative_tolerance = 1e-16
""" % (dim, path)


def context_ini(tiff_a, tiff_b, n=20):
    """Three species whose initial concentrations come from grayscale TIFF images (the
    shape of the reference's test/time_snap.ini, on a structured square), with a function
    tabulated over position (clamped), a function tabulated over the state, and an
    interpolation table in the coefficients."""
    return """
[grid]
dimension = 2
cells = {n} {n}

[compartments.domain]
expression = 1

[parser_context.A_initialConcentration]
type = tiff
path = {a}

[parser_context.B_initialConcentration]
type = tiff
path = {b}

[parser_context.dprofile]
type = function
expression = x: 0.2 + 0.1*sin(6*x)
interpolate = true
interpolation.intervals = 64
interpolation.domain.x = 0 1
interpolation.out_of_bounds = clamp

[parser_context.sat]
type = function
expression = c: c/(50 + c)
interpolate = true
interpolation.intervals = 4000
interpolation.domain.c = 0 2000
interpolation.out_of_bounds = clamp

[parser_context.ramp]
type = interpolation
domain = 0 0.3 0.7 1
range = 1 1.5 0.5 1

[model.scalar_field.A]
compartment = domain
cross_diffusion.A.expression = 0.4
reaction.expression = A*B*1e-06*-100.0*ramp(position_y) - 0.01*sat(A)
reaction.jacobian.A.expression = B*1e-06*-100.0*ramp(position_y)
reaction.jacobian.B.expression = A*1e-06*-100.0*ramp(position_y)
storage.expression = 1
initial.expression = 1000*A_initialConcentration(position_x,position_y)

[model.scalar_field.B]
compartment = domain
cross_diffusion.B.expression = 0.4
reaction.expression = A*B*1e-06*-100.0*ramp(position_y)
reaction.jacobian.A.expression = B*1e-06*-100.0*ramp(position_y)
reaction.jacobian.B.expression = A*1e-06*-100.0*ramp(position_y)
storage.expression = 1
initial.expression = 1000*B_initialConcentration(position_x,position_y)

[model.scalar_field.C]
compartment = domain
cross_diffusion.C.expression = 25*dprofile(position_x)
reaction.expression = A*B*1e-06*100.0*ramp(position_y) + B_initialConcentration(position_x, position_y)
reaction.jacobian.A.expression = B*1e-06*100.0*ramp(position_y)
reaction.jacobian.B.expression = A*1e-06*100.0*ramp(position_y)
storage.expression = 1
initial.expression = 0

[model.time_step_operator]
type = ImplicitEuler
time_step_initial = 0.1
time_end = 0.2
""".format(n=n, a=tiff_a, b=tiff_b)
