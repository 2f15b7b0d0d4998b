"""CPU oracle for the implicit-step hot path of DuneCopasi (TEST INFRASTRUCTURE).

This package is a plain numpy/scipy restatement of the reference algorithm:
P1 continuous-Galerkin residual and Jacobian assembly of the multi-compartment
diffusion-reaction operator (dune/copasi/model/diffusion_reaction/local_operator.hh),
the Newton solve configured in dune/copasi/model/make_step_operator.hh:246-288,
the Runge-Kutta stage loop (ImplicitEuler / Alexander2 / ...), and the adaptive
stepper of dune/copasi/common/stepper.hh.

It is a CHECKER only.  Only tests, the smoke check and the CPU-baseline leg of the
benchmark may import it; the GPU product never links, imports or falls back to it.

Parity pins: the reference ships no golden vectors for this path.  The oracle is
pinned against the reference's own known-answer system tests (test/exp.ini,
test/gauss.ini analytic-error thresholds) and against closed-form finite-element
identities (P1 mass/stiffness stencils on the structured simplex grid); per-species
1e-8 parity with the reference binary itself is unpinned because the reference
(DUNE + PDELab + UGGrid + SuiteSparse) cannot be built in this environment.
"""
