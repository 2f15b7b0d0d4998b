"""Failure detection on the GPU without a fault: the single-launch solve's grid-wide waits
are bounded in time; a barrier that cannot complete must give up in every block, report it
to the host, and leave the CUDA context usable."""

import pytest

import cases

pytestmark = pytest.mark.gpu


def test_bounded_barrier_wait_gives_up_and_context_survives(dcgpu_lib):
    gave_up, ms = dcgpu_lib.selftest_barrier_timeout()
    assert gave_up == 4            # every block's wait ran out and flagged it
    assert 40.0 <= ms <= 2000.0    # the 50 ms limit, not a hang
    # the context still runs work: a model steps normally afterwards
    ini, _ = cases.small_heat(n=8, steps=1)
    gm = dcgpu_lib.Model(ini)
    info = gm.step(0.01)
    gm.close()
    assert info["status"] == 0 and info["newton_iterations"] >= 1
