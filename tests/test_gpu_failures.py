"""Failure detection on the GPU without a GPU fault: the bounded device wait gives up and
reports through the error word, and the handle keeps working afterwards."""
import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_handle_stays_usable(native):
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    lib = _lib.load()
    p = synth.make_problem("tiny", nt=30, seed=81)
    with Simulation.from_problem(p) as ref:
        ref.run()
        want = ref.field("vz_global"), np.concatenate(ref.seismograms(0))
    with Simulation.from_problem(p) as sim:
        sim.step(10)
        rc = lib.ses3d_gpu_selftest_wait(sim.h, 50)    # a wait that nothing completes, 50 ms limit
        assert rc == -3
        assert b"bounded wait expired" in lib.ses3d_gpu_last_error(sim.h)
        assert lib.ses3d_gpu_selftest_wait(sim.h, 0) == -1   # limit validated
        sim.step(20)                                      # the context and handle are still usable
        assert np.array_equal(sim.field("vz_global"), want[0])
        assert np.array_equal(np.concatenate(sim.seismograms(0)), want[1])
