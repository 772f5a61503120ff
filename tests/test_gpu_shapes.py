"""Run-time block shapes of the element and node kernels (ses3d_gpu_set_kernel_shape) and the
autotuner that searches them: every shape gives the same bits, lean and full state, and
the autotuner keeps one of the timed candidates."""
import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu


def run(p, steps, lean, shape, node_block, graph=10):
    from ses3d_gb300.solver import Simulation
    with Simulation.from_problem(p) as sim:
        sim.set_lean(lean)
        sim.set_kernel_shape(shape, node_block)
        if graph:
            sim.use_graph(True, graph)
        sim.step(steps)
        return [sim.field("vx_global"), sim.field("vz_global"), sim.field("sxz_pml"),
                np.concatenate(sim.seismograms(0))]


@pytest.mark.parametrize("lean", [False, True])
def test_all_shapes_bit_identical(native, lean):
    from ses3d_gb300 import _lib
    p = synth.make_problem("small", nt=30, seed=81)
    ref = run(p, 30, lean, 0, 256)
    assert np.abs(ref[0]).max() > 0
    n = int(_lib.load().ses3d_gpu_kernel_shape_count())
    assert n >= 2
    for shape in range(n):
        for nb in (128, 256, 512):
            out = run(p, 30, lean, shape, nb)
            for a, b in zip(ref, out):
                assert np.array_equal(a, b), (shape, nb)


def test_shape_arguments_checked(native):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=4, seed=82)
    with Simulation.from_problem(p) as sim:
        assert sim.lib.ses3d_gpu_set_kernel_shape(sim.h, -1, 256) == -1
        assert sim.lib.ses3d_gpu_set_kernel_shape(sim.h, 0, 300) == -1
        assert sim.lib.ses3d_gpu_set_kernel_shape(sim.h, 99, 256) == -1


def test_autotune_keeps_a_timed_candidate(native):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("small", nt=60, seed=83)
    with Simulation.from_problem(p) as sim:
        tuned = sim.autotune(steps_each=2)
        chosen = tuned["chosen"]
        assert tuned["element"] and tuned["node"]
        best = min(tuned["element"], key=tuned["element"].get)
        assert "epb=%d" % chosen["elements_per_cta"] in best
        assert chosen["node_block"] == min(tuned["node"], key=tuned["node"].get)
        assert sim.shape == chosen
        it = sim.it
        sim.run()                                   # the run continues with the chosen shape
        assert sim.it == 60 and it < 60
