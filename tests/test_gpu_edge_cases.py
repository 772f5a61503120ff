"""Edge cases of the inputs: the smallest mesh, no PML, events without receivers next to
events with receivers, a source outside the box, a single time step, receivers outside
the box. Compared with the oracle where it applies, else checked for the exact expected
behaviour."""
import numpy as np
import pytest

from ses3d_gb300 import formats as F
from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n_el,pml", [((1, 1, 1), 0), ((2, 1, 3), 0), ((3, 3, 2), 1)])
def test_smallest_meshes_match_oracle(native, oracle_mod, n_el, pml):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=30, seed=51, n_el=n_el, pml=pml)
    with Simulation.from_problem(p) as sim:
        sim.run()
        v = sim.field("vz_global")
        seis = sim.seismograms(0)
    o = oracle_mod.Oracle(p)
    o.run(30)
    assert np.abs(o.get("vz_global")).max() > 0
    assert rel(v, o.get("vz_global")) <= 1e-5
    r = o.seismograms()
    for c in range(3):
        if np.abs(r[c]).max() > 0:
            assert rel(seis[c], r[c]) <= 1e-5


def test_event_without_receivers_in_a_batch(native):
    """A batch where event 1 has no receivers: its seismograms are empty, the others equal
    their single-event runs."""
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=30, seed=52, n_events=3)
    p.events[1].receivers = F.Receivers([], np.zeros((0, 3), np.float32))
    with Simulation.from_problem(p) as sim:
        sim.run()
        assert sim.n_receivers(1) == 0 and sim.seismograms(1)[0].shape == (0, 30)
        batched = [sim.seismograms(k) for k in (0, 2)]
    for k, got in zip((0, 2), batched):
        q = synth.Problem(p.setup, p.box, p.tau, p.D, p.model, [p.events[k]], pml=p.pml)
        with Simulation.from_problem(q) as one:
            one.run()
            ref = one.seismograms(0)
        for c in range(3):
            assert np.array_equal(got[c], ref[c])


def test_source_outside_the_box_leaves_the_field_at_rest(native):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=20, seed=53)
    ev = p.events[0]
    with Simulation.from_problem(p) as sim:
        is_src = sim.set_source(0, np.float32(85.0), ev.event.yys, ev.event.zzs, ev.event.source_type, ev.event.mom,
                                ev.stf)
        assert not is_src
        sim.run()
        assert np.all(sim.field("vz_global") == 0) and np.all(np.concatenate(sim.seismograms(0)) == 0)


def test_receivers_outside_the_box_are_dropped(native, oracle_mod):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=20, seed=54)
    inside = p.events[0].receivers.loc
    outside = np.array([[89.0, 5.0, 0.0], [45.0, 95.0, 0.0], [50.0, 10.0, 700000.0]], np.float32)
    loc = np.concatenate([inside[:2], outside[:2], inside[2:], outside[2:]])
    with Simulation.from_problem(p) as sim:
        kept = sim.set_receivers(0, loc)
        assert list(kept) == [0, 1] + list(range(4, 2 + len(inside)))
        sim.run()
        got = sim.seismograms(0)
    o = oracle_mod.Oracle(p)
    o.run(20)
    want = o.seismograms()
    for c in range(3):
        assert got[c].shape == want[c].shape and rel(got[c], want[c]) <= 1e-5


def test_single_time_step(native, oracle_mod):
    """nt = 1: the receivers record the initial (zero) velocity, the field moves."""
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=1, seed=55)
    with Simulation.from_problem(p) as sim:
        sim.run()
        assert sim.it == 1
        assert np.all(np.concatenate(sim.seismograms(0)) == 0)   # seismogram(1) = v before the update
        v = sim.field("vx_global")
    o = oracle_mod.Oracle(p)
    o.run(1)
    assert rel(v, o.get("vx_global")) <= 1e-5
