"""C-ABI argument and call-order validation: each bad call returns its status code and a
message, launches nothing, and leaves the handle usable -- a run with every rejected call
interleaved gives the same bits as an undisturbed run."""
import ctypes

import numpy as np
import pytest

from ses3d_gb300 import _lib as L
from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

CONFIG, STATE = -1, -4


def bad_calls(sim, lib):
    """(name, thunk returning the status, expected status, message fragment)."""
    h = sim.h
    out_f = np.zeros(sim.N, np.float32)
    out_d = np.zeros(sim.N, np.float64)
    stf = np.zeros(sim.nt, np.float32)
    mom = np.zeros(6, np.float32)
    nr = ctypes.c_int(0)
    return [
        ("event out of range", lambda: lib.ses3d_gpu_set_source(h, 5, 50.0, 10.0, 1000.0, 10, L.fptr(mom), L.fptr(stf),
                                                                 None), CONFIG, b"event index"),
        ("null stf", lambda: lib.ses3d_gpu_set_source(h, 0, 50.0, 10.0, 1000.0, 10, L.fptr(mom), None, None),
         CONFIG, b"stf"),
        ("negative receiver count", lambda: lib.ses3d_gpu_set_receivers(h, 0, -1, None, ctypes.byref(nr), None),
         CONFIG, b"receiver"),
        ("negative adjoint count", lambda: lib.ses3d_gpu_set_adjoint_sources(h, 0, -1, None, None, None),
         CONFIG, b"adjoint source"),
        ("negative step count", lambda: lib.ses3d_gpu_step(h, -1), CONFIG, b"n must be"),
        ("unknown field", lambda: lib.ses3d_gpu_get_field(h, 0, 999, L.fptr(out_f)), CONFIG, b"unknown field"),
        ("mass matrix is read-only", lambda: lib.ses3d_gpu_set_field(h, 0, L.FIELD_ID["MM_global"], L.fptr(out_f)),
         CONFIG, b"read-only"),
        ("kernel of a forward run", lambda: lib.ses3d_gpu_get_kernel(h, 0, 0, L.dptr(out_d)), STATE, b"adjoint"),
        ("kernel sum of a forward run", lambda: lib.ses3d_gpu_get_kernel_sum(h, 0, L.dptr(out_d)), STATE, b"adjoint"),
        ("bad kernel id", lambda: lib.ses3d_gpu_get_kernel_sum(h, 99, L.dptr(out_d)), CONFIG, b"kernel id"),
        ("wait limit", lambda: lib.ses3d_gpu_selftest_wait(h, 0), CONFIG, b"limit_ms"),
        ("graph length", lambda: lib.ses3d_gpu_use_graph(h, 1, 0), CONFIG, b"n_per_graph"),
        ("checkpointing outside a flag-1 run", lambda: lib.ses3d_gpu_set_checkpointing(h, 4), STATE, b"checkpointing"),
        ("record of a forward run", lambda: lib.ses3d_gpu_get_record(h, 0, 0, L.fptr(out_f)), CONFIG, b"record"),
        ("unknown setup real", lambda: lib.ses3d_gpu_get_setup_real(h, 0, b"nope", None), CONFIG, b"unknown setup"),
        ("unknown setup integer", lambda: lib.ses3d_gpu_get_setup_int(h, 0, b"nope", None), CONFIG, b"unknown setup"),
    ]


def test_rejected_calls_leave_the_handle_usable(native):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=20, seed=61)
    with Simulation.from_problem(p) as ref:
        ref.run()
        want = (ref.field("vz_global"), np.concatenate(ref.seismograms(0)))
    with Simulation.from_problem(p) as sim:
        calls = bad_calls(sim, native)
        for k, (name, call, code, frag) in enumerate(calls):
            before = sim.launch_count
            rc = call()
            assert rc == code, (name, rc)
            assert frag in native.ses3d_gpu_last_error(sim.h), (name, native.ses3d_gpu_last_error(sim.h))
            assert sim.launch_count == before, name
            if k % 4 == 0:
                sim.step(1)
        sim.run()
        got = (sim.field("vz_global"), np.concatenate(sim.seismograms(0)))
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_adjoint_handle_rejections(native):
    """Lean stepping of a flag-1 run is chosen before it starts and cannot change during it;
    records are refused once checkpointing replaces them; external stepping needs a 16-byte
    aligned state buffer and a plain run."""
    import torch
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=20, seed=62, adjoint_flag=1)
    with Simulation.from_problem(p, adjoint_flag=1) as sim:
        assert native.ses3d_gpu_set_lean(sim.h, 1) == 0
        assert native.ses3d_gpu_set_checkpointing(sim.h, 4) == 0
        sim.step(2)
        assert native.ses3d_gpu_set_lean(sim.h, 0) == STATE
        assert b"chosen before the run starts" in native.ses3d_gpu_last_error(sim.h)
        sim.run()
        out = np.zeros(sim.N * 9, np.float32)
        assert native.ses3d_gpu_get_record(sim.h, 0, 0, L.fptr(out)) == STATE
        state = torch.empty(36 * sim.N, dtype=torch.float32, device="cuda")
        v = torch.empty(3 * sim.G, dtype=torch.float32, device="cuda")
        assert native.ses3d_gpu_step_external(sim.h, ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(v.data_ptr()),
                                              1) == CONFIG
    with Simulation.from_problem(synth.make_problem("tiny", nt=20, seed=62)) as sim:
        state = torch.empty(36 * sim.N + 4, dtype=torch.float32, device="cuda")
        v = torch.empty(3 * sim.G, dtype=torch.float32, device="cuda")
        rc = native.ses3d_gpu_step_external(sim.h, ctypes.c_void_p(state.data_ptr() + 4),
                                            ctypes.c_void_p(v.data_ptr()), 1)
        assert rc == CONFIG and b"16-byte" in native.ses3d_gpu_last_error(sim.h)
        assert sim.it == 0


def test_out_of_memory_is_reported_and_leaves_the_library_usable(native):
    """A handle whose element state cannot fit (64 events on the 96 x 96 x 40 mesh, 424 GB)
    fails with SES3D_E_OOM and frees what it had allocated; a following handle steps and
    its launches are not blamed for the failed allocation."""
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation, config_from
    p = synth.make_problem("c2", nt=5, seed=63, model=False, n_events=1)
    cfg = config_from(p.box, p.setup, 5, p.events[0].event.dt, p.tau, p.D, pml=p.pml, n_events=64)
    with pytest.raises(_lib.Ses3dError) as ei:
        Simulation(cfg)
    assert ei.value.code == -2 and "allocation" in str(ei.value)
    q = synth.make_problem("tiny", nt=10, seed=64)
    with Simulation.from_problem(q) as sim:
        sim.run()
        assert np.abs(np.concatenate(sim.seismograms(0))).max() > 0


def test_select_device(native):
    """Device selection for one-rank-per-GPU processes: an index outside the visible devices
    is refused, the first device is accepted and handles are created on it."""
    import torch
    from ses3d_gb300.solver import Simulation, select_device
    assert native.ses3d_gpu_select_device(torch.cuda.device_count() + 3) == CONFIG
    assert b"device index" in native.ses3d_gpu_last_error(None)
    select_device(0)
    with Simulation.from_problem(synth.make_problem("tiny", nt=5, seed=65)) as sim:
        sim.run()
