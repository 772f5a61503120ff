"""The allocation-free entry point ses3d_gpu_step_external.

It serves callers that cannot call cudaMalloc where they step the solver (their device
memory belongs to another allocator, such as PyTorch's caching allocator used here, or
they run in a loop that must not allocate): the caller owns the wavefield, and the
element forces live in the library's fixed 32 MiB device array. These tests call it
through the C ABI with torch-owned buffers and check, on two calls in a row, that it
gives what the allocating entry point ses3d_gpu_step gives. Both run the same kernels on
the same values, so the results must agree bit for bit (a stricter bar than the FP32
tolerance of the oracle parity tests). This file sorts last so that a run stopping at
the first failure has run every other test already.
"""
import ctypes

import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

STRESSES = ("sxx_pml", "syy_pml", "szz_pml", "sxy_pml", "sxz_pml", "syz_pml", "syx_pml", "szx_pml", "szy_pml")
# position of each field in the element-blocked state (the header's field order)
BLOCK_INDEX = {"sxx_pml": 0, "syy_pml": 1, "szz_pml": 2, "sxy_pml": 3, "sxz_pml": 4, "syz_pml": 5,
               "syx_pml": 6, "szx_pml": 7, "szy_pml": 8, "dxux": 9, "dzuy": 17}
MEMVARS = ("Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz")


def block_to_reference(state, n_ev, n_el, ev, field):
    """One field of one event of the element-blocked state (event, element, 36 fields, 125
    nodes) in the reference layout (element index fastest)."""
    return np.ascontiguousarray(state.reshape(n_ev, n_el, 36, 125)[ev, :, field, :].T).reshape(-1)


def memvar_to_reference(state, n_ev, n_el, ev, comp):
    """Memory variable comp (0..5) of one event in the reference layout (3, elements x 125
    points, mechanism fastest)."""
    m = state.reshape(n_ev, n_el, 36, 125)[ev, :, 18 + 3 * comp:21 + 3 * comp, :]  # (E, 3, 125)
    return np.ascontiguousarray(np.transpose(m, (2, 0, 1))).reshape(-1)


def external(lib, sim, state, v, n):
    rc = lib.ses3d_gpu_step_external(sim.h, ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(v.data_ptr()), n)
    assert rc == 0, lib.ses3d_gpu_last_error(sim.h)


def check_same(a, state, v, n_ev, stresses, memvars=True, extra=()):
    """The caller-owned wavefield and the handle's seismograms against the handle `a` that
    stepped with ses3d_gpu_step: bit-identical."""
    G, N = a.G, a.N
    E = N // 125
    vb = v.cpu().numpy()
    sb = state.cpu().numpy()
    for ev in range(n_ev):
        for c, name in enumerate(("vx_global", "vy_global", "vz_global")):
            va = a.field(name, ev)
            assert np.abs(va).max() > 0
            got = vb[(3 * ev + c) * G:(3 * ev + c + 1) * G]
            assert np.array_equal(got, va), (ev, name)
        for name in tuple(stresses) + tuple(extra):
            assert np.array_equal(block_to_reference(sb, n_ev, E, ev, BLOCK_INDEX[name]), a.field(name, ev)), (ev, name)
        if memvars:
            for comp, name in enumerate(MEMVARS):
                assert np.array_equal(memvar_to_reference(sb, n_ev, E, ev, comp), a.field(name, ev)), (ev, name)
    return True


def test_external_step_matches_step_two_calls(native):
    """One event, two calls in a row of three steps: wavefield and seismograms equal those
    of ses3d_gpu_step bit for bit after each call."""
    import torch
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    lib = _lib.load()
    p = synth.make_problem("tiny", nt=12, seed=44)
    with Simulation.from_problem(p) as a, Simulation.from_problem(p) as b:
        state = torch.zeros(36 * a.N, dtype=torch.float32, device="cuda")
        v = torch.zeros(3 * a.G, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        for call in range(2):
            a.step(3)
            external(lib, b, state, v, 3)
            torch.cuda.synchronize()
            assert a.it == b.it == 3 * (call + 1)
            check_same(a, state, v, 1, STRESSES, extra=("dxux", "dzuy"))
            sa, sbs = a.seismograms(0), b.seismograms(0)
            for c in range(3):
                assert np.abs(sa[c]).max() > 0
                assert np.array_equal(sbs[c], sa[c]), (call, c)


def test_external_step_several_items_per_cta(native):
    """A 20 x 20 x 10 mesh (several elements per CTA of the persistent element kernel) from
    the same random initial velocity in both handles: two calls of three steps equal
    ses3d_gpu_step bit for bit."""
    import torch
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    lib = _lib.load()
    p = synth.make_problem("tiny", nt=12, seed=48, n_el=(20, 20, 10))
    rng = np.random.default_rng(3)
    with Simulation.from_problem(p) as a, Simulation.from_problem(p) as b:
        vel = [(1e-3 * rng.standard_normal(a.G)).astype(np.float32) for _ in range(3)]
        for name, x in zip(("vx_global", "vy_global", "vz_global"), vel):
            a.set_field(name, x)
        state = torch.zeros(36 * a.N, dtype=torch.float32, device="cuda")
        v = torch.from_numpy(np.concatenate(vel)).to("cuda")
        torch.cuda.synchronize()
        for call in range(2):
            a.step(3)
            external(lib, b, state, v, 3)
            torch.cuda.synchronize()
            check_same(a, state, v, 1, STRESSES, extra=("dxux", "dzuy"))
            sa, sbs = a.seismograms(0), b.seismograms(0)
            for c in range(3):
                assert np.abs(sa[c]).max() > 0
                assert np.array_equal(sbs[c], sa[c]), (call, c)


def test_external_step_two_events_lean_then_full(native):
    """Two events on a mesh with elements outside the PML: a lean call, then a call with
    lean stepping off (the mirror stresses of the caller's buffer are brought up to date
    first), each compared bit for bit with ses3d_gpu_step doing the same switch."""
    import torch
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    lib = _lib.load()
    p = synth.make_problem("small", nt=12, seed=46, n_events=2)
    with Simulation.from_problem(p) as a, Simulation.from_problem(p) as b:
        state = torch.zeros(2 * 36 * a.N, dtype=torch.float32, device="cuda")
        v = torch.zeros(2 * 3 * a.G, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        for call, lean in enumerate((True, False)):
            a.set_lean(lean)
            b.set_lean(lean)
            a.step(3)
            external(lib, b, state, v, 3)
            torch.cuda.synchronize()
            # after the lean call the caller's mirrors outside the PML are behind: the first
            # six stresses are compared then, all nine after the full-state call
            check_same(a, state, v, 2, STRESSES[:6] if lean else STRESSES)
            for ev in range(2):
                sa, sbs = a.seismograms(ev), b.seismograms(ev)
                for c in range(3):
                    assert np.abs(sa[c]).max() > 0
                    assert np.array_equal(sbs[c], sa[c]), (call, ev, c)


def test_external_and_own_stepping_do_not_mix(native):
    """A handle steps either its own wavefield or caller-owned ones: the other path is
    refused with SES3D_E_STATE, and nothing is stepped."""
    import torch
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    lib = _lib.load()
    p = synth.make_problem("tiny", nt=6, seed=47)
    with Simulation.from_problem(p) as a, Simulation.from_problem(p) as b:
        state = torch.zeros(36 * a.N, dtype=torch.float32, device="cuda")
        v = torch.zeros(3 * a.G, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        a.step(1)
        rc = lib.ses3d_gpu_step_external(a.h, ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(v.data_ptr()), 1)
        assert rc == -4 and a.it == 1
        external(lib, b, state, v, 1)
        assert lib.ses3d_gpu_step(b.h, 1) == -4 and b.it == 1
        with pytest.raises(_lib.Ses3dError) as err:
            b.field("vz_global")
        assert err.value.code == -4
        assert b.field("MM_global").size == b.G


def test_external_step_rejects_too_large_runs(native):
    import torch
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    lib = _lib.load()
    p = synth.make_problem("tiny", nt=2, n_el=(30, 30, 30), seed=45)  # 3.375M points: 3 x N > 8,388,608
    with Simulation.from_problem(p) as s:
        state = torch.zeros(16, dtype=torch.float32, device="cuda")
        v = torch.zeros(16, dtype=torch.float32, device="cuda")
        rc = lib.ses3d_gpu_step_external(s.h, ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(v.data_ptr()), 1)
        assert rc == -1
        assert b"32 MiB" in lib.ses3d_gpu_last_error(s.h)
        assert s.it == 0
