"""The allocation-free entry point ses3d_gpu_step_external.

It serves callers that cannot call cudaMalloc where they step the solver (their device
memory belongs to another allocator, such as PyTorch's caching allocator used here, or
they run in a loop that must not allocate): the caller owns the wavefield, and the
element forces live in the library's fixed 32 MiB device array. These tests call it
through the C ABI with torch-owned buffers and check, on two calls in a row, that it
gives what the allocating entry point ses3d_gpu_step gives, within the tolerances of
the other GPU tests. This file sorts last so that a run stopping at the first failure
has run every other test already.
"""
import ctypes

import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

SEIS_TOL = 1e-5   # the FP32 seismogram tolerance of the forward parity tests
FIELD_TOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def internal_to_reference(state, n_el, field):
    """One field of the element-blocked state (element, 36 fields, 125 nodes) in the
    reference layout (element index fastest)."""
    return np.ascontiguousarray(state.reshape(n_el, 36, 125)[:, field, :].T).reshape(-1)


def test_external_step_matches_step_two_calls(native):
    import torch
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    lib = _lib.load()
    p = synth.make_problem("tiny", nt=12, seed=44)
    with Simulation.from_problem(p) as a, Simulation.from_problem(p) as b:
        N, G = a.N, a.G
        E = N // 125
        state = torch.zeros(36 * N, dtype=torch.float32, device="cuda")
        v = torch.zeros(3 * G, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        for call in range(2):
            a.step(3)
            rc = lib.ses3d_gpu_step_external(b.h, ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(v.data_ptr()), 3)
            assert rc == 0, lib.ses3d_gpu_last_error(b.h)
            torch.cuda.synchronize()
            assert a.it == b.it == 3 * (call + 1)
            vb = v.cpu().numpy()
            for c, name in enumerate(("vx_global", "vy_global", "vz_global")):
                va = a.field(name)
                assert np.abs(va).max() > 0
                assert rel(vb[c * G:(c + 1) * G], va) <= FIELD_TOL, (call, name)
            sb = state.cpu().numpy()
            for f, name in ((0, "sxx_pml"), (6, "syx_pml"), (9, "dxux"), (17, "dzuy")):
                assert rel(internal_to_reference(sb, E, f), a.field(name)) <= FIELD_TOL, (call, name)
            sa, sbs = a.seismograms(0), b.seismograms(0)
            for c in range(3):
                assert rel(sbs[c], sa[c]) <= SEIS_TOL, (call, c)


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
