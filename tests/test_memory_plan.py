"""Memory plans of the misfit gradient (CPU, no GPU): which storage the gradient takes for a
mesh, time axis and device budget. The reference-kernel gradient keeps every forward record,
checkpoints every K records (one recompute pass), or adds a second level (two passes). The
exact discrete adjoint keeps full-state checkpoints and per-iteration slots of the fields
its backward iteration reads."""
import math

import numpy as np
import pytest

from ses3d_gb300 import _lib as L
from ses3d_gb300 import adjoint as A


def setup_for(elements, nt, n_events=1, is_diss=1, budget=None):
    c = L.Config()
    c.nx, c.ny, c.nz = elements[0] - 1, elements[1] - 1, elements[2] - 1
    c.lpd, c.pml, c.is_diss, c.nt = 4, 3, is_diss, nt
    ev = A.EventData(50.0, 10.0, 15e3, 10, np.zeros(6, np.float32), np.zeros(nt, np.float32),
                     np.zeros((1, 3), np.float32))
    return A.MisfitSetup(c, [ev] * n_events, samp_ad=10, memory_budget=budget)


def points(elements):
    ex, ey, ez = elements
    return 125.0 * ex * ey * ez, float((4 * ex + 1) * (4 * ey + 1) * (4 * ez + 1))


def test_gradient_plan_prefers_fewest_recompute_passes():
    """64 x 64 x 32, nt = 4000: every record kept when the budget allows it, else one
    checkpoint level, else two; a sub-batch grows only within the first storage that fits."""
    s = setup_for((64, 64, 32), 4000, n_events=4, budget=280e9)
    m = s.memory_model()
    assert m["keep"] + m["shared"] < 280e9
    pl = s.plan()
    assert (pl.events_per_batch, pl.K, pl.K2) == (1, 0, 0)
    s.memory_budget = 150e9
    pl = s.plan()
    assert pl.K == m["K"] and pl.K2 == 0 and pl.events_per_batch >= 1
    assert m["shared"] + pl.events_per_batch * m["one_level"] <= 150e9
    s.memory_budget = m["shared"] + m["two_level"] + 1e9
    pl = s.plan()
    assert (pl.K, pl.K2) == (m["K1"], m["K2"]) and pl.events_per_batch == 1


def test_config5_gradient_fits_150_gb():
    """96 x 96 x 40, nt = 4000, 16 events, 150 GB: one event per sub-batch. Lean runs
    checkpoint 24 of the 36 fields outside the PML, which fits one level; full-state runs
    take two."""
    s = setup_for((96, 96, 40), 4000, n_events=16, budget=150e9)
    m = s.memory_model()
    pl = s.plan()
    assert pl.events_per_batch == 1 and pl.K2 == 0 and pl.K == m["K"]
    assert m["shared"] + m["one_level"] <= 150e9
    assert len(pl.groups) == 16
    s.lean = False
    m = s.memory_model()
    pl = s.plan()
    assert pl.events_per_batch == 1 and pl.K2 > 0 and (pl.K, pl.K2) == (m["K1"], m["K2"])
    assert m["shared"] + m["two_level"] <= 150e9 < m["shared"] + m["one_level"]


def exact_bytes(elements, nt, K, K2, is_diss):
    """Checkpoint and slot bytes of one event of the exact adjoint, restated from the
    library's allocation: checkpoints of 36 N + 3 G floats; slots of 1,876 E + 6 G floats
    with attenuation (15 fields of 125 nodes per element, padded to 16 bytes), 1,128 E + 6 G
    without."""
    N, G = points(elements)
    E = N / 125
    ckpt = (36 * N + 3 * G) * 4
    slot = ((1876 if is_diss else 1128) * E + 6 * G) * 4
    if K2:
        return math.ceil(nt / K) * ckpt + (math.ceil(K / K2) - 1) * ckpt + K2 * slot
    return math.ceil(nt / K) * ckpt + K * slot


@pytest.mark.parametrize("is_diss", [1, 0])
def test_exact_plan_one_level_on_the_64x64x32_misfit(is_diss):
    """The packed iteration slots let the 64 x 64 x 32, nt = 4000 exact gradient run with one
    checkpoint level (one recompute pass) inside 265 GB; at 150 GB it takes two levels."""
    s = setup_for((64, 64, 32), 4000, is_diss=is_diss, budget=265e9)
    pl = s.exact_plan()
    assert pl.K2 == 0 and pl.events_per_batch == 1
    assert exact_bytes((64, 64, 32), 4000, pl.K, 0, is_diss) < 225e9
    s.memory_budget = 150e9
    pl = s.exact_plan()
    assert 0 < pl.K2 < pl.K
    assert exact_bytes((64, 64, 32), 4000, pl.K, pl.K2, is_diss) < 110e9


def test_exact_plan_checkpoint_steps_override():
    s = setup_for((22, 22, 10), 1000, budget=100e9)
    s.checkpoint_steps = 50
    pl = s.exact_plan()
    assert pl.K == 50 and pl.K2 == 0
