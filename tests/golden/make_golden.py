"""Writes tests/golden/oracle_tiny.npz: outputs of the FP64 CPU oracle (the reference's
algorithm restated, oracle/) on two small seeded cases, with every input that is not a
deterministic function of the mesh, so that the fixture replays without the generator's
random streams.

  forward: 6 x 5 x 4 elements, anelastic, PML 3, moment-tensor source, 4 receivers,
           40 steps: seismograms and the final vertical velocity
  adjoint: the same mesh, records every 5 steps over 40 steps, two adjoint sources driven
           by the time-reversed forward seismograms: Frechet kernels (every 7th GLL point
           and the full-kernel L2 norms)

The reference itself cannot run in this environment (Fortran, no compiler), so these are
regression fixtures of the oracle, not reference outputs. Regenerate with
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ses3d_gb300 import synth  # noqa: E402

NT = 40
SAMP = 5
STRIDE = 7
OUT = os.path.join(HERE, "oracle_tiny.npz")


def case_inputs(seed: int):
    p = synth.make_problem("tiny", nt=NT, seed=seed, adjoint_flag=1)
    p.setup.samp_ad = SAMP
    e = p.events[0]
    return {"tau": p.tau, "D": p.D, "src": np.array([e.event.xxs, e.event.yys, e.event.zzs], np.float32),
            "mom": np.asarray(e.event.mom, np.float32), "dt": np.float32(e.event.dt),
            "stf": np.asarray(e.stf[:NT], np.float32), "recloc": np.asarray(e.receivers.loc, np.float32)}


def problem_from(g, prefix: str):
    """The synth.Problem of one golden case, rebuilt from the fixture's inputs."""
    p = synth.make_problem("tiny", nt=NT, seed=0, adjoint_flag=1)
    p.setup.samp_ad = SAMP
    p.tau = g[prefix + "tau"].copy()
    p.D = g[prefix + "D"].copy()
    e = p.events[0]
    e.event.xxs, e.event.yys, e.event.zzs = (np.float32(v) for v in g[prefix + "src"])
    e.event.mom = g[prefix + "mom"].copy()
    e.event.dt = np.float32(g[prefix + "dt"])
    e.stf = np.concatenate([g[prefix + "stf"], np.zeros(1, np.float32)])
    loc = g[prefix + "recloc"]
    e.receivers = type(e.receivers)(["G%03d" % i for i in range(len(loc))], loc.copy())
    return p


def adjoint_sources(p, seis):
    """Two adjoint sources at the first two receivers (1 km depth), driven by the
    time-reversed forward velocity, scaled to 1e10."""
    loc = p.events[0].receivers.loc[:2].copy()
    loc[:, 2] = np.float32(1000.0)
    stf = np.zeros((2, 3, NT), np.float32)
    for k in range(2):
        for c in range(3):
            stf[k, c] = seis[c][k][::-1]
    stf *= np.float32(1e10) / np.abs(stf).max()
    return loc, stf


def main():
    import oracle
    oracle.build()
    out = {}
    for prefix, seed in (("fwd_", 101), ("adj_", 102)):
        for k, v in case_inputs(seed).items():
            out[prefix + k] = v
    g = dict(out)
    p = problem_from(g, "fwd_")
    o = oracle.Oracle(p, fp64=True, adjoint_flag=0)
    o.run(NT)
    out["fwd_seismograms"] = np.stack(o.seismograms())
    out["fwd_vz_global"] = o.get("vz_global").astype(np.float32)
    p = problem_from(g, "adj_")
    o = oracle.Oracle(p, fp64=True, adjoint_flag=1)
    o.run(NT)
    recs = np.stack([o.record(r) for r in range(o.nrecords())])
    sv = o.get_int("saving_vector")[1:NT + 1]
    loc, stf = adjoint_sources(p, [s.astype(np.float32) for s in o.seismograms()])
    oa = oracle.Oracle(p, fp64=True, adjoint_flag=2, saving_vector=sv, ad_loc=loc, ad_stf=stf)
    oa.set_records(recs)
    oa.run(NT)
    out["adj_adsrc_loc"], out["adj_adsrc_stf"] = loc, stf
    for k in ("rho", "cp", "csh", "csv"):
        full = oa.get("grad_" + k)
        out["adj_grad_" + k] = full[::STRIDE].astype(np.float64)
        out["adj_norm_" + k] = np.float64(np.linalg.norm(full))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
