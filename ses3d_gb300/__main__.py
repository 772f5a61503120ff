"""Command-line runner.

  python -m ses3d_gb300 run --workload c4 --events 1 --steps 10 [--epb 1] [--graph 0] [--lean 0]
          [--adjoint | --exact K [--exact-k2 K2]]
      generates a seeded workload in memory and runs it on cuda:0, printing the
      per-iteration time (used for profiling captures and quick checks); --adjoint adds the
      reference's adjoint run with kernel correlation, --exact the exact discrete adjoint
      (checkpoints every K iterations, a second level every K2) driven by the seismograms;
  python -m ses3d_gb300 generate --workload c1 --out DIR [--nt 1000]
      writes the workload as a reference directory tree (INPUT/, MODELS/MODELS/);
  python -m ses3d_gb300 adjoint-sources --seismograms OFD --out ADJOINT/1 --kind cc
          --component z --window 10 50 [--taper 5 | --freq 0.05] [--stations A B ...]
          [--bandpass FMIN FMAX] [--integrate] [--depth METRES]
      writes ad_srcfile and ad_src_<k> for the listed (default: all) stations from SES3D
      seismogram files, one measurement per station (TOOLS/adjoint_source.py);
  python -m ses3d_gb300 generate-models --root DIR [--profile TABLE] [--perturb [BLOCKDIR]]
      writes MODELS/MODELS (boxfile, per-rank records) and DATA/COORDINATES for the tree's
      INPUT/setup (generate_models.f90), optionally adding the block-model perturbations of
      MODELS/MODELS_3D (add_perturbation.f90). TABLE: one layer per line, top depth [km],
      rho [g/cm^3], vp, vs [km/s][, Q]; without it the setup's model_type (1 homogeneous,
      2 isotropic PREM, 3 homogeneous + QL6 Q, 4 EUMOD background, 7 ak135).
"""
import argparse
import json
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m ses3d_gb300")
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run")
    r.add_argument("--workload", default="c1")
    r.add_argument("--events", type=int, default=None)
    r.add_argument("--steps", type=int, default=10)
    r.add_argument("--epb", type=int, default=1)
    r.add_argument("--graph", type=int, default=0)
    r.add_argument("--lean", type=int, default=0, help="1: lean plain-forward stepping")
    r.add_argument("--seed", type=int, default=1234)
    r.add_argument("--adjoint", action="store_true", help="forward with records, then adjoint with kernels")
    r.add_argument("--exact", type=int, default=0, help="forward with exact-adjoint checkpoints every EXACT "
                   "iterations, then the exact backward run")
    r.add_argument("--exact-k2", type=int, default=0, help="second checkpoint level of --exact")
    g = sub.add_parser("generate")
    g.add_argument("--workload", default="c1")
    g.add_argument("--out", required=True)
    g.add_argument("--nt", type=int, default=None)
    g.add_argument("--seed", type=int, default=1234)
    q = sub.add_parser("adjoint-sources")
    q.add_argument("--seismograms", required=True, help="directory holding <station>.{x,y,z}")
    q.add_argument("--out", required=True)
    q.add_argument("--kind", default="cc", choices=["cc", "L2amp", "mttime", "mtamp"])
    q.add_argument("--component", default="z", choices=["x", "y", "z"])
    q.add_argument("--window", type=float, nargs=2, required=True, metavar=("LEFT", "RIGHT"))
    q.add_argument("--taper", type=float, default=None, help="cosine taper width [s] (cc, L2amp)")
    q.add_argument("--freq", type=float, default=None, help="frequency [Hz] (mttime, mtamp)")
    q.add_argument("--stations", nargs="*", default=None)
    q.add_argument("--bandpass", type=float, nargs=2, default=None, metavar=("FMIN", "FMAX"))
    q.add_argument("--integrate", action="store_true", help="integrate velocity to displacement first")
    q.add_argument("--depth", type=float, default=None, help="adjoint source depth [m] (default: receiver's)")
    gm = sub.add_parser("generate-models")
    gm.add_argument("--root", required=True, help="SES3D tree holding INPUT/setup")
    gm.add_argument("--profile", default=None, help="layered 1-D profile table")
    gm.add_argument("--perturb", nargs="?", const="", default=None, help="add block perturbations")
    gm.add_argument("--no-coordinates", action="store_true")
    a = ap.parse_args(argv)

    if a.cmd == "adjoint-sources":
        return adjoint_sources_cmd(a)
    if a.cmd == "generate-models":
        return generate_models_cmd(a)

    from . import synth
    if a.cmd == "generate":
        p = synth.make_problem(a.workload, nt=a.nt, seed=a.seed)
        synth.write_problem(p, a.out)
        print("wrote %s (%d elements, %d events)" % (a.out, p.n_elements, len(p.events)))
        return 0

    from . import build
    build.build()
    from .solver import Simulation
    p = synth.make_problem(a.workload, nt=a.steps + (1 if a.exact else 2), seed=a.seed, n_events=a.events)
    sim = Simulation.from_problem(p, adjoint_flag=1 if a.adjoint else None)
    sim.set_block_elements(a.epb)
    if a.exact:
        sim.exact_adjoint(a.exact, a.exact_k2)
    if a.lean:
        sim.set_lean(True)
    if a.graph:
        sim.use_graph(True, a.graph)
    sim.step(1)
    t0 = time.perf_counter()
    sim.step(a.steps)
    t1 = time.perf_counter()
    out = {"workload": a.workload, "events": sim.n_events, "gll_points": p.n_nodes, "steps": a.steps,
           "ms_per_step": (t1 - t0) * 1e3 / a.steps, "launches": sim.launch_count,
           "vmax": [float(v) for v in sim.vmax()]}
    if a.adjoint:
        sim.begin_adjoint()
        t2 = time.perf_counter()
        sim.step(a.steps + 1)
        out["adjoint_ms_per_step"] = (time.perf_counter() - t2) * 1e3 / (a.steps + 1)
    if a.exact:
        for ev in range(sim.n_events):
            sim.set_seismogram_adjoint(ev, *sim.seismograms(ev))
        t2 = time.perf_counter()
        sim.exact_backward()
        out["exact_backward_ms_per_step"] = (time.perf_counter() - t2) * 1e3 / (a.steps + 1)
        out["launches"] = sim.launch_count
    sim.close()
    print(json.dumps(out))
    return 0


def adjoint_sources_cmd(a):
    import os
    from . import adjoint_sources as AS
    if a.kind in ("cc", "L2amp") and a.taper is None:
        raise SystemExit("--taper is required for %s" % a.kind)
    if a.kind in ("mttime", "mtamp") and a.freq is None:
        raise SystemExit("--freq is required for %s" % a.kind)
    names = a.stations
    if not names:
        names = sorted(f[:-2] for f in os.listdir(a.seismograms) if f.endswith(".x"))
    sources = []
    for nm in names:
        s = AS.Seismogram().read(a.seismograms, nm, integrate=a.integrate)
        if a.bandpass:
            s.bandpass(*a.bandpass)
        src = AS.AdjointSource()
        src.fetch_seismogram(s)
        arg = a.taper if a.kind in ("cc", "L2amp") else a.freq
        getattr(src, "make_adsrc_" + a.kind)(a.component, a.window[0], a.window[1], arg)
        sources.append(src)
    AS.write_adjoint_directory(a.out, sources, depth=a.depth)
    print(json.dumps({"adjoint_sources": len(sources), "kind": a.kind, "out": a.out}))
    return 0


def generate_models_cmd(a):
    import os
    from . import formats as F
    from . import models as M
    setup = F.read_setup(os.path.join(a.root, "INPUT", "setup"))
    prof = M.LayeredProfile.read(a.profile) if a.profile else None
    boxes = M.generate_models(setup, a.root, prof, coordinates=not a.no_coordinates)
    if a.perturb is not None:
        M.add_perturbation_tree(a.root, a.perturb or None)
    print(json.dumps({"boxes": len(boxes), "root": a.root, "perturbed": a.perturb is not None}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
