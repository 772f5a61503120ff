"""Command-line runner.

  python -m ses3d_gb300 run --workload c4 --events 1 --steps 10 [--epb 1] [--graph 0] [--lean 0]
      generates a seeded workload in memory and runs it on cuda:0, printing the
      per-iteration time (used for profiling captures and quick checks);
  python -m ses3d_gb300 generate --workload c1 --out DIR [--nt 1000]
      writes the workload as a reference directory tree (INPUT/, MODELS/MODELS/).
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
    g = sub.add_parser("generate")
    g.add_argument("--workload", default="c1")
    g.add_argument("--out", required=True)
    g.add_argument("--nt", type=int, default=None)
    g.add_argument("--seed", type=int, default=1234)
    a = ap.parse_args(argv)

    from . import synth
    if a.cmd == "generate":
        p = synth.make_problem(a.workload, nt=a.nt, seed=a.seed)
        synth.write_problem(p, a.out)
        print("wrote %s (%d elements, %d events)" % (a.out, p.n_elements, len(p.events)))
        return 0

    from . import build
    build.build()
    from .solver import Simulation
    p = synth.make_problem(a.workload, nt=a.steps + 2, seed=a.seed, n_events=a.events)
    sim = Simulation.from_problem(p, adjoint_flag=1 if a.adjoint else None)
    sim.set_block_elements(a.epb)
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
    sim.close()
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
