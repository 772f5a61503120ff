"""Benchmark of the GB300 SES3D time step: GLL point-steps/s on the plain 3-D forward
workload (96 x 96 x 40 elements, lpd 4: 46.08M GLL points; anelastic, PML 3, one
moment-tensor source, 200 receivers), synthetic seeded inputs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0. `value` is device-timed (CUDA events on the library's
stream) whole-job throughput with the model resident in HBM; `e2e` is the same
metric through the public API (Simulation: create, model upload from pinned host
memory, K steps, seismogram download), host clock around all of it. The field
state (36 floats x 46.08M points = 6.6 GB) exceeds the 129 MB L2 many times over,
so no L2 flush is needed between steps. With --gpus N > 1 (torchrun) every rank
runs an independent replica of the workload on its own GPU (the solver shards by
event, not by domain: replicas only); value = all ranks' points x steps / max time.
--impl reference times the CPU restatement of the reference solver (the oracle,
FP32, OpenMP on all host cores) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GLL point-steps/s"
# Algorithmic bytes per local GLL node and iteration (forward, anelastic, 3 SLS, FP32):
# element-local state 36 floats read+write (288 B) + 6 material floats (24 B) + per unique
# node v read+write and 1/M read (28 B x unique/local ratio).
STATE_B, MAT_B, UNIQ_B = 288.0, 24.0, 28.0
# k_element alone: state + material + v gather (12 B x ratio).
ELEM_UNIQ_B = 12.0
# An isotropic model (A = B = C = 0, the library reports it) needs three of the six
# material floats: the element kernels read 12 B per point of material then.
MAT_ISO_B = 12.0


def load_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(workload):
    """dram bytes per k_element launch from the committed ncu summary (null if absent)."""
    path = os.path.join(ROOT, "profiles", "k_element_%s_traffic.json" % workload)
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        load = [s for s, p in zip(sm, pw) if p > 0.25 * max(pw)] if pw else sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(load or sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "samples": len(rows), "reasons": reasons}


def dist_init(n_gpus):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(problem, steps):
    """The oracle (CPU restatement of the reference, FP32, all host cores) on `steps`
    iterations of the same workload; set-up excluded."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    o = oracle.Oracle(problem)
    o.run(1)  # first iteration touches every page: untimed warm-up
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": problem.n_nodes * steps / dt, "unit": METRIC, "cores": int(os.environ["OMP_NUM_THREADS"]),
            "kind": "port", "sample": "%d time steps of the %s workload (%d GLL points), after one untimed "
                                      "step; set-up excluded" % (steps, problem.label, problem.n_nodes)}


def workload_config(p):
    """The workload description both arms print as `config` (identical for the same
    --workload and --seed): sizes and inputs only, nothing measured."""
    ex, ey, ez = p.nx + 1, p.ny + 1, p.nz + 1
    N = p.n_nodes
    G = (4 * ex + 1) * (4 * ey + 1) * (4 * ez + 1)
    state_gb = 36 * 4 * N / 1e9
    return {"workload": "%s: plain 3-D forward, %dx%dx%d elements, lpd 4, %d GLL points, anelastic (3 SLS), "
                        "PML %d, 1 moment-tensor source, %d receivers" %
                        (p.label, ex, ey, ez, N, p.pml, len(p.events[0].receivers.names)),
            "gll_points": N, "unique_nodes": G,
            "l2": "inputs larger than L2 (%.1f GB field state), no flush" % state_gb}


def run_ours(args, rank, world, local):
    import numpy as np
    import torch
    from ses3d_gb300 import build as B
    from ses3d_gb300 import synth
    from ses3d_gb300.solver import Simulation

    if rank == 0 or not os.path.exists(B.LIB):
        B.build()
    barrier(world)
    from ses3d_gb300.solver import select_device
    select_device(local if world > 1 else 0)   # the library's runtime follows torch's device
    nt = args.warmup + args.steps + 32  # the block-shape autotuner spends up to 27 warm-up steps
    p = synth.make_problem(args.workload, nt=nt, seed=args.seed)
    N = p.n_nodes
    ex, ey, ez = p.nx + 1, p.ny + 1, p.nz + 1
    G = (4 * ex + 1) * (4 * ey + 1) * (4 * ez + 1)
    r_u = G / N
    # lean stepping: displacement gradients and mirror stresses only in PML elements
    # (outputs unchanged)
    E = ex * ey * ez
    pml = p.pml
    n_pml_el = E - max(0, ex - 2 * pml) * max(0, ey - 2 * pml) * max(0, ez - pml)
    interior_frac = 0.0 if not args.lean else (E - n_pml_el) / E
    DU_B = 96.0  # 9 displacement gradients + 3 mirror stresses, read + written
    sim = Simulation.from_problem(p)
    sim.set_lean(args.lean)
    iso = bool(sim.setup_int("isotropic")[0])
    mat_b = MAT_ISO_B if iso else MAT_B
    tuned = None
    args.autotuned = not args.epb
    if args.epb:
        sim.set_block_elements(args.epb)
    else:  # the library's block-shape autotuner, on warm-up steps
        tuned = sim.autotune(steps_each=2)
        args.epb = tuned["chosen"]["elements_per_cta"]
    shape = sim.shape
    if args.graph:
        sim.use_graph(True, args.graph)
    # warm-up (the autotune steps above count towards it)
    remaining_warm = max(0, args.warmup - sim.it)
    sim.step(remaining_warm)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = sim.launch_count
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        sim.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    launches = sim.launch_count - launches0
    clocks = clk.summary()
    ms_max = max_over_ranks(ms, world)
    value = world * N * args.steps / (ms_max / 1e3)
    steps_done = sim.it
    seis = sim.seismograms(0)
    finite = bool(np.all(np.isfinite(seis[0]))) and bool(np.all(np.isfinite(sim.vmax())))
    sim.close()

    # dominant kernel, timed live with CUDA events on the library's stream (eager launches)
    prof = Simulation.from_problem(p)
    prof.set_lean(args.lean)
    prof.set_block_elements(args.epb)
    prof.set_kernel_shape(shape["element_shape"], shape["node_block"])
    prof.step(2)
    prof.profile(True)
    prof.step(args.prof_steps)
    el_ms, el_n = prof.kernel_time("element")
    nd_ms, nd_n = prof.kernel_time("node")
    rc_ms, rc_n = prof.kernel_time("receivers")
    prof.close()
    el_avg = el_ms / max(el_n, 1)
    elem_bytes = N * (STATE_B + mat_b + ELEM_UNIQ_B * r_u - DU_B * interior_frac)
    peak, peak_kind = load_peak()
    achieved = elem_bytes / (el_avg / 1e3) / 1e9
    tr = load_traffic(args.workload)
    step_bytes = N * (STATE_B + mat_b + UNIQ_B * r_u - DU_B * interior_frac)
    step_gbs = step_bytes / (ms / args.steps / 1e3) / 1e9

    # end to end through the public API with host buffers (pinned)
    e2e = None
    if not args.no_e2e:
        pinned = {}
        for k, v in p.model.items():
            t = torch.empty(v.size, dtype=torch.float32, pin_memory=True)
            t.numpy()[:] = v
            pinned[k] = t.numpy()
        ev = p.events[0]
        # three independent runs (handle creation to seismograms each); the median is reported
        # (host work and the host-to-device link are shared with other jobs on the machine)
        secs = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cfg_sim = Simulation.from_problem(p, nt=args.steps, model=False)
            cfg_sim.set_lean(args.lean)
            cfg_sim.set_block_elements(args.epb)
            cfg_sim.set_kernel_shape(shape["element_shape"], shape["node_block"])
            cfg_sim.set_model(pinned)
            if args.graph:
                cfg_sim.use_graph(True, args.graph)
            cfg_sim.step(args.steps)
            out = cfg_sim.seismograms(0)
            t1 = time.perf_counter()
            cfg_sim.close()
            secs.append(max_over_ranks(t1 - t0, world))
        t_e2e = sorted(secs)[1]
        h2d = sum(a.nbytes for a in pinned.values()) + 4 * args.steps + ev.receivers.loc.nbytes + 24
        d2h = sum(o.nbytes for o in out)
        e2e = {"value": world * N * args.steps / t_e2e, "unit": METRIC,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "seconds": t_e2e, "seconds_each_run": secs, "statistic": "median of 3 runs",
               "includes": "create + model upload + %d steps + seismogram download" % args.steps}
        del pinned

    res = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(p),
        "run_details": {"elements_per_cta": args.epb, "kernel_shape": shape, "autotune": tuned,
                        "graph_steps": args.graph,
                        "lean": bool(args.lean), "non_pml_element_fraction": (E - n_pml_el) / E,
                        "step_algorithmic_bytes_per_point": step_bytes / N,
                        "step_algorithmic_bytes_per_point_full_state": STATE_B + mat_b + UNIQ_B * r_u,
                        "isotropic_model": iso, "material_bytes_per_point": mat_b,
                        "step_achieved_gbs": step_gbs, "step_frac_of_peak": step_gbs / peak,
                        "finite": finite, "steps_completed": steps_done,
                        "kernel_ms": {"k_element": el_avg, "k_node": nd_ms / max(nd_n, 1),
                                      "k_receivers": rc_ms / max(rc_n, 1)}},
        "roofline": {"bound": "hbm", "kernel": "k_element", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes_per_launch": elem_bytes,
                     "traffic": tr.get("dram_bytes_per_launch_full")
                     if tr and bool(tr.get("lean")) == bool(args.lean) else None},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if e2e:
        res["e2e"] = e2e
    if args.lean:
        res["full_state"] = run_full_state(args, p, world, peak, STATE_B + mat_b + UNIQ_B * r_u)
    if not args.no_batched:
        res["batched"] = run_batched(args, world)
        res["forward_c1"] = run_forward_small(args, world)
    if rank == 0 and world == 1 and not args.no_grad:
        res["gradient"] = run_gradient(args)
    if rank == 0 and world == 1 and not args.no_cpu:
        res["cpu_baseline"] = cpu_baseline(p, args.cpu_steps)
    return res


def run_full_state(args, p, world, peak, bytes_per_point):
    """The same workload without lean stepping (every displacement gradient and mirror
    stress read and written, as the reference does), timed the same way."""
    import torch
    from ses3d_gb300.solver import Simulation
    sim = Simulation.from_problem(p)
    tuned = sim.autotune(steps_each=2) if args.autotuned else None
    if not args.autotuned:
        sim.set_block_elements(args.epb)
    warm = 3
    steps = max(1, min(args.steps, 100, p.events[0].event.nt - sim.it - warm))
    if args.graph:
        sim.use_graph(True, args.graph)
    sim.step(warm)
    stream = torch.cuda.ExternalStream(sim.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    e1.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), world) / steps
    sim.close()
    gbs = p.n_nodes * bytes_per_point / (ms / 1e3) / 1e9
    return {"steps": steps, "ms_per_step": ms, "value": world * p.n_nodes / (ms / 1e3), "unit": METRIC,
            "step_algorithmic_bytes_per_point": bytes_per_point, "step_achieved_gbs": gbs,
            "step_frac_of_peak": gbs / peak, "kernel_shape": sim_shape(tuned)}


def sim_shape(tuned):
    return tuned["chosen"] if tuned else None


def run_forward_small(args, world):
    """The small plain-forward workload (22 x 22 x 10 elements, 605,000 GLL points), lean,
    CUDA graph of 10 iterations, with its own autotuned block shapes."""
    import torch
    from ses3d_gb300 import synth
    from ses3d_gb300.solver import Simulation
    steps = 100
    p = synth.make_problem("c1", nt=steps + 40, seed=args.seed)
    sim = Simulation.from_problem(p)
    sim.set_lean(True)
    tuned = sim.autotune(steps_each=2)
    sim.use_graph(True, 10)
    sim.step(5)
    stream = torch.cuda.ExternalStream(sim.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    sim.close()
    return {"workload": "c1: 22x22x10 elements, %d GLL points, lean, CUDA graph of 10 iterations" % p.n_nodes,
            "steps": steps, "ms_per_step": ms, "value": world * p.n_nodes / (ms / 1e3), "unit": METRIC,
            "kernel_shape": tuned["chosen"], "autotune": tuned}


def run_batched(args, world):
    """16 events on one 48x48x24 mesh (uneven receiver counts), one launch sequence per
    time step for all events, replayed from a CUDA graph; against the same mesh with one event."""
    import torch
    from ses3d_gb300 import synth
    from ses3d_gb300.solver import Simulation
    steps = args.batched_steps
    out, shapes = {}, {}
    for nev in (1, 16):
        p = synth.make_problem("c4", nt=steps + 45, seed=args.seed, n_events=nev)
        sim = Simulation.from_problem(p)
        sim.set_lean(args.lean)
        shapes[nev] = sim.autotune(steps_each=2)["chosen"]
        sim.use_graph(True, 10)
        sim.step(10)
        stream = torch.cuda.ExternalStream(sim.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        sim.step(steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[nev] = (ms, p.n_nodes, [len(e.receivers.names) for e in p.events])
        sim.close()
    ms1, n, _ = out[1]
    ms16, _, nrec = out[16]
    return {"workload": "c4: 48x48x24 elements, %d GLL points per event, 16 events, receivers per event %d-%d, "
                        "CUDA graph of 10 iterations" % (n, min(nrec), max(nrec)),
            "events": 16, "ms_per_step": ms16, "value": world * 16 * n / (ms16 / 1e3), "unit": METRIC,
            "single_event_ms_per_step": ms1, "per_event_speedup_vs_single": 16 * ms1 / ms16,
            "kernel_shape_16_events": shapes[16], "kernel_shape_single_event": shapes[1]}


def gradient_once(workload, nt, nev, seed, truth_kind, memory_budget=None, exact=False):
    """One misfit gradient through the public autograd API (waveform_misfit forward +
    backward: forward run with records or checkpoints, misfit, adjoint sources, adjoint run,
    kernel readout), timed end to end. Observed data come from a perturbed model (untimed).
    memory_budget: device bytes the gradient may use (None: the free device memory).
    exact: the exact discrete adjoint of the time stepping instead of the reference's kernels."""
    import numpy as np
    import torch
    from ses3d_gb300 import adjoint as A
    from ses3d_gb300 import synth
    p = synth.make_problem(workload, nt=nt, seed=seed, n_events=nev, adjoint_flag=1)
    setup = A.MisfitSetup.from_problem(p, samp_ad=10, memory_budget=memory_budget, exact=exact)
    m0 = A.problem_tensors(p)
    if truth_kind == "blob":    # +-5 % vs Gaussian blob, radius 150 km at 200 km depth
        truth = synth.build_model(p.box, blob=(0.05, 150e3, 200e3), is_diss=1)
    else:                       # +-4 % vs checkerboard, 200 km cells
        truth = synth.build_model(p.box, checker=(0.04, 200e3), is_diss=1)
    setup.set_observed(A.problem_tensors(synth.Problem(p.setup, p.box, p.tau, p.D, truth, p.events, pml=p.pml)))
    ms = [t.clone().requires_grad_(True) for t in m0]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    chi = A.waveform_misfit(setup, *ms)
    chi.backward()
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    finite = bool(all(torch.isfinite(t.grad).all() for t in ms)) and bool(np.isfinite(float(chi.detach())))
    nrec = [len(e.receivers.names) for e in p.events]
    plan = setup.last.get("plan")
    info = {"events": nev, "nt": nt, "samp_ad": 10, "gll_points_per_event": p.n_nodes,
            "backward": "exact discrete adjoint" if exact else "reference kernels (ses3d_grad_Q)",
            "receivers_per_event": [min(nrec), max(nrec)],
            "events_per_sub_batch": plan.events_per_batch if plan else nev,
            "records_per_checkpoint_segment": setup.last.get("records_per_segment", 0),
            "records_per_checkpoint_subsegment": setup.last.get("records_per_subsegment", 0),
            "memory_budget_bytes": memory_budget, "modeled_bytes_per_sub_batch": modeled_bytes(setup, plan),
            "steps_per_checkpoint": setup.last.get("steps_per_checkpoint") if exact else None,
            "steps_per_subsegment": setup.last.get("steps_per_subsegment") if exact else None,
            "seconds": sec, "s_per_event_gradient": sec / nev, "finite": finite}
    del setup, ms, chi
    torch.cuda.empty_cache()
    return info


def modeled_bytes(setup, plan):
    """Device bytes one sub-batch of the plan needs by the setup's memory model."""
    if plan is None or setup.exact:
        return None
    m = setup.memory_model()
    per = m["two_level"] if plan.K2 else (m["one_level"] if plan.K else m["keep"])
    return m["shared"] + plan.events_per_batch * per


def gradient_files_once(workload, nt, seed):
    """One single-event gradient in the reference's own workflow, on this library: the
    ses3d_gpu_main forward job (adjoint_flag 1) writes seismograms, forward-field records
    and the saving vector to disk; the L2 adjoint sources are computed from the seismogram
    files and written to ADJOINT/; the adjoint job (adjoint_flag 2) reads the records back
    and writes the grad_* files, which are read. Same misfit, mesh and observed data as
    gradient_once. The directory tree is written before the clock starts."""
    import shutil
    import numpy as np
    from ses3d_gb300 import adjoint as A
    from ses3d_gb300 import formats as F
    from ses3d_gb300 import synth
    p = synth.make_problem(workload, nt=nt, seed=seed, n_events=1, adjoint_flag=1)
    p.setup.samp_ad = 10
    setup = A.MisfitSetup.from_problem(p, samp_ad=10)
    truth = synth.build_model(p.box, checker=(0.04, 200e3), is_diss=1)
    setup.set_observed(A.problem_tensors(synth.Problem(p.setup, p.box, p.tau, p.D, truth, p.events, pml=p.pml)))
    root = tempfile.mkdtemp(prefix="ses3d_grad_")
    try:
        synth.write_problem(p, root)
        main = os.path.join(root, "MAIN")
        driver = os.path.join(ROOT, "ses3d_gb300", "ses3d_gpu_main")
        ev = p.events[0]
        t0 = time.perf_counter()
        subprocess.run([driver, "--main", main, "--pml", str(p.pml)], check=True, capture_output=True)
        ofd = os.path.join(main, ev.event.ofd)
        syn = np.stack([np.stack([F.read_seismogram(os.path.join(ofd, nm + "." + c))[2] for nm in ev.receivers.names])
                        for c in "xyz"]).astype(np.float64)                     # (3, nr, nt)
        srcs = setup.adjoint_sources([syn], float(ev.event.dt))[0]              # (nr, 3, nt)
        adir = os.path.join(root, "ADJOINT", ev.name)
        os.makedirs(adir, exist_ok=True)
        loc = np.asarray(ev.receivers.loc, np.float32)
        F.write_ad_srcfile(os.path.join(adir, "ad_srcfile"), loc)
        for k in range(len(loc)):
            F.write_ad_src(os.path.join(adir, "ad_src_%d" % (k + 1)), srcs[k], loc[k])
        p.setup.adjoint_flag = 2
        F.write_setup(os.path.join(root, "INPUT", "setup"), p.setup)
        subprocess.run([driver, "--main", main, "--pml", str(p.pml)], check=True, capture_output=True)
        grads = [F.read_record(os.path.join(ofd, "grad_%s_0" % nm), p.n_nodes) for nm in ("rho", "cp", "csh", "csv")]
        sec = time.perf_counter() - t0
        finite = all(bool(np.all(np.isfinite(g))) for g in grads)
        ffd_bytes = sum(os.path.getsize(os.path.join(dp, f)) for dp, _, fs in os.walk(os.path.join(main, p.setup.ffd))
                        for f in fs)
    finally:
        shutil.rmtree(root, ignore_errors=True)
    return {"events": 1, "nt": nt, "samp_ad": 10, "gll_points_per_event": p.n_nodes,
            "forward_record_bytes_on_disk": ffd_bytes, "disk": tempfile.gettempdir(),
            "seconds": sec, "s_per_event_gradient": sec, "finite": finite}


def run_gradient(args):
    """'s per event gradient': the 64x64x32 single-event gradient of the misfit workload at
    its full length; 16 events batched in one handle against single-event gradients on the
    48x48x24 mesh (nt 3000) and the 22x22x10 mesh (nt 1000); two events of the 96x96x40
    16-event gradient at nt 4000 under a 150 GB device-memory budget (two checkpoint
    levels, one event per sub-batch); and the reference's file workflow on 48x48x24 against
    the same gradient kept in HBM."""
    out = {"api": "ses3d_gb300.adjoint.waveform_misfit forward + backward (torch.autograd)",
           "dtype": "f32 fields, f64 kernel and misfit accumulation"}
    out["single_64x64x32"] = gradient_once("c3", args.grad_nt, 1, args.seed, "blob")
    if not args.no_exact:
        out["exact_64x64x32"] = gradient_once("c3", args.grad_nt, 1, args.seed, "blob", exact=True)
    for wl, tag, nt in (("c4", "48x48x24", args.grad_c4_nt), ("c1", "22x22x10", args.grad_c1_nt)):
        one = gradient_once(wl, nt, 1, args.seed, "checker")
        many = gradient_once(wl, nt, 16, args.seed, "checker")
        out["single_" + tag] = one
        out["batched_" + tag] = many
        out["batched_per_event_speedup_vs_single_" + tag] = one["s_per_event_gradient"] / many["s_per_event_gradient"]
    if args.grad_c5_events > 0:
        out["c5_96x96x40"] = gradient_once("c5", args.grad_c5_nt, args.grad_c5_events, args.seed, "checker",
                                           memory_budget=150e9)
    files = gradient_files_once("c4", args.grad_files_nt, args.seed)
    hbm = gradient_once("c4", args.grad_files_nt, 1, args.seed, "checker")
    out["single_files_48x48x24"] = files
    out["single_hbm_48x48x24_same_nt"] = hbm
    out["hbm_speedup_vs_files_48x48x24"] = files["s_per_event_gradient"] / hbm["s_per_event_gradient"]
    return out


def run_reference(args, rank, world):
    """The reference arm: the oracle (the reference solver restated on the CPU, FP32,
    OpenMP on every host core) stepping the same workload as the GPU arm, --warmup untimed
    steps and then --steps timed ones. Under torchrun only rank 0 runs it."""
    from ses3d_gb300 import synth
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    steps, warm = args.steps, args.warmup
    p = synth.make_problem(args.workload, nt=steps + warm + 1, seed=args.seed)
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    o = oracle.Oracle(p)
    o.run(warm)
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    o.close()
    v = p.n_nodes * steps / dt
    sample = ("%d time steps (after %d untimed) of the %s workload, %d GLL points, CPU restatement of the "
              "reference (FP32, OpenMP)" % (steps, warm, args.workload, p.n_nodes))
    return {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world, "steps": steps, "warmup": warm,
            "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": workload_config(p),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--epb", type=int, default=0, help="elements per CTA (0: autotune)")
    ap.add_argument("--graph", type=int, default=10, help="steps per CUDA graph (0: eager)")
    ap.add_argument("--prof-steps", type=int, default=10)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--lean", type=int, default=1, help="1: displacement gradients only in PML elements")
    ap.add_argument("--batched-steps", type=int, default=40)
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--grad-nt", type=int, default=4000, help="time steps of the 64x64x32 gradient")
    ap.add_argument("--no-exact", action="store_true", help="skip the exact-adjoint gradient")
    ap.add_argument("--grad-c4-nt", type=int, default=3000, help="time steps of the 48x48x24 gradients")
    ap.add_argument("--grad-c1-nt", type=int, default=1000, help="time steps of the 22x22x10 gradients")
    ap.add_argument("--grad-c5-nt", type=int, default=4000, help="time steps of the 96x96x40 gradient")
    ap.add_argument("--grad-c5-events", type=int, default=2, help="events of the 96x96x40 gradient timed (0: skip)")
    ap.add_argument("--grad-files-nt", type=int, default=200, help="time steps of the file-workflow gradient")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
        res = run_reference(args, rank, world)
    else:
        rank, world, local = dist_init(args.gpus)
        res = run_ours(args, rank, world, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
