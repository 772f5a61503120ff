"""ses3d_gpu_main, the reference program flow on the GPU library: run on generated SES3D
directory trees, its output files (seismograms, snapshots, forward-field records,
saving_vector, grad_* kernels) are compared with the oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

from ses3d_gb300 import formats as F
from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "ses3d_gb300", "ses3d_gpu_main")


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_driver(root, pml):
    res = subprocess.run([DRIVER, "--main", os.path.join(root, "MAIN"), "--pml", str(pml)], capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr + res.stdout
    return res.stdout


def test_forward_tree(native, oracle_mod, tmp_path):
    p = synth.make_problem("tiny", nt=40, seed=61)
    ev = p.events[0].event
    ev.ssamp, ev.output_displacement = 20, 1
    ev.ofd = "../DATA/OUTPUT/1/"
    root = str(tmp_path)
    synth.write_problem(p, root)
    out = run_driver(root, p.pml)
    summary = json.loads(out.strip().splitlines()[-1])
    assert summary["iterations"] == 40 and summary["boxes"] == 1 and summary["gll_points"] == p.n_nodes
    ofd = os.path.join(root, "MAIN", "../DATA/OUTPUT/1/")
    o = oracle_mod.Oracle(p)
    o.run(20)
    snap20 = o.get("vz")
    o.run(20)
    ref = o.seismograms()
    kept = o.get_int("nr")[0]
    names = p.events[0].receivers.names
    for r in range(kept):
        for c, comp in enumerate("xyz"):
            nt, dt, tr = F.read_seismogram(os.path.join(ofd, names[r] + "." + comp))
            assert nt == 40 and np.float32(dt) == ev.dt
            assert rel(tr, ref[c][r]) <= 1e-5 or np.abs(ref[c][r]).max() == 0, (r, comp)
    vz20 = F.read_record(os.path.join(ofd, "vz_0_20"), p.n_nodes)
    assert rel(vz20, snap20) <= 1e-5
    vz40 = F.read_record(os.path.join(ofd, "vz_0_40"), p.n_nodes)
    assert rel(vz40, o.get("vz")) <= 1e-5


def test_adjoint_round_trip_through_files(native, oracle_mod, tmp_path):
    nt = 50
    p = synth.make_problem("tiny", nt=nt, seed=62, adjoint_flag=1)
    p.setup.samp_ad = 5
    p.setup.ffd = "../DATA/FFD"
    root = str(tmp_path)
    synth.write_problem(p, root)
    run_driver(root, p.pml)
    ffd = os.path.join(root, "MAIN", "../DATA/FFD/1/")
    sv = F.read_saving_vector(os.path.join(ffd, "saving_vector_0"), nt)
    o = oracle_mod.Oracle(p, adjoint_flag=1)
    o.run(nt)
    assert np.array_equal(sv, o.get_int("saving_vector")[1:nt + 1])
    recs = {nm: F.read_records(os.path.join(ffd, nm + "_0")) for nm in ("vx", "exx", "eyz")}
    assert len(recs["vx"]) == o.nrecords()
    for r in range(o.nrecords()):
        orec = o.record(r)
        for f, nm in ((0, "vx"), (3, "exx"), (8, "eyz")):
            if np.abs(orec[f]).max() > 0:
                assert rel(recs[nm][r], orec[f]) <= 1e-4, (r, nm)
    # adjoint run from the files: two adjoint sources at the first receivers
    seis = o.seismograms()
    loc = p.events[0].receivers.loc[:2].copy()
    loc[:, 2] = 1000.0
    adir = os.path.join(root, "ADJOINT", "1")
    os.makedirs(adir, exist_ok=True)
    F.write_ad_srcfile(os.path.join(adir, "ad_srcfile"), loc)
    stf = np.zeros((2, 3, nt), np.float32)
    for k in range(2):
        for c in range(3):
            stf[k, c] = seis[c][k][::-1]
        stf[k] *= np.float32(1e10) / np.abs(stf[k]).max()
        F.write_ad_src(os.path.join(adir, "ad_src_%d" % (k + 1)), stf[k], loc[k])
    stf = np.stack([F.read_ad_src(os.path.join(adir, "ad_src_%d" % (k + 1)), nt) for k in range(2)])
    p.setup.adjoint_flag = 2
    F.write_setup(os.path.join(root, "INPUT", "setup"), p.setup)
    run_driver(root, p.pml)
    ofd = os.path.join(root, "MAIN", p.events[0].event.ofd)
    recs_all = np.stack([o.record(r) for r in range(o.nrecords())])
    oa = oracle_mod.Oracle(p, adjoint_flag=2, saving_vector=sv, ad_loc=loc, ad_stf=stf)
    oa.set_records(recs_all)
    oa.run(nt)
    for nm in ("rho", "cp", "csh", "csv"):
        g = F.read_record(os.path.join(ofd, "grad_%s_0" % nm), p.n_nodes)
        ref = oa.get("grad_" + nm)
        assert np.abs(ref).max() > 0
        assert rel(g, ref) <= 1e-3, nm


def test_model_files_inconsistent_with_boxfile_are_rejected(native, tmp_path):
    """A boxfile of two boxes over a single-box model: rank 0's model record has the wrong
    size, which the driver reports before touching the GPU."""
    p = synth.make_problem("tiny", nt=5, seed=63)
    root = str(tmp_path)
    synth.write_problem(p, root)
    s = synth.split_setup(p.setup, (p.nx + 1, p.ny + 1, p.nz + 1), (2, 1, 1))
    F.write_boxfile(os.path.join(root, "MODELS", "MODELS", "boxfile"), F.make_boxes(s), 2, 1, 1)
    res = subprocess.run([DRIVER, "--main", os.path.join(root, "MAIN")], capture_output=True, text=True, timeout=120)
    assert res.returncode != 0 and "does not hold" in res.stderr


def test_adjoint_sources_tool_in_the_file_workflow(native, oracle_mod, tmp_path):
    """Forward job -> seismogram files -> cross-correlation adjoint sources written by
    `python -m ses3d_gb300 adjoint-sources` -> adjoint job -> grad_* files, against the
    oracle run on the same records and adjoint sources."""
    from ses3d_gb300.__main__ import main
    nt = 60
    p = synth.make_problem("tiny", nt=nt, seed=64, adjoint_flag=1)
    p.setup.samp_ad = 5
    p.setup.ffd = "../DATA/FFD"
    root = str(tmp_path)
    synth.write_problem(p, root)
    run_driver(root, p.pml)
    ev = p.events[0]
    ofd = os.path.join(root, "MAIN", ev.event.ofd)
    adir = os.path.join(root, "ADJOINT", ev.name)
    assert main(["adjoint-sources", "--seismograms", ofd, "--out", adir, "--kind", "cc", "--component", "z",
                 "--window", "0.5", "5.5", "--taper", "0.5", "--stations"] + list(ev.receivers.names)) == 0
    loc = F.read_ad_srcfile(os.path.join(adir, "ad_srcfile"))
    stf = np.stack([F.read_ad_src(os.path.join(adir, "ad_src_%d" % (k + 1)), nt) for k in range(len(loc))])
    assert np.abs(stf).max() > 0
    p.setup.adjoint_flag = 2
    F.write_setup(os.path.join(root, "INPUT", "setup"), p.setup)
    run_driver(root, p.pml)
    o = oracle_mod.Oracle(p, adjoint_flag=1)
    o.run(nt)
    recs = np.stack([o.record(r) for r in range(o.nrecords())])
    sv = o.get_int("saving_vector")[1:nt + 1]
    oa = oracle_mod.Oracle(p, adjoint_flag=2, saving_vector=sv, ad_loc=loc, ad_stf=stf)
    oa.set_records(recs)
    oa.run(nt)
    for nm in ("rho", "cp", "csh", "csv"):
        g = F.read_record(os.path.join(ofd, "grad_%s_0" % nm), p.n_nodes)
        ref = oa.get("grad_" + nm)
        assert np.abs(ref).max() > 0
        assert rel(g, ref) <= 1e-3, nm
