"""Multi-rank SES3D trees (px, py, pz > 1): processor boxes of the reference's model
generator are stitched into one mesh on input and every per-rank output file is split
back out (SOURCE/ses3d_input.f90:44-170, SOURCE/ses3d_output.f90:270-342)."""
import os
import subprocess

import numpy as np
import pytest

from ses3d_gb300 import formats as F
from ses3d_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "ses3d_gb300", "ses3d_gpu_main")


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n_el,procs", [((6, 5, 4), (2, 1, 2)), ((9, 8, 7), (3, 2, 2)), ((5, 5, 5), (1, 1, 1))])
def test_boxes_tile_and_split_stitch_round_trip(n_el, procs):
    s = synth.split_setup(synth.make_setup(n_el), n_el, procs)
    boxes = F.make_boxes(s)
    (ex, ey, ez), offs = F.box_offsets(boxes)
    assert (ex, ey, ez) == n_el
    cover = np.zeros((ez, ey, ex), int)
    for b, (ox, oy, oz) in zip(boxes, offs):
        cover[oz:oz + b.nz + 1, oy:oy + b.ny + 1, ox:ox + b.nx + 1] += 1
    assert np.all(cover == 1)
    g = np.random.default_rng(1).standard_normal(125 * ex * ey * ez).astype(np.float32)
    pieces = F.split_field(g, boxes)
    assert sum(p.size for p in pieces) == g.size
    assert np.array_equal(F.stitch_field(pieces, boxes), g)
    pad = (max(b.nx for b in boxes) + 1, max(b.ny for b in boxes), max(b.nz for b in boxes) + 2)
    padded = F.split_field(g, boxes, pad=pad)
    assert all(p.size == 125 * (pad[0] + 1) * (pad[1] + 1) * (pad[2] + 1) for p in padded)
    assert np.array_equal(F.stitch_field(padded, boxes, pad=pad), g)


def test_bottom_box_holds_the_lowest_elements():
    """Box mz = 1 is the bottom of the section: its local k = 0 element lies directly below
    the box above it, and its physical z range is the lowest."""
    n_el, procs = (4, 4, 6), (1, 1, 2)
    boxes = F.make_boxes(synth.split_setup(synth.make_setup(n_el), n_el, procs))
    (_, _, ez), offs = F.box_offsets(boxes)
    bottom = [b for b in boxes if b.multi[2] == 1][0]
    top = [b for b in boxes if b.multi[2] == 2][0]
    assert bottom.zmax <= top.zmin + 1e-3 and bottom.zmin < top.zmin
    assert offs[boxes.index(top)][2] == 0 and offs[boxes.index(bottom)][2] == top.nz + 1


def test_driver_stitches_multirank_model(native, tmp_path):
    """ses3d_gpu_main --stitch-model (no GPU): the stitched model equals the global one bit
    for bit, and its boxfile describes the union box."""
    p = synth.make_problem("tiny", nt=5, seed=71, n_el=(6, 5, 4))
    root = str(tmp_path / "tree")
    synth.write_problem(p, root, procs=(2, 1, 2))
    out = str(tmp_path / "stitched")
    res = subprocess.run([DRIVER, "--main", os.path.join(root, "MAIN"), "--stitch-model", out], capture_output=True,
                         text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    assert "6 x 5 x 4" in res.stdout
    for k, v in p.model.items():
        got = F.read_record(os.path.join(out, k + "0"), p.n_nodes)
        assert np.array_equal(got, v), k
    (b,) = F.read_boxfile(os.path.join(out, "boxfile"))
    boxes = F.read_boxfile(os.path.join(root, "MODELS", "MODELS", "boxfile"))
    assert (b.nx, b.ny, b.nz) == (5, 4, 3)
    assert b.xmin == min(x.xmin for x in boxes) and b.zmax == max(x.zmax for x in boxes)


def run_driver(root, pml, *extra):
    res = subprocess.run([DRIVER, "--main", os.path.join(root, "MAIN"), "--pml", str(pml)] + list(extra),
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr + res.stdout
    return res.stdout


@pytest.mark.gpu
def test_multirank_forward_matches_single_box(native, tmp_path):
    """A 2 x 1 x 2 decomposed tree gives the single-box seismograms and, split per rank and
    padded to the largest box, its snapshots."""
    p = synth.make_problem("small", nt=60, seed=72, n_el=(10, 9, 8))
    ev = p.events[0].event
    ev.ssamp, ev.output_displacement = 30, 1
    one, many = str(tmp_path / "one"), str(tmp_path / "many")
    synth.write_problem(p, one)
    synth.write_problem(p, many, procs=(2, 1, 2))
    run_driver(one, p.pml)
    run_driver(many, p.pml)
    o1, o2 = (os.path.join(r, "MAIN", ev.ofd) for r in (one, many))
    names = p.events[0].receivers.names
    for nm in names:
        for c in "xyz":
            a, b = F.read_seismogram(os.path.join(o1, nm + "." + c))[2], F.read_seismogram(os.path.join(o2, nm + "." + c))[2]
            assert rel(b, a) <= 1e-5 or np.abs(a).max() == 0, (nm, c)
    boxes = F.read_boxfile(os.path.join(many, "MODELS", "MODELS", "boxfile"))
    pad = (max(b.nx for b in boxes), max(b.ny for b in boxes), max(b.nz for b in boxes))
    ref = F.read_record(os.path.join(o1, "vz_0_60"), p.n_nodes)
    size = 125 * (pad[0] + 1) * (pad[1] + 1) * (pad[2] + 1)
    pieces = [F.read_record(os.path.join(o2, "vz_%d_60" % r), size) for r in range(len(boxes))]
    assert rel(F.stitch_field(pieces, boxes, pad=pad), ref) <= 1e-5


@pytest.mark.gpu
def test_multirank_adjoint_through_padded_files(native, tmp_path):
    """Forward job with per-rank forward-field files padded to --max-elements, adjoint job
    reading them back: per-rank grad_* files equal the single-box kernels split per rank."""
    nt = 50
    p = synth.make_problem("tiny", nt=nt, seed=73, adjoint_flag=1, n_el=(6, 6, 4))
    p.setup.samp_ad = 5
    p.setup.ffd = "../DATA/FFD"
    trees = {"one": ((1, 1, 1), ()), "many": ((2, 2, 1), ("--max-elements", "3", "3", "4"))}
    grads = {}
    for tag, (procs, extra) in trees.items():
        root = str(tmp_path / tag)
        synth.write_problem(p, root, procs=procs)
        run_driver(root, p.pml, *extra)
        seis = F.read_seismogram(os.path.join(root, "MAIN", p.events[0].event.ofd,
                                              p.events[0].receivers.names[0] + ".z"))[2]
        loc = p.events[0].receivers.loc[:1].copy()
        loc[:, 2] = 1000.0
        adir = os.path.join(root, "ADJOINT", "1")
        os.makedirs(adir, exist_ok=True)
        F.write_ad_srcfile(os.path.join(adir, "ad_srcfile"), loc)
        stf = np.zeros((3, nt), np.float32)
        stf[2] = np.float32(1e10) * seis[::-1] / max(np.abs(seis).max(), 1e-30)
        F.write_ad_src(os.path.join(adir, "ad_src_1"), stf, loc[0])
        s = F.read_setup(os.path.join(root, "INPUT", "setup"))
        s.adjoint_flag = 2
        F.write_setup(os.path.join(root, "INPUT", "setup"), s)
        run_driver(root, p.pml, *extra)
        ofd = os.path.join(root, "MAIN", p.events[0].event.ofd)
        boxes = F.read_boxfile(os.path.join(root, "MODELS", "MODELS", "boxfile"))
        pad = (3, 3, 4) if extra else (boxes[0].nx, boxes[0].ny, boxes[0].nz)
        size = 125 * (pad[0] + 1) * (pad[1] + 1) * (pad[2] + 1)
        ffd = os.path.join(root, "MAIN", "../DATA/FFD/1/")
        assert all(len(F.read_records(os.path.join(ffd, "vx_%d" % r))[0]) == size for r in range(len(boxes)))
        grads[tag] = {nm: F.stitch_field([F.read_record(os.path.join(ofd, "grad_%s_%d" % (nm, r)), size)
                                          for r in range(len(boxes))], boxes, pad=pad)
                      for nm in ("rho", "cp", "csh", "csv")}
    for nm in ("rho", "cp", "csh", "csv"):
        assert np.abs(grads["one"][nm]).max() > 0
        assert rel(grads["many"][nm], grads["one"][nm]) <= 1e-4, nm
