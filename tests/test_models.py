"""Model generation (MODELS/SOURCE/generate_models.f90, add_perturbation.f90, block format
of TOOLS/models.py): coordinates, 1-D backgrounds, block files, and the perturbation
against the oracle's literal transcription (bit-exact, FP32)."""
import os

import numpy as np
import pytest

from ses3d_gb300 import formats as F
from ses3d_gb300 import models as M
from ses3d_gb300 import synth

# block-model fixtures of the reference project (MODELS/MODELS_3D), read when
# SES3D_REFERENCE_ROOT names the reference tree
REF_BLOCKS = os.path.join(os.environ.get("SES3D_REFERENCE_ROOT", "/nonexistent"), "MODELS", "MODELS_3D")


def test_box_axes_match_solver_geometry():
    p = synth.make_problem("tiny", nt=5, seed=1, model=False)
    x, y, z = M.box_axes(p.box)
    sx, sy, sz = synth.node_axes(p.box)
    assert np.array_equal(x, sx) and np.array_equal(y, sy) and np.array_equal(z, sz)


def test_layered_profile_conversion():
    p = synth.make_problem("tiny", nt=5, seed=1, model=False)
    prof = M.LayeredProfile([0.0, 35.0], [2.9, 3.4], [6.8, 8.1], [3.9, 4.5], [300.0, 150.0])
    m = M.profile_model(p.box, prof, 1)
    x, y, z = M.box_axes(p.box)
    depth = (np.float32(6371000.0) - z).astype(np.float64) / 1000
    k = lambda v: np.float32(1000.0) * np.float32(v)     # km/s, g/cm^3 read as REAL(4), times 1000
    rho = np.where(depth > 35.0, k(3.4), k(2.9)).astype(np.float32)
    cs = np.where(depth > 35.0, k(4.5), k(3.9)).astype(np.float32)
    cp = np.where(depth > 35.0, k(8.1), k(6.8)).astype(np.float32)
    assert cp.max() != np.float32(8100.0)                # 8.1 km/s is not exactly 8100 m/s in FP32
    ex, ey, ez = p.nx + 1, p.ny + 1, p.nz + 1
    mu = ((cs * cs) * rho).astype(np.float32)
    lam = ((cp * cp - np.float32(2) * cs * cs) * rho).astype(np.float32)
    grid = lambda a: np.broadcast_to(a.T[:, None, None, :, None, None], (5, 5, 5, ez, ey, ex)).reshape(-1)
    assert np.array_equal(m["mu"], grid(mu)) and np.array_equal(m["lambda"], grid(lam))
    assert np.array_equal(m["rhoinv"], grid((np.float32(1) / rho).astype(np.float32)))
    assert np.all(m["A"] == 0) and np.all(m["B"] == 0) and np.all(m["C"] == 0)
    assert set(np.unique(m["Q"])) <= {np.float32(300.0), np.float32(150.0)}


def test_generate_models_tree(tmp_path):
    s = synth.split_setup(synth.make_setup((6, 5, 4)), (6, 5, 4), (2, 1, 2))
    prof = M.LayeredProfile([0.0, 35.0], [2.9, 3.4], [6.8, 8.1], [3.9, 4.5], [300.0, 150.0])
    boxes = M.generate_models(s, str(tmp_path), prof)
    assert len(boxes) == 4
    assert len(F.read_boxfile(str(tmp_path / "MODELS" / "MODELS" / "boxfile"))) == 4
    for r, b in enumerate(boxes):
        m = F.read_model(str(tmp_path / "MODELS" / "MODELS"), r, 125 * (b.nx + 1) * (b.ny + 1) * (b.nz + 1), 1)
        ref = M.profile_model(b, prof, 1)
        for k in ref:
            assert np.array_equal(m[k], ref[k]), (r, k)
        xco = np.loadtxt(str(tmp_path / "DATA" / "COORDINATES" / ("xco_%d" % r)), dtype=np.float64)
        assert np.array_equal(xco.astype(np.float32), M.box_axes(b)[0].reshape(-1))


def checker_blocks(box, rng):
    """Two overlapping-range subvolumes covering the box (colat/lon degrees, radius km)."""
    xd = float(box.xmin) * 180 / np.pi, float(box.xmax) * 180 / np.pi
    yd = float(box.ymin) * 180 / np.pi, float(box.ymax) * 180 / np.pi
    zk = float(box.zmin) / 1000, float(box.zmax) / 1000
    subs = []
    for n in ((4, 5, 3), (7, 3, 6)):
        bx = np.linspace(xd[0] - 1.0, xd[1] + 1.0, n[0] + 1).astype(np.float32)
        by = np.linspace(yd[0] - 0.7, yd[1] + 0.3, n[1] + 1).astype(np.float32)
        bz = np.linspace(zk[0] - 10, zk[1] + 5, n[2] + 1).astype(np.float32)
        v = lambda: (0.1 * rng.standard_normal(n)).astype(np.float32)
        subs.append((bx, by, bz, v(), v(), v(), (0.05 * rng.standard_normal(n)).astype(np.float32)))
    return subs


def test_block_files_round_trip(tmp_path):
    p = synth.make_problem("tiny", nt=5, seed=2, model=False)
    subs = checker_blocks(p.box, np.random.default_rng(0))
    svs = [M.SubVolume(s[0], s[1], s[2], s[3]) for s in subs]
    M.write_block_model(str(tmp_path), "dvsh", svs)
    back = M.read_block_model(str(tmp_path), "dvsh")
    for a, b in zip(svs, back):
        assert np.array_equal(a.x, b.x) and np.array_equal(a.z, b.z) and np.array_equal(a.v, b.v)


@pytest.mark.parametrize("seed", [3, 4])
def test_add_perturbation_matches_oracle(oracle_mod, tmp_path, seed):
    from models_oracle import add_perturbation as oracle_add
    rng = np.random.default_rng(seed)
    p = synth.make_problem("tiny", nt=5, seed=seed, n_el=(7, 6, 5))
    b = p.box
    subs = checker_blocks(b, rng)
    for name, col in (("dvsh", 3), ("dvsv", 4), ("dvp", 5), ("drho", 6)):
        M.write_block_model(str(tmp_path), name, [M.SubVolume(s[0], s[1], s[2], s[col]) for s in subs],
                            coords=(name == "dvsh"))
    m = {k: v.copy() for k, v in p.model.items()}
    m["B"] = (np.float32(0.05) * m["mu"]).astype(np.float32)   # radially anisotropic start
    got = M.add_perturbation(m, b, str(tmp_path))
    x, y, z = M.box_axes(b)
    cox, coy, coz = M._grid(x, y, z, b.nx + 1, b.ny + 1, b.nz + 1)
    # the oracle reads the same decimal files the product read
    svs = [M.read_block_model(str(tmp_path), nm) for nm in ("dvsh", "dvsv", "dvp", "drho")]
    osubs = [(svs[0][q].x, svs[0][q].y, svs[0][q].z, svs[0][q].v, svs[1][q].v, svs[2][q].v, svs[3][q].v)
             for q in range(len(subs))]
    ri, mu, lam, B = oracle_add(m["rhoinv"], m["mu"], m["lambda"], m["B"], cox, coy, coz,
                                tuple(np.float32(v) for v in (b.xmin, b.xmax, b.ymin, b.ymax, b.zmin, b.zmax)), osubs)
    changed = np.count_nonzero(got["mu"] != p.model["mu"])
    assert changed > 0.5 * got["mu"].size
    assert np.array_equal(got["rhoinv"], ri)
    assert np.array_equal(got["mu"], mu)
    assert np.array_equal(got["lambda"], lam)
    assert np.array_equal(got["B"], B)
    assert np.array_equal(got["A"], p.model["A"]) and np.array_equal(got["Q"], p.model["Q"])


@pytest.mark.skipif(not os.path.isdir(REF_BLOCKS), reason="reference block fixture not present")
def test_reads_reference_block_fixture():
    """The block_x/y/z fixture shipped with the reference parses (2 subvolumes)."""
    for ax in "xyz":
        lines = M.read_block_lines(os.path.join(REF_BLOCKS, "block_" + ax))
        assert len(lines) == 2 and all(len(a) > 1 for a in lines)
    z = M.read_block_lines(os.path.join(REF_BLOCKS, "block_z"))
    assert np.all(np.diff(z[0]) > 0)          # radius [km], increasing


def test_cli_generate_and_perturb_tree(tmp_path):
    """generate-models writes a tree the driver's stitcher reads back; --perturb changes it
    exactly as add_perturbation does box by box."""
    from ses3d_gb300.__main__ import main
    root = tmp_path / "tree"
    s = synth.split_setup(synth.make_setup((6, 5, 4)), (6, 5, 4), (2, 1, 1))
    os.makedirs(root / "INPUT")
    F.write_setup(str(root / "INPUT" / "setup"), s)
    table = tmp_path / "profile.txt"
    table.write_text("# top depth rho vp vs Q\n0 2.9 6.8 3.9 300\n35 3.4 8.1 4.5 150\n")
    assert main(["generate-models", "--root", str(root), "--profile", str(table)]) == 0
    boxes = F.read_boxfile(str(root / "MODELS" / "MODELS" / "boxfile"))
    before = [F.read_model(str(root / "MODELS" / "MODELS"), r, 125 * (b.nx + 1) * (b.ny + 1) * (b.nz + 1), 1)
              for r, b in enumerate(boxes)]
    subs = checker_blocks(boxes[0], np.random.default_rng(9))
    bdir = root / "MODELS" / "MODELS_3D"
    for name, col in (("dvsh", 3), ("dvsv", 4), ("dvp", 5), ("drho", 6)):
        M.write_block_model(str(bdir), name, [M.SubVolume(q[0], q[1], q[2], q[col]) for q in subs])
    assert main(["generate-models", "--root", str(root), "--profile", str(table), "--perturb"]) == 0
    for r, b in enumerate(boxes):
        after = F.read_model(str(root / "MODELS" / "MODELS"), r, 125 * (b.nx + 1) * (b.ny + 1) * (b.nz + 1), 1)
        want = M.add_perturbation(before[r], b, str(bdir))
        for k in ("rhoinv", "mu", "lambda", "B"):
            assert np.array_equal(after[k], want[k]), (r, k)
        assert np.array_equal(after["Q"], before[r]["Q"])
