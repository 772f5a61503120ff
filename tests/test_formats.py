"""Reference file formats: the example inputs shipped with the reference (parsed when the
reference tree is present) and writer/reader round trips."""
import os

import numpy as np
import pytest

from ses3d_gb300 import formats as F
from ses3d_gb300 import synth

# the reference project's root (its example INPUT files are the parser fixtures); the tests
# that read them are skipped when SES3D_REFERENCE_ROOT does not name a reference tree
REF = os.environ.get("SES3D_REFERENCE_ROOT", "")
needs_ref = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "INPUT"))),
                               reason="SES3D_REFERENCE_ROOT does not name the reference tree")


@needs_ref
def test_reference_setup():
    s = F.read_setup(os.path.join(REF, "INPUT", "setup"))
    assert (s.xmin, s.xmax, s.ymin, s.ymax) == (np.float32(47.1), np.float32(55.9), np.float32(23.1), np.float32(42.9))
    assert (s.zmin, s.zmax) == (np.float32(5900000.0), np.float32(6371000.0))
    assert (s.is_diss, s.model_type) == (0, 1)
    assert (s.nx_global, s.ny_global, s.nz_global, s.lpd, s.px, s.py, s.pz) == (66, 108, 28, 4, 3, 4, 4)
    assert (s.adjoint_flag, s.samp_ad) == (0, 15)
    assert s.ffd == "../DATA/OUTPUT/NEEDS_A_LOT_OF_SPACE/ADJOINT"


@needs_ref
def test_reference_event_and_relax():
    e = F.read_event(os.path.join(REF, "INPUT", "event_1"))
    assert (e.nt, e.dt) == (4000, np.float32(0.13))
    assert (e.xxs, e.yys, e.zzs, e.source_type) == (np.float32(50.74), np.float32(41.04), np.float32(5000.0), 10)
    assert np.array_equal(e.mom, np.array([1e16, 1e16, 1e16, 0, 0, 0], np.float32))
    assert e.ofd == "../DATA/OUTPUT/1.8s/" and (e.ssamp, e.output_displacement) == (15000, 0)
    tau, D = F.read_relax(os.path.join(REF, "INPUT", "relax"))
    assert np.array_equal(tau, np.array([1.7308, 14.3961, 22.9973], np.float32))
    assert np.array_equal(D, np.array([2.51, 2.4354, 0.0879], np.float32))
    assert F.read_event_list(os.path.join(REF, "INPUT", "event_list")) == ["1"]


@needs_ref
def test_reference_stf_skips_four_lines():
    """INPUT/stf has no header, yet the reader skips 4 lines (ses3d_input.f90:419-422)."""
    so = F.read_stf(os.path.join(REF, "INPUT", "stf"), 4000)
    with open(os.path.join(REF, "INPUT", "stf")) as f:
        lines = f.read().split()
    assert so.size == 4000
    assert so[0] == F.strtof(lines[4]) and so[-1] == F.strtof(lines[4003])


@needs_ref
def test_reference_recfile_and_adjoint_files():
    r = F.read_recfile(os.path.join(REF, "INPUT", "recfile_1"))
    assert len(r.names) == 320
    assert r.names[0] == "ADVT_.KO.___" and len(r.names[0]) == 12
    assert np.array_equal(r.loc[0], np.array([49.5668, 29.7383, 0.0], np.float32))
    loc = F.read_ad_srcfile(os.path.join(REF, "ADJOINT", "1", "ad_srcfile"))
    assert np.array_equal(loc, np.array([[50.36, 27.88, 1000.0]], np.float32))
    stf = F.read_ad_src(os.path.join(REF, "ADJOINT", "1", "ad_src_1"), 4000)
    assert stf.shape == (3, 4000)


def test_roundtrip_text_inputs(tmp_path):
    p = synth.make_problem("tiny", nt=20, seed=1)
    synth.write_problem(p, str(tmp_path))
    s = F.read_setup(str(tmp_path / "INPUT" / "setup"))
    assert (s.xmin, s.xmax, s.nx_global, s.is_diss) == (p.setup.xmin, p.setup.xmax, p.setup.nx_global, p.setup.is_diss)
    e = F.read_event(str(tmp_path / "INPUT" / "event_1"))
    assert e.nt == 20 and e.dt == p.events[0].event.dt and np.array_equal(e.mom, p.events[0].event.mom)
    assert (e.xxs, e.yys, e.zzs) == (p.events[0].event.xxs, p.events[0].event.yys, p.events[0].event.zzs)
    so = F.read_stf(str(tmp_path / "INPUT" / "stf"), 20)
    assert np.array_equal(so, p.events[0].stf[:20])
    r = F.read_recfile(str(tmp_path / "INPUT" / "recfile_1"))
    assert np.array_equal(r.loc, p.events[0].receivers.loc)
    tau, D = F.read_relax(str(tmp_path / "INPUT" / "relax"))
    assert np.array_equal(tau, p.tau) and np.array_equal(D, p.D)
    b = F.read_boxfile(str(tmp_path / "MODELS" / "MODELS" / "boxfile"))[0]
    assert (b.nx, b.ny, b.nz) == (p.nx, p.ny, p.nz)
    assert (b.xmin, b.xmax, b.zmin, b.zmax) == (p.box.xmin, p.box.xmax, p.box.zmin, p.box.zmax)
    m = F.read_model(str(tmp_path / "MODELS" / "MODELS"), 0, p.n_nodes, 1)
    for k in F.MODEL_NAMES:
        assert np.array_equal(m[k], p.model[k])


def test_boxfile_decomposition_matches_generator_formula():
    """Multi-box decomposition as MODELS/SOURCE/generate_models.f90:200-283 (FP32)."""
    s = synth.make_setup((23, 22, 11))
    s.px, s.py, s.pz = 3, 2, 2
    s.nx_global, s.ny_global, s.nz_global = 23 - 3, 22 - 2, 11 - 2
    boxes = F.make_boxes(s)
    assert len(boxes) == 12
    assert [b.index for b in boxes] == list(range(1, 13))
    assert boxes[0].nx_min == 0 and boxes[-1].nx_max == s.nx_global
    # neighbouring boxes share the physical boundary exactly
    assert boxes[0].xmax == boxes[1].xmin
    total = sum((b.nx + 1) for b in boxes[:3])
    assert total == 23


def test_records_roundtrip(tmp_path):
    a = [np.arange(10, dtype=np.float32), np.ones(3, np.float32)]
    F.write_records(str(tmp_path / "r"), a)
    F.write_records(str(tmp_path / "r"), [np.full(4, 2.5, np.float32)], append=True)
    back = F.read_records(str(tmp_path / "r"))
    assert len(back) == 3 and np.array_equal(back[0], a[0]) and np.array_equal(back[2], np.full(4, 2.5, np.float32))
    raw = (tmp_path / "r").read_bytes()
    assert raw[:4] == (40).to_bytes(4, "little") and raw[44:48] == (40).to_bytes(4, "little")


def test_seismogram_writer_layout_and_roundtrip(tmp_path):
    rng = np.random.default_rng(3)
    tr = [rng.standard_normal(25).astype(np.float32) * np.float32(1e-7) for _ in range(3)]
    tr[0][0] = 0.0
    F.write_seismograms(str(tmp_path) + "/", "ABC", *tr, nt=25, dt=np.float32(0.1),
                        recloc=(45.0, 10.0, 0.0), src=(50.0, 10.0, 10000.0))
    path = str(tmp_path / ("ABC" + " " * 9 + ".x"))  # 12-character padded station name
    nt, dt, x = F.read_seismogram(path)
    assert nt == 25 and abs(dt - 0.1) < 1e-7
    assert np.array_equal(x, tr[0])
    with open(path) as f:
        lines = f.read().splitlines()
    assert lines[0] == " theta component seismograms"
    assert lines[3].strip().startswith("receiver location")


@pytest.mark.parametrize("v,expect", [(0.0, "   0.00000000    "), (1.0, "   1.00000000    "),
                                      (0.1, "  0.100000001    "), (1e-5, "   9.99999975E-06")])
def test_fortran_list_directed_real_format(v, expect):
    assert F.fmt_real(np.float32(v)) == expect
