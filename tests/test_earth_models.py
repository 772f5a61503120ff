"""The reference's built-in 1-D Earth models (model_type 1/2/3/4/7 of generate_models) against
the oracle's statement-by-statement restatement: FP32 values bit for bit at every GLL
radius of several boxes (including one that reaches the inner core) and at every layer
boundary and its FP32 neighbours."""
import os
import re

import numpy as np
import pytest

from ses3d_gb300 import earth_models as EM
from ses3d_gb300 import formats as F
from ses3d_gb300 import models as M

import earth_models_oracle as O

f32 = np.float32


def box(nz, zmin, zmax, nx=3, ny=2):
    return F.Box(index=0, multi=(1, 1, 1), nx_min=0, nx_max=nx - 1, ny_min=0, ny_max=ny - 1, nz_min=0,
                 nz_max=nz - 1, xmin=f32(0.7), xmax=f32(1.0), ymin=f32(0.1), ymax=f32(0.3), zmin=f32(zmin),
                 zmax=f32(zmax))


BOXES = [box(10, 5771000.0, 6371000.0), box(40, 5771000.0, 6371000.0), box(60, 1000000.0, 6371000.0),
         box(7, 3000000.0, 6200000.0)]

BOUNDS = sorted({6371000.0, 6356000.0, 6346600.0, 6291000.0, 6191000.0, 6151000.0, 6100000.0, 6051000.0,
                 5971000.0, 5771000.0, 5701000.0, 5600000.0, 3630000.0, 3480000.0, 1221500.0, 1221000.0})


def boundary_radii():
    """Every layer boundary with its FP32 neighbours, as a (n, 5) array."""
    z = []
    for b in BOUNDS:
        v = f32(b)
        z += [np.nextafter(v, f32(-np.inf)), v, np.nextafter(v, f32(np.inf))]
    z += [f32(500e3), f32(0.0)]
    z = np.array(z, f32)
    pad = (-len(z)) % 5
    return np.concatenate([z, np.full(pad, f32(4000e3))]).reshape(-1, 5)


def same(a, b):
    return np.array_equal(np.asarray(a, f32), np.asarray(b, f32))


@pytest.mark.parametrize("is_diss", [1, 0])
def test_profiles_at_boundaries(is_diss):
    z = boundary_radii()
    for mine, ref in ((EM.prem_iso(z, is_diss), O.prem_iso(z, is_diss)),
                      (EM.eumod_bg(z, is_diss), O.eumod_bg(z, is_diss)),
                      (EM.ak135(z, is_diss), O.ak135(z, EM.AK135, is_diss))):
        for a, b in zip(mine, ref):
            assert same(a, b)
    assert same(EM.ql6(z, is_diss), O.ql6(z, is_diss))


@pytest.mark.parametrize("b", BOXES, ids=lambda b: "nz%d_%d" % (b.nz + 1, int(b.zmin)))
@pytest.mark.parametrize("model_type", [1, 2, 3, 4, 7])
@pytest.mark.parametrize("is_diss", [1, 0])
def test_builtin_records_match_oracle(b, model_type, is_diss):
    """The MODELS records of a box for each model_type, bit for bit."""
    mine = M.builtin_model(b, model_type, is_diss)
    ex, ey, ez = b.nx + 1, b.ny + 1, b.nz + 1
    _, _, z = M.box_axes(b)
    if model_type == 1:
        ref = M.homogeneous(b, is_diss)
    elif model_type == 3:
        ref = M.homogeneous(b, is_diss)
        if is_diss:
            ref["Q"] = O.records(np.ones_like(z), z * 0, z * 0, O.ql6(z, is_diss), ex, ey, 1)["Q"]
    else:
        prof = {2: lambda: O.prem_iso(z, is_diss), 4: lambda: O.eumod_bg(z, is_diss),
                7: lambda: O.ak135(z, EM.AK135, is_diss)}[model_type]()
        ref = O.records(*prof, ex, ey, is_diss)
    assert set(mine) == set(ref)
    n = 125 * ex * ey * ez
    for k in ref:
        assert mine[k].size == n and same(mine[k], ref[k]), (model_type, k)
    if model_type in (2, 4, 7):
        assert np.all(mine["rhoinv"] > 0)


def test_published_values():
    """Spot values of the tabulated models: surface layers and the 670 km discontinuity."""
    z = np.array([[6371000.0, 6360000.0, 5711000.0, 5701000.0, 4000000.0]], f32)
    rho, vp, vs, q = EM.prem_iso(z, 1)
    assert (rho[0, 0], vp[0, 0], vs[0, 0], q[0, 0]) == (f32(2600.0), f32(5800.0), f32(3200.0), f32(600.0))
    assert vs[0, 4] > 7000 and q[0, 4] == f32(312.0)
    rho, vp, vs, _ = EM.ak135(z, 1)
    assert (rho[0, 0], vp[0, 0], vs[0, 0]) == (f32(2720.0), f32(5800.0), f32(3460.0))
    e = np.full((2, 5), f32(6371000.0))
    e[1] = f32(6300000.0)
    rho, vp, vs, _ = EM.eumod_bg(e, 1)
    assert np.all(rho[0] == f32(3000.0)) and np.all(vs[0] == f32(4100.0))


def test_generate_models_uses_setup_model_type(tmp_path):
    from ses3d_gb300 import synth
    setup = synth.make_setup((4, 3, 5), is_diss=1)
    setup.model_type = 2
    boxes = M.generate_models(setup, str(tmp_path), coordinates=False)
    n = 125 * 4 * 3 * 5
    rhoinv = F.read_record(os.path.join(str(tmp_path), "MODELS", "MODELS", "rhoinv0"), n)
    assert np.array_equal(rhoinv, M.builtin_model(boxes[0], 2, 1)["rhoinv"])
    with pytest.raises(ValueError):
        M.builtin_model(boxes[0], 5, 1)


REF = os.environ.get("SES3D_REFERENCE_ROOT", "")


@pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "MODELS", "MODELS_1D"))),
                    reason="SES3D_REFERENCE_ROOT does not name the reference tree")
def test_ak135_table_equals_reference_source():
    """The transcribed ak135 table equals the arrays of MODELS_1D/ak135.f90, read as REAL(4)."""
    src = open(os.path.join(REF, "MODELS", "MODELS_1D", "ak135.f90")).read()
    for col, name in ((0, "ak135_r"), (1, "ak135_rho"), (2, "ak135_cp"), (3, "ak135_cs")):
        m = re.search(name + r"\(:\)=\(/(.*?)/\)", src, re.S)
        vals = [F.strtof(v.strip()) for v in m.group(1).replace("&", "").split(",") if v.strip()]
        assert np.array_equal(np.array(vals, f32), EM.AK135[:, col]), name
