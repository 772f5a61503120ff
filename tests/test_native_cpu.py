"""CPU checks of the native boundary: the library builds, loads, and exports every
entry point include/ses3d_gpu.h declares; without a GPU it fails cleanly."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "ses3d_gpu.h")) as f:
        txt = f.read()
    return sorted(set(re.findall(r"\b(ses3d_gpu_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "ses3d_gpu_create" in syms and "ses3d_gpu_step" in syms
    assert len(syms) >= 30


def test_library_exports_every_declared_symbol(native):
    lib = ctypes.CDLL(os.path.join(ROOT, "ses3d_gb300", "libses3d_gpu.so"))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header(native):
    from ses3d_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), set(declared_symbols()) - set(_lib.SIGNATURES)


def test_version_string(native):
    assert b"sm_103a" in native.ses3d_gpu_version()


def test_create_without_gpu_fails_cleanly(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ses3d_gb300 import _lib
    from ses3d_gb300 import synth
    from ses3d_gb300.solver import Simulation, config_from
    p = synth.make_problem("tiny", nt=5, model=False)
    cfg = config_from(p.box, p.setup, 5, p.events[0].event.dt, p.tau, p.D, pml=3)
    with pytest.raises(_lib.Ses3dError) as ei:
        Simulation(cfg)
    assert ei.value.code == -7


def test_create_rejects_bad_config(native):
    from ses3d_gb300 import _lib
    cfg = _lib.Config()
    cfg.lpd = 5
    h = ctypes.c_void_p()
    rc = native.ses3d_gpu_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == -1
    assert b"lpd" in native.ses3d_gpu_last_error(None)


def test_driver_builds_and_reports_missing_gpu(native, tmp_path):
    """The reference-style driver parses a generated SES3D tree and fails cleanly without a GPU."""
    import subprocess
    import torch
    from ses3d_gb300 import synth
    drv = os.path.join(ROOT, "ses3d_gb300", "ses3d_gpu_main")
    assert os.path.exists(drv)
    assert subprocess.run([drv, "--help"], capture_output=True).returncode == 0
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = synth.make_problem("tiny", nt=5, seed=1)
    synth.write_problem(p, str(tmp_path))
    res = subprocess.run([drv, "--main", str(tmp_path / "MAIN"), "--pml", "3"], capture_output=True, text=True)
    assert res.returncode == 1 and "no CUDA device" in res.stderr


def _header():
    import re
    h = open(os.path.join(ROOT, "include", "ses3d_gpu.h")).read()
    decl = dict((name, ret) for ret, name in re.findall(r"^(const char \*|void \*|int64_t|long|int) ?(ses3d_gpu_\w+)\(",
                                                        h, re.M))
    return h, decl


def test_fortran_module_covers_header():
    """include/ses3d_gpu.f90 (the ISO_C_BINDING module) declares every entry point of the
    header with the header's return kind."""
    import re
    h, decl = _header()
    mod = open(os.path.join(ROOT, "include", "ses3d_gpu.f90")).read()
    fort = dict((name, kind) for kind, name in re.findall(r"(integer\(c_\w+\)|type\(c_ptr\)) function (ses3d_gpu_\w+)",
                                                          mod))
    assert set(decl) == set(fort), sorted(set(decl) ^ set(fort))
    want = {"int": "integer(c_int)", "long": "integer(c_long)", "int64_t": "integer(c_int64_t)",
            "const char *": "type(c_ptr)", "void *": "type(c_ptr)"}
    for name, ret in decl.items():
        assert fort[name] == want[ret], (name, ret, fort[name])
    for name in decl:   # every interface binds the C name and ends
        assert re.search(r"function %s\([^)]*\) bind\(c\)" % name, mod), name


def test_fortran_module_constants_match_header():
    """Status codes, field and kernel identifiers of the Fortran module equal the header's."""
    import re
    h, _ = _header()
    mod = open(os.path.join(ROOT, "include", "ses3d_gpu.f90")).read()
    fort = {k: int(v) for k, v in re.findall(r"(SES3D_\w+) = (-?\d+)", mod)}
    codes = {k: int(v) for k, v in re.findall(r"#define (SES3D_\w+) \(?(-?\d+)\)?", h)}
    for k, v in codes.items():
        assert fort[k] == v, k
    for enum in re.findall(r"enum \{([^}]*)\}", h):
        names = re.findall(r"(SES3D_(?:FIELD|KERNEL)_\w+)", re.sub(r"/\*.*?\*/", "", enum, flags=re.S))
        for i, k in enumerate(n for n in names if not n.endswith("_COUNT")):
            assert fort[k] == i, k


def test_fortran_driver_calls_declared_entry_points():
    """The Fortran driver calls only entry points the module declares, and its build
    recipe names the module and the library."""
    import re
    mod = open(os.path.join(ROOT, "include", "ses3d_gpu.f90")).read()
    drv = open(os.path.join(ROOT, "ses3d_gb300", "fortran", "ses3d_gpu_main.f90")).read()
    declared = set(re.findall(r"function (ses3d_gpu_\w+)", mod))
    used = set(re.findall(r"(ses3d_gpu_\w+)\(", drv))
    assert used and used <= declared, sorted(used - declared)
    mk = open(os.path.join(ROOT, "ses3d_gb300", "fortran", "Makefile")).read()
    assert "ses3d_gpu.f90" in mk and "-lses3d_gpu" in mk
