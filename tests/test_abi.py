"""The C-ABI library loads and exports every function include/*.h declares
(no device work: runs without a GPU)."""
import os
import re
import subprocess

from framelab_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src,
                             flags=re.M):
            if m.group(1) not in ("defined",):
                names.add(m.group(1))
    return names


def test_library_loads_and_exports_all_declared_symbols():
    L = _lib.load()
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    declared = _declared()
    assert len(declared) >= 10
    missing = sorted(declared - exported)
    assert not missing, missing
    for n in declared:
        assert getattr(L, n) is not None


def test_status_functions_without_gpu():
    L = _lib.load()
    assert L.fl_version().startswith(b"framelab_gb300")
    assert isinstance(L.fl_last_status(), int)


def test_plan_rejects_bad_geometry_without_touching_the_gpu():
    import ctypes as C
    L = _lib.load()
    s = _lib.Scan()
    s.ndim = 4
    h = C.c_void_p()
    assert L.fl_plan_create(C.byref(s), C.byref(h)) == _lib.FL_ERR_INVALID
    assert b"ndim" in L.fl_last_error()
    s.ndim = 3; s.nx = s.ny = s.nz = 8; s.nv = 0; s.na = s.nb = 4
    assert L.fl_plan_create(C.byref(s), C.byref(h)) == _lib.FL_ERR_INVALID


def test_python_constants_match_the_header_enums():
    """Every enumerator of include/*.h that the Python binding also names
    (with or without the FL_ prefix) has the same value there, and the
    plan options, tunables and status codes are all named."""
    values = {}
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", f)).read(), flags=re.S)
        for body in re.findall(r"\benum\s*\{(.*?)\}", src, flags=re.S):
            for m in re.finditer(r"\b(FL_\w+)\s*=\s*(\d+)", body):
                values[m.group(1)] = int(m.group(2))
    assert len(values) >= 30
    matched = {}
    for name, v in values.items():
        for py in (name, name[3:]):
            if hasattr(_lib, py):
                assert getattr(_lib, py) == v, (name, py)
                matched[name] = py
    must = [n for n in values if n.startswith(("FL_OPT_", "FL_TUNE_", "FL_ERR_", "FL_DEBUG_"))]
    assert not [n for n in must if n not in matched], must
