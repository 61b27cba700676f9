"""libmrhyde_gb.so builds for sm_103a, loads without a GPU and exports every symbol include/*.h declares."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(mrg_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    from mrhyde_gb300 import _lib

    L = _lib.lib()
    declared = _declared()
    assert len(declared) >= 14
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding covers every declared entry point too
    assert declared <= set(_lib.SIGNATURES), sorted(declared - set(_lib.SIGNATURES))


def test_version_and_error_buffer_without_gpu():
    from mrhyde_gb300 import _lib

    L = _lib.lib()
    assert b"sm_103a" in L.mrg_version()
    buf = ctypes.create_string_buffer(64)
    assert L.mrg_last_error(buf, 64) == 0
    assert L.mrg_last_error(None, 0) == _lib.MRG_EINVAL


def test_null_arguments_rejected_without_touching_the_gpu():
    from mrhyde_gb300 import _lib

    L = _lib.lib()
    assert L.mrg_problem_create(None, None, None) == _lib.MRG_EINVAL
    assert L.mrg_problem_get_info(None, None) == _lib.MRG_EINVAL
    assert L.mrg_assemble(None, None, None, None, 3, None) == _lib.MRG_EINVAL
    assert "null" in _lib.last_error()


def test_bad_descriptors_rejected_before_any_allocation():
    from mrhyde_gb300 import _lib

    L = _lib.lib()
    m, ph = _lib.MeshDesc(), _lib.PhysicsDesc()
    out = ctypes.c_void_p()
    m.dim, m.order, m.nx, m.ny, m.nz = 4, 1, 2, 2, 2
    assert L.mrg_problem_create(ctypes.byref(m), ctypes.byref(ph), ctypes.byref(out)) == _lib.MRG_EINVAL
    m.dim, m.order = 3, 3
    assert L.mrg_problem_create(ctypes.byref(m), ctypes.byref(ph), ctypes.byref(out)) == _lib.MRG_EINVAL
    m.order, m.nx = 1, 0
    assert L.mrg_problem_create(ctypes.byref(m), ctypes.byref(ph), ctypes.byref(out)) == _lib.MRG_EINVAL
    m.nx = 2
    ph.kind = 9
    assert L.mrg_problem_create(ctypes.byref(m), ctypes.byref(ph), ctypes.byref(out)) == _lib.MRG_EINVAL
    assert not out.value
