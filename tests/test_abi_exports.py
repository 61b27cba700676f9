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


def _declarations():
    """name -> list of parameter declarations, from include/*.h (comments removed)."""
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(mrg_[a-z0-9_]+)\s*\(([^()]*)\)\s*;", src):
            params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
            out[m.group(1)] = params
    return out


def _param_class(decl):
    """pointer / i32 / u32 / i64 / u64 / f64 / size of one C parameter declaration."""
    if "*" in decl or "mrg_stream_t" in decl:
        return "ptr"
    t = decl.split()[0] if not decl.startswith("const ") else decl.split()[1]
    return {"int32_t": "i32", "int": "i32", "uint32_t": "u32", "int64_t": "i64", "uint64_t": "u64",
            "double": "f64", "size_t": "size"}[t]


def _ctype_class(ct):
    import ctypes as C

    if ct in (C.c_void_p, C.c_char_p) or (isinstance(ct, type) and issubclass(ct, C._Pointer)):
        return "ptr"
    return {C.c_int32: "i32", C.c_uint32: "u32", C.c_int64: "i64", C.c_uint64: "u64", C.c_double: "f64",
            C.c_size_t: "size"}[ct]


def test_binding_signatures_match_the_header():
    """Every entry point's ctypes argument list in the Python binding has the header's parameter count and
    classes (pointer, 32/64-bit integer, double), so an argument cannot be passed with the wrong width."""
    from mrhyde_gb300 import _lib

    decls = _declarations()
    assert set(decls) == _declared()
    for name, params in decls.items():
        _, argtypes = _lib.SIGNATURES[name]
        assert len(argtypes) == len(params), (name, params)
        got = [_ctype_class(t) for t in argtypes]
        want = [_param_class(p) for p in params]
        # int and int32_t are the same width; size_t is 64-bit on both hosts
        norm = {"size": "u64"}
        assert [norm.get(x, x) for x in got] == [norm.get(x, x) for x in want], (name, params, got)


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
