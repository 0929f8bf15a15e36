"""The C ABI library: built, loadable without a GPU, exporting exactly what
include/seisfat2d.h declares. No compute calls here."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(sf_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(engine_lib):
    names = declared_symbols()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(engine_lib, n), n


def test_binding_table_covers_header():
    from seisfat2d_gb300 import _lib
    assert set(_lib.SIGNATURES) == declared_symbols()


def test_status_strings(engine_lib):
    for st in range(0, 7):
        s = engine_lib.sf_status_string(st)
        assert s and len(s) > 1


def test_engine_refuses_missing_library(tmp_path, monkeypatch):
    from seisfat2d_gb300 import _lib, build
    monkeypatch.setattr(build, "LIB", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    try:
        _lib.load()
    except RuntimeError as e:
        assert "no CPU fallback" in str(e)
    else:
        raise AssertionError("load() must fail without the library")


def test_every_entry_point_rejects_a_null_context(engine_lib):
    """Host-side argument checks, no device work: every entry point that takes
    a context returns SF_ERR_ARG for a null one (destroying a null context is
    a no-op, as free(NULL) is), and the no-allocation solver rejects a null
    field."""
    from seisfat2d_gb300 import _lib
    L = _lib.load()
    skip = {"sf_ctx_create", "sf_status_string", "sf_ctx_last_error", "sf_time_propagation_noalloc"}
    for name, (res, args) in sorted(_lib.SIGNATURES.items()):
        if name in skip:
            continue
        vals = []
        for a in args:
            if a in (C.c_int, C.c_uint, C.c_long, C.c_size_t):
                vals.append(0)
            elif a in (C.c_float, C.c_double):
                vals.append(0.0)
            elif isinstance(a, type) and issubclass(a, C.Array):
                vals.append(a())
            else:
                vals.append(None)
        st = getattr(L, name)(*vals)
        assert st == (0 if name == "sf_ctx_destroy" else 1), (name, st)
    assert L.sf_ctx_last_error(None) == b"null context"
    st = L.sf_time_propagation_noalloc(None, 10, 10, 1.0, 1.0, 0.0, 0.0, None, None)
    assert st == 1


def test_context_creation_fails_cleanly_without_a_gpu(engine_lib):
    import pytest
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from seisfat2d_gb300 import _lib
    L = _lib.load()
    ctx = C.c_void_p()
    st = L.sf_ctx_create(C.byref(ctx), 40, 20, 10.0, 10.0, 0)
    assert st == 2 and not ctx.value  # SF_ERR_CUDA, no context handed out
