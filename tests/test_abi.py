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
