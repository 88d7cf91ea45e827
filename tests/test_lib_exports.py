"""The C-ABI library loads and exports every symbol include/*.h declares; no
compute calls (no GPU needed)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(gpda_[A-Za-z0-9_]+)\s*\(", src))
    return names


def test_every_declared_symbol_is_exported(gpda_lib):
    decl = declared_functions()
    assert len(decl) >= 40
    missing = [n for n in sorted(decl) if not hasattr(gpda_lib, n)]
    assert not missing, missing


def test_binding_covers_header(gpda_lib):
    from gsmfretda_gb300._lib import SIGNATURES
    assert declared_functions() <= set(SIGNATURES)


def test_library_is_in_tree_and_loaded_from_there(gpda_lib):
    from gsmfretda_gb300._lib import LIB_PATH
    assert os.path.dirname(LIB_PATH) == os.path.join(ROOT, "gsmfretda_gb300")
    with open("/proc/self/maps") as f:
        assert LIB_PATH in f.read()


def test_host_only_entry_points(gpda_lib):
    assert gpda_lib.gpda_version().startswith(b"gpda")
    assert gpda_lib.gpda_params_size() == 284
    from gsmfretda_gb300._lib import GpdaModel
    m = GpdaModel()
    gpda_lib.gpda_model_defaults(C.byref(m))
    assert m.nbins == 21 and m.left_pad == 2
    assert abs(m.rc_gamma - 0.34) < 1e-7 and abs(m.rc_r0 - 52.0) < 1e-6


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    import gsmfretda_gb300._lib as L
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(L, "_lib", None)
    try:
        L.load()
        raise AssertionError("load() must raise without the CUDA library")
    except ImportError as e:
        assert "no CPU fallback" in str(e)
