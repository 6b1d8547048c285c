"""CPU-side checks of the C-ABI library: it builds, loads without a GPU and
exports every entry point the header declares (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ultradmrg_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(udmrg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    from ultradmrg_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("udmrg_eff_ham_mul_two_site_state", "udmrg_lanczos_solver", "udmrg_svd",
              "udmrg_update_site_lenvs", "udmrg_update_site_renvs",
              "udmrg_two_site_finite_vmps", "udmrg_lanczos_expmv_solver"):
        assert s in syms


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(libpath):
    from ultradmrg_gb300 import _lib
    bound = set(_lib.SIGNATURES) | {"udmrg_last_error"}
    assert set(declared_symbols()) <= bound


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from ultradmrg_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(_lib.UdmrgError):
        _lib.lib()
