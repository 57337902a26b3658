"""CPU-side checks of the C ABI: the library builds, loads without a GPU and exports every symbol
declared in include/mhdgb.h; argument validation that needs no device."""
import ctypes as C
import os
import re

import pytest

from mhdturbulence_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "mhdgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mhdgb_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def libm():
    build.build(driver=False)
    return _lib.lib()


def test_library_exports_every_declared_symbol(libm):
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(libm, s), s
    assert set(syms) == set(_lib.SIGNATURES), set(syms) ^ set(_lib.SIGNATURES)


def test_config_default_is_reference_config(libm):
    cfg = _lib.Config()
    assert libm.mhdgb_config_default(C.byref(cfg)) == 0
    assert (cfg.nx, cfg.ny, cfg.nz) == (150, 150, 150)
    assert (cfg.x2min, cfg.x2max) == (-1.0, 1.0)
    assert list(cfg.bc) == [1, 1, 2, 2, 1, 1]
    assert cfg.cfl == 0.05


def test_create_rejects_bad_config_before_touching_a_device(libm):
    cfg = _lib.Config()
    libm.mhdgb_config_default(C.byref(cfg))
    h = C.c_void_p()
    for field, value in (("nx", 1), ("gam", 1.0), ("cfl", 0.0), ("precision", 7)):
        bad = _lib.Config.from_buffer_copy(cfg)
        setattr(bad, field, value)
        assert libm.mhdgb_create(C.byref(bad), C.byref(h)) == -1
    bad = _lib.Config.from_buffer_copy(cfg)
    bad.bc[3] = 9
    assert libm.mhdgb_create(C.byref(bad), C.byref(h)) == -1
    bad = _lib.Config.from_buffer_copy(cfg)
    bad.nx, bad.ny, bad.spacing_quirk = 32, 16, 1  # quirk needs nx <= ny, nz
    assert libm.mhdgb_create(C.byref(bad), C.byref(h)) == -1


def test_status_strings(libm):
    for code in range(-7, 1):
        assert libm.mhdgb_status_string(code)
