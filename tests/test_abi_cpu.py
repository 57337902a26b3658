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


def test_z_chunk_planner(libm):
    """The host-side z-chunk planner of the fused step's work queue: chunks cover every plane once,
    stay within the kernel's chunk table, and at the benchmark sizes are the chunkings the measured
    runs used (16x8 tiles; 304 CTAs for the mixed form, 152 for FP64)."""
    def plan(n, ctas, nz=None):
        buf = (C.c_int * 64)()
        k = libm.mhdgb_plan_zchunks(n, n, nz or n, 16, 8, ctas, buf, 64)
        assert k > 0, (n, ctas, k)
        return list(buf[:k])

    assert plan(150, 304) == [91, 36, 15, 6, 2]
    assert plan(150, 152) == [91, 36, 15, 6, 2]
    assert plan(256, 304) == [216, 34, 6]
    assert plan(512, 304) == [384, 128]
    for n in (2, 9, 33, 64, 97, 150, 257, 512, 1000):
        for ctas in (152, 304):
            for nz in (n, 3, 2 * n + 1):
                c = plan(n, ctas, nz)
                assert sum(c) == nz and min(c) >= 1 and len(c) <= 64, (n, ctas, nz, c)
    small = (C.c_int * 2)()
    assert libm.mhdgb_plan_zchunks(150, 150, 150, 16, 8, 304, small, 2) == -1  # needs 5 entries
    for bad in ((0, 8, 8, 16, 8, 152), (8, 8, 8, 0, 8, 152), (8, 8, 8, 16, 8, 0)):
        assert libm.mhdgb_plan_zchunks(*bad, small, 2) == -1
