"""The C-ABI library loads and exports every entry point include/mmh.h declares
(no compute call: this file runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mmh.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mmh_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import build as pkg_build
    import mmh as M
    if not os.path.exists(M.LIB_PATH):
        pkg_build.build()
    return M.lib()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("mmh_create", "mmh_destroy", "mmh_calcdefp", "mmh_multigrid", "mmh_relaxing",
                 "mmh_scalar2gradient", "mmh_defp2delta", "mmh_iterate"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_python_mirror_lists_every_symbol(lib):
    import mmh as M
    assert sorted(M.EXPORTS) == declared_functions()


def test_host_only_calls(lib):
    import mmh as M
    assert M.strerror(-3) == "grid size must be a power of two"
    cfg = M.Config()
    lib.mmh_config_default(C.byref(cfg), 64)
    assert cfg.n == 64 and cfg.nu1 == 2 and cfg.schedule == M.MMH_SCHED_REF
    h = C.c_void_p()
    cfg.n = 24  # rejected before any CUDA call
    assert lib.mmh_create(C.byref(h), C.byref(cfg)) == -3
    cfg.n = 2048
    assert lib.mmh_create(C.byref(h), C.byref(cfg)) == -2
    cfg.n = 64
    cfg.precision, cfg.schedule = M.MMH_MIXED, M.MMH_SCHED_REF
    assert lib.mmh_create(C.byref(h), C.byref(cfg)) == -1
    assert lib.mmh_destroy(None) == 0
