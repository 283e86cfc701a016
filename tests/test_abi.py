"""The C ABI library loads and exports every entry point include/*.h declares.

CPU-only: no compute call is made. Without a GPU the library must refuse to
create a context instead of falling back to the CPU.
"""
import ctypes
import os
import subprocess

import pytest

from leo2d_gb300 import _abi


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_abi.LIB_PATH):
        from leo2d_gb300 import build
        build.build()
    return ctypes.CDLL(_abi.LIB_PATH)


def test_every_declared_symbol_is_exported(lib):
    names = _abi.exported_symbols_from_header()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared in include/ but not exported: {missing}"


def test_exports_are_c_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", _abi.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for n in _abi.exported_symbols_from_header():
        assert n in exported, n  # unmangled: extern "C"


def test_abi_version_and_status_strings(lib):
    L = _abi.load()
    assert L.leo2d_abi_version() == 2
    assert L.leo2d_status_string(0) == b"ok"
    assert b"argument" in L.leo2d_status_string(1)


def test_geom_prepare_is_host_only_and_matches_oracle():
    from oracle import oracle
    L = _abi.load()
    for mn in [(2, 1), (3, 2), (2, 3), (31, 32), (5, 4)]:
        g = _abi.make_geom(boundary_condition=1, supercell_mn=mn, size=20)
        g2 = _abi.make_geom(boundary_condition=1, supercell_mn=mn, size=20)
        assert L.leo2d_geom_prepare(ctypes.byref(g)) == 0
        o = oracle.geom_prepare(g2)
        assert bytes(g) == bytes(o), mn


def test_no_silent_cpu_fallback_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = _abi.load()
    h = ctypes.c_void_p()
    st = L.leo2d_ctx_create(ctypes.byref(h), 0)
    assert st == _abi.ERR_CUDA and not h.value
