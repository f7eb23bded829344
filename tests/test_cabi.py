"""The C-ABI library loads and exports every symbol declared in include/*.h.

CPU-only: no compute call is made; only argument validation paths that return
before touching the GPU are exercised.
"""
from __future__ import annotations

import ctypes
import re
import subprocess

from conftest import REPO


def _declared_symbols():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"JSCC_API\s+[^;(]*?\b(jscc_\w+)\s*\(", text, flags=re.S))
    return names


def test_header_declares_symbols():
    assert "jscc_sc_weight" in _declared_symbols()


def test_library_exports_every_declared_symbol(lib):
    from jscc_recon_spect_cylinder_gb300 import _lib

    declared = _declared_symbols()
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.library_path())], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (jscc_\w+)$", out, flags=re.M))
    assert declared <= exported, f"declared but not exported: {sorted(declared - exported)}"
    assert exported <= declared, f"exported but not declared: {sorted(exported - declared)}"
    for name in declared:
        assert hasattr(lib, name)
    # the ctypes signature table covers every declared entry point
    assert declared == set(_lib._SIGNATURES)


def test_abi_version_and_counters(lib):
    assert lib.jscc_abi_version() >= 1
    lib.jscc_reset_launch_count()
    assert lib.jscc_launch_count() == 0


def test_invalid_arguments_return_error_without_gpu(lib):
    from jscc_recon_spect_cylinder_gb300 import _lib

    rc = lib.jscc_sc_weight(None, 0, 4, None, 2, 4, None, 1, 0, None, None, None, 0, 0, 0.0, 1.0, None,
                            None, 0, None)
    assert rc == _lib.JSCC_ERR_INVALID
    assert b"n_rot" in lib.jscc_last_error()
    rc = lib.jscc_sc_weight(None, 7, 4, None, 2, 4, None, 1, 1, None, None, None, 0, 0, 0.0, 1.0, None,
                            None, 0, None)
    assert rc == _lib.JSCC_ERR_INVALID
    assert b"dtype" in lib.jscc_last_error()
    # empty problem is a no-op success
    rc = lib.jscc_sc_weight(None, 0, 4, None, 0, 4, None, 1, 1, None, None, None, 0, 0, 0.0, 1.0, None,
                            None, 0, None)
    assert rc == _lib.JSCC_OK
    rc = lib.jscc_em_update(None, None, None, 0, 0.0, None, 0.0, None, 5, 9, 0.0, None)
    assert rc == _lib.JSCC_ERR_INVALID


def test_workspace_bytes_scale(lib):
    small = lib.jscc_sc_weight_workspace_bytes(1024, 4800, 1)
    big = lib.jscc_sc_weight_workspace_bytes(10240, 36000, 1)
    assert 0 < small < big
    # partial sums stay a small fraction of the streamed matrix
    assert big < 0.05 * 10240 * 36000 * 4
