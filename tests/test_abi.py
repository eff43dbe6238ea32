"""The C-ABI library builds, loads and exports every symbol include/nfx.h declares. No compute
calls are made here, so this runs without a GPU."""

import ctypes as C

from nofluidx3d_gb300 import _lib


def test_exports_every_declared_symbol(nfx_lib):
    declared = _lib.header_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if not hasattr(nfx_lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(_lib.header_symbols()) == set(_lib._SIGS)


def test_version_and_error_calls(nfx_lib):
    assert nfx_lib.nfx_version() >= 100
    buf = C.create_string_buffer(64)
    assert nfx_lib.nfx_last_error(buf, 64) == 0
    # argument checks happen before any device work
    assert nfx_lib.nfx_create(0, None) == 1
    assert nfx_lib.nfx_step(None, 1) == 1
    assert "null" in _lib.last_error()
