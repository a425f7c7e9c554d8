"""The C ABI: the library builds, loads and exports every entry point the
header declares; on a machine without a GPU its calls fail cleanly."""
import ctypes as C
import os
import re

import pytest

from treeamr import _native

HEADERS = [os.path.join(_native.INCLUDE_DIR, h) for h in os.listdir(_native.INCLUDE_DIR)
           if h.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|void|int32_t|int64_t)\s+\**\s*(tam_\w+)\s*\(", text, re.M):
            names.append(m.group(1))
    return names


def test_header_declares_the_entry_points():
    names = declared_functions()
    for need in ("tam_init", "tam_free", "tam_schedule_upload", "tam_schedule_free",
                 "tam_fill", "tam_fill_plain", "tam_last_error", "tam_device_status"):
        assert need in names


def test_library_exports_every_declared_symbol():
    _native.build()
    lib = _native.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.tam_abi_version() == _native.ABI_VERSION


def test_struct_layout_matches_header():
    # The descriptor structs are the ABI: offsets are plain C layout.
    assert C.sizeof(_native.tam_stencil) == 32
    assert C.sizeof(_native.tam_group) == 24 + 16 + 3 * 32
    assert _native.tam_group.orientation.offset == 16
    assert _native.tam_group.first.offset == 24
    assert _native.tam_schedule_desc.groups.offset == 40
    assert C.sizeof(_native.tam_state_layout) == 56
    assert C.sizeof(_native.tam_boundary_region) == 128
    assert _native.tam_boundary_region.base.offset == 72
    assert C.sizeof(_native.tam_boundary_fn) == 12 + 12 * _native.TAM_BC_MAX_TERMS
    assert _native.tam_state_layout.nblocks.offset == 48
    assert _native.tam_state_layout.ghosts.offset == 32


def test_calls_fail_cleanly_without_arguments():
    lib = _native.lib()
    assert lib.tam_init(0, None) != 0                     # NULL out pointer
    buf = C.create_string_buffer(256)
    assert lib.tam_last_error(None, buf, 256) == 0
    assert b"NULL" in buf.value
    assert lib.tam_fill(None, None, 1, 1, None, -1, 1, None) != 0
    assert lib.tam_schedule_upload(None, None, None) != 0
    assert lib.tam_scatter(None, None, None, None) != 0
    assert lib.tam_gather(None, None, None, None) != 0
    # the adjoint without allocation names a NULL schedule in the last error
    assert lib.tam_fill_adjoint_static(None, None, 1, 1, None, -1, 1, None) == -1
    assert lib.tam_last_error(None, buf, 256) == 0
    assert b"NULL schedule" in buf.value


def test_no_gpu_init_reports_an_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _native.lib()
    ctx = C.c_void_p()
    rc = lib.tam_init(0, C.byref(ctx))
    assert rc != 0
    buf = C.create_string_buffer(256)
    lib.tam_last_error(None, buf, 256)
    assert buf.value
