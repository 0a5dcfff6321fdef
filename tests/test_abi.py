"""The C-ABI library builds, loads without a GPU and exports every entry
point that include/rfgpu.h declares (no compute calls here)."""
import ctypes as C
import os
import re

import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import build as rfbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def libpath():
    return rfbuild.build()


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "rfgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rf_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("rf_render", "rf_render_draws", "rf_target_create", "rf_target_clear",
              "rf_target_read", "rf_mesh_upload", "rf_texture_upload", "rf_ctx_create"):
        assert s in syms


def test_library_exports_all_declared(libpath):
    L = C.CDLL(libpath)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_python_bindings_cover_header(libpath):
    bound = set(rf._SIGS) | {"rf_status_str", "rf_ctx_last_error", "rf_obj_free"}
    assert set(declared_symbols()) <= bound, set(declared_symbols()) - bound


def test_rust_binding_covers_header():
    """The Rust -sys crate (retrofire_gb300/rust/rf-gpu-sys) declares every
    entry point of the header, and no other."""
    src = open(os.path.join(ROOT, "retrofire_gb300", "rust", "rf-gpu-sys", "src", "lib.rs")).read()
    bound = set(re.findall(r"\bpub fn (rf_[a-z_0-9]+)\s*\(", src))
    declared = set(declared_symbols())
    assert declared <= bound, sorted(declared - bound)
    assert bound <= declared, sorted(bound - declared)


def test_status_strings(libpath):
    L = rf.lib()
    assert L.rf_status_str(0) == b"ok"
    assert L.rf_status_str(3).startswith(b"texture")
    assert L.rf_ctx_last_error(None) == b""


def test_no_device_reports_status(libpath):
    """Without a visible GPU, rf_ctx_create fails with RF_ERR_NO_DEVICE."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    p = C.c_void_p()
    assert rf.lib().rf_ctx_create(None, C.byref(p)) == 9
    with pytest.raises(rf.RfError):
        rf.Device()


def test_null_arguments_rejected(libpath):
    L = rf.lib()
    assert L.rf_ctx_create(None, None) == 2
    assert L.rf_ctx_destroy(None) == 2
    assert L.rf_render(None, 0, 0, None, None, 0, None, None) == 2


def test_batch_and_server_null_arguments(libpath):
    L = rf.lib()
    assert L.rf_render_batch(None, None, 0, None) == 2
    assert L.rf_ctx_autotune(None, None, 0, 1, None, None, None) == 2
    assert L.rf_ctx_set_graphs(None, 1) == 2
    assert L.rf_ctx_counts(None, None, None, None) == 2
    assert L.rf_mesh_info(None, 1, None, None, None) == 2
    p = C.c_void_p()
    assert L.rf_server_create(None, None, C.byref(p)) == 2
    assert L.rf_server_submit(None, None, None) == 2
    assert L.rf_server_wait(None, 1, 0, None) == 2
    assert L.rf_server_counts(None, None, None, None) == 2
    assert L.rf_server_destroy(None) == 2
