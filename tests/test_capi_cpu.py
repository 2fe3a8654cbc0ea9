"""C ABI checks that need no GPU: the library loads, exports every entry point
include/compute_c.h declares, and behaves as the reference's C interface does
without a device (lib/test/Compute/capi.c:51-62, CApi.cpp:228-283)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "compute_c.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GBC_EXPORT\s+[\w\s\*]+?\b(clc_\w+)\s*\(", text)))


def test_header_declares_reference_entry_points():
    names = set(declared_symbols())
    # every function of the reference C interface (compute_c.h:64-202)
    reference = {
        "clc_last_error", "clc_last_cl_error", "clc_device_count", "clc_device_get_info", "clc_context_create",
        "clc_context_create_with_cache", "clc_context_release", "clc_context_get_info", "clc_finish",
        "clc_buffer_alloc", "clc_buffer_release", "clc_buffer_size", "clc_buffer_write", "clc_buffer_read",
        "clc_buffer_copy", "clc_file_size", "clc_file_read", "clc_file_write", "clc_fill", "clc_sequence",
        "clc_transform", "clc_transform2", "clc_reduce", "clc_scan", "clc_sort", "clc_copy_if", "clc_add_header",
        "clc_kernel_create", "clc_kernel_release", "clc_kernel_set_buffer", "clc_kernel_set_value",
        "clc_kernel_set_local", "clc_kernel_work_group_size", "clc_kernel_launch",
    }
    assert reference <= names


def test_library_exports_every_declared_symbol(gbc):
    nm = subprocess.run(["nm", "-D", "--defined-only", gbc.LIBRARY_PATH], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\s[TW]\s+(\w+)$", nm.stdout, re.M))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    # and the binding binds exactly those
    assert set(gbc.EXPORTED_SYMBOLS) == set(declared_symbols())
    # nothing else of the implementation leaks out
    leaked = sorted(s for s in exported if s.startswith("_ZN3gbc"))
    assert not leaked, leaked[:5]


def test_header_compiles_as_c99(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "compute_c.h"\nint main(void){ clc_status s = CLC_SUCCESS; clc_type t = CLC_TYPE_F64;'
                   ' return (int)s + (int)t - 9 + (CLC_ERROR_IO - 8) + (CLC_DEFAULT_DEVICE != (size_t)-1); }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src),
                    "-o", str(tmp_path / "t")], check=True)
    assert subprocess.run([str(tmp_path / "t")]).returncode == 0


def test_enum_values_match_reference(gbc):
    # compute_c.h:30-56 of the reference
    assert (gbc.SUCCESS, gbc.ERROR_OPENCL, gbc.ERROR_INVALID_ARGUMENT, gbc.ERROR_BUILD, gbc.ERROR_NO_DEVICE,
            gbc.ERROR_OUT_OF_MEMORY, gbc.ERROR_UNSUPPORTED, gbc.ERROR_INTERNAL, gbc.ERROR_IO) == tuple(range(9))
    assert (gbc.TYPE_I8, gbc.TYPE_F64) == (0, 9)


def test_null_arguments_and_stubs(gbc):
    L = gbc.lib
    assert L.clc_device_count(None) == gbc.ERROR_INVALID_ARGUMENT
    assert len(L.clc_last_error()) > 0
    assert L.clc_context_create(0, None) == gbc.ERROR_INVALID_ARGUMENT
    assert L.clc_finish(None) == gbc.ERROR_INVALID_ARGUMENT
    L.clc_buffer_release(None)  # no-op
    L.clc_context_release(None)
    assert L.clc_buffer_size(None) == 0
    assert L.clc_transform(None, None, 4, None, 8, 10, b"(float)x") == gbc.ERROR_INVALID_ARGUMENT
    assert L.clc_transform2(None, None, 4, None, 4, None, 4, 10, b"x + y") == gbc.ERROR_INVALID_ARGUMENT
    # out-of-scope entry points link and report UNSUPPORTED
    done = C.c_size_t(7)
    assert L.clc_file_read(None, b"x", 0, None, 0, 0, C.byref(done)) == gbc.ERROR_UNSUPPORTED and done.value == 0
    k = C.c_void_p(1)
    assert L.clc_kernel_create(None, b"", b"", None, None, None, 0, C.byref(k)) == gbc.ERROR_UNSUPPORTED
    assert k.value is None


def test_no_device_behaviour(gbc):
    if gbc.device_count() > 0:
        pytest.skip("a GPU is visible: covered by the gpu tests")
    n = C.c_size_t(99)
    assert gbc.lib.clc_device_count(C.byref(n)) == gbc.SUCCESS and n.value == 0
    h = C.c_void_p()
    assert gbc.lib.clc_context_create(gbc.DEFAULT_DEVICE, C.byref(h)) == gbc.ERROR_NO_DEVICE
    assert h.value is None
    with pytest.raises(gbc.NoDeviceError):
        gbc.Context()


def test_tuning_keys(gbc):
    assert gbc.tuning_sort_key(4, False, 1 << 28) == "sort:u32k:2^28"
    assert gbc.tuning_sort_key(8, True, (1 << 20) + 1) == "sort:u64kv:2^21"
    assert gbc.tuning_sort_variants(4, True) >= 2
    assert gbc.tuning_sort_variants(3, True) == 0
