"""The C-ABI library loads without a GPU, exports every entry point that
include/*.h declares, and fails cleanly (status codes, no crash) where a
device is required but absent."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(bf_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_lbm_api():
    names = declared_symbols()
    for must in ("bf_create", "bf_destroy", "bf_initialize_fields", "bf_iterate_time", "bf_get_field",
                 "bf_copy_field_to_host", "bf_set_boundry_properties", "bf_clear_boundry_properties",
                 "bf_reduce", "bf_last_error", "bf_save_snapshot", "bf_load_snapshot"):
        assert must in names


def test_library_exports_every_declared_symbol(product_lib):
    lib = C.CDLL(os.path.join(ROOT, "boltzmannfluids_gb300", "libbfgb300.so"))
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "boltzmannfluids_gb300", "libbfgb300.so")],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bf_\w+)", out))
    assert declared_symbols() <= exported


def test_python_mirror_binds_every_symbol(product_lib):
    from boltzmannfluids_gb300.lbm import ABI
    assert declared_symbols() == set(ABI)


def test_no_device_is_an_error_status(product_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    import boltzmannfluids_gb300 as bf
    with pytest.raises(bf.LBMError) as e:
        bf.LBM()
    assert e.value.code == -8


def test_null_and_invalid_arguments(product_lib):
    lib = product_lib
    assert lib.bf_create(None) == -1
    assert lib.bf_destroy(None) == 0
    assert lib.bf_iterate_time(None, 1, 0) == -1
    assert b"NULL" in lib.bf_last_error()
    n = C.c_int32()
    assert lib.bf_get_velosity_vectors(7, 0, None, C.byref(n)) == -1
    w = C.c_size_t()
    assert lib.bf_pack_boundries(None, 10, 3, None, 0, C.byref(w)) == -1
    # the allocation-free reduction refuses a misaligned field before touching the device
    out = (C.c_double * 5)()
    assert lib.bf_reduce_field_noalloc(C.c_void_p(8), 1024, None, out) == -1
    assert b"aligned" in lib.bf_last_error()
