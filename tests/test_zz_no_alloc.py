"""The allocation-free reduction entry point, bf_reduce_field_noalloc.

Callers such as a renderer's per-frame callback under a fixed device-memory
budget, or code that must not stall other streams (cudaFree synchronizes the
device), cannot allocate; this entry point works from a fixed device array.
Its sums must agree with the allocating reduction, bf_reduce, on two calls
in a row.  This file is collected last so that a run stopping at the first
failure has run every other test already."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_CELLS = 134_217_728


def test_noalloc_reduction_matches_bf_reduce(product_lib):
    import boltzmannfluids_gb300 as bf
    lib = product_lib
    res = (48, 40, 36)
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(17)
    rho = (1 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    u = (0.02 * rng.uniform(-1, 1, (n, 3))).astype(np.float32)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.initialize_fields_from_arrays(res, 0.6, density=rho, velocity=u, velocity_set=bf.VelocitySet.D3Q19)
    s.iterate_time(steps=12, save=False)
    ref = s.reduce()  # allocating path; also refreshes the u/rho field it measured
    s.synchronize()
    ptr, nbytes = s.get_field_device(bf.Field.velocity_density)
    s.synchronize()
    assert nbytes == 16 * n
    outs = []
    for _ in range(2):
        out = (C.c_double * 5)()
        rc = lib.bf_reduce_field_noalloc(C.c_void_p(ptr), n, None, out)
        assert rc == 0, lib.bf_last_error()
        outs.append(np.array(out[:], np.float64))
    for got in outs:
        # FP64 sums of the same FP32 cells in a different blocking order
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-10), (got, ref)
    assert np.array_equal(outs[0], outs[1])  # fixed-order sums: repeatable bit for bit


def test_noalloc_reduction_rejects_oversize(product_lib):
    lib = product_lib
    out = (C.c_double * 5)()
    rc = lib.bf_reduce_field_noalloc(C.c_void_p(1), MAX_CELLS + 1, None, out)
    assert rc == -1 and b"capacity" in lib.bf_last_error()
    assert lib.bf_reduce_field_noalloc(None, 0, None, out) == 0 and list(out) == [0.0] * 5


def test_noalloc_reduction_rejects_misaligned_field(product_lib):
    """A field pointer off a 16-byte boundary is refused before any launch."""
    lib = product_lib
    out = (C.c_double * 5)()
    rc = lib.bf_reduce_field_noalloc(C.c_void_p(8), 1024, None, out)
    assert rc == -1 and b"aligned" in lib.bf_last_error()
