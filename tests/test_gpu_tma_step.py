"""The staged 16-bit fast step (row tiles in shared memory by bulk copies)
against the oracle, bit for bit: single-tile and multi-tile rows (halo wrap
at both row ends), every velocity set (fp16s storage; the other storages take
the plain step, checked the same way)."""
import os

import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from gpu_helpers import make_pair, seeded_fields, step_and_compare

pytestmark = pytest.mark.gpu


@pytest.fixture
def staged(monkeypatch):
    monkeypatch.setenv("BF_TMA_STEP", "1")
    yield


@pytest.mark.parametrize("vs,res,storage,collision,forced", [
    (bf.VelocitySet.D3Q19, (256, 6, 5), bf.FloatingPointAccuracy.fp16s, 1, False),
    (bf.VelocitySet.D3Q19, (512, 4, 3), bf.FloatingPointAccuracy.fp16s, 0, True),
    (bf.VelocitySet.D3Q19, (768, 3, 2), bf.FloatingPointAccuracy.fp16s, 1, True),
    (bf.VelocitySet.D2Q9, (256, 10, 1), bf.FloatingPointAccuracy.fp16s, 0, False),
    (bf.VelocitySet.D3Q15, (256, 4, 4), bf.FloatingPointAccuracy.fp16s, 1, False),
    (bf.VelocitySet.D3Q27, (256, 4, 3), bf.FloatingPointAccuracy.fp16s, 1, False),
])
def test_staged_step_matches_oracle(staged, vs, res, storage, collision, forced, product_lib):
    dims = 2 if vs == bf.VelocitySet.D2Q9 else 3
    rho, u = seeded_fields(res, 7, dims=dims)
    n = res[0] * res[1] * res[2]
    force = None
    if forced:
        force = np.zeros((n, 3), np.float32)
        force[:, 0] = 3e-5
    s, o = make_pair(res, 0.55, vs, density=rho, velocity=u, force=force, storage=storage, collision=collision,
                     esoteric=True)
    step_and_compare(s, o, [1, 2, 5, 12])
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))
