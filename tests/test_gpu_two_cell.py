"""The 16-bit fast step with two cells per thread against the oracle, bit
for bit: paired 32-bit moves of the c_x = 0 directions, 16-bit moves of the
others, x wrap at both row ends, rows on and off the y/z faces, block widths from
one warp to rows of several blocks."""
import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from gpu_helpers import make_pair, seeded_fields, step_and_compare

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("vs,res,storage,collision,forced", [
    (bf.VelocitySet.D3Q19, (24, 20, 16), bf.FloatingPointAccuracy.fp16s, 1, False),
    (bf.VelocitySet.D3Q19, (2, 6, 5), bf.FloatingPointAccuracy.fp16s, 0, True),
    (bf.VelocitySet.D3Q19, (34, 3, 4), bf.FloatingPointAccuracy.fp16c, 1, True),
    (bf.VelocitySet.D3Q15, (16, 12, 10), bf.FloatingPointAccuracy.fp16c, 0, False),
    (bf.VelocitySet.D2Q9, (40, 24, 1), bf.FloatingPointAccuracy.fp16s, 1, True),
    (bf.VelocitySet.D2Q9, (4, 8, 1), bf.FloatingPointAccuracy.fp16c, 0, False),
    # rows of several blocks (the last one partly filled) and a block of 96 threads
    (bf.VelocitySet.D3Q19, (600, 3, 2), bf.FloatingPointAccuracy.fp16s, 1, False),
    (bf.VelocitySet.D3Q19, (170, 6, 4), bf.FloatingPointAccuracy.fp16c, 1, True),
])
def test_two_cell_step_matches_oracle(vs, res, storage, collision, forced, product_lib):
    dims = 2 if vs == bf.VelocitySet.D2Q9 else 3
    rho, u = seeded_fields(res, 11, dims=dims)
    n = res[0] * res[1] * res[2]
    force = None
    if forced:
        force = np.zeros((n, 3), np.float32)
        force[:, 1] = -2e-5
    s, o = make_pair(res, 0.56, vs, density=rho, velocity=u, force=force, storage=storage, collision=collision,
                     esoteric=True)
    step_and_compare(s, o, [1, 2, 3, 8, 17])
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))


def test_two_cell_equals_one_cell(monkeypatch, product_lib):
    res = (64, 12, 10)
    rho, u = seeded_fields(res, 12)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("BF_TWO_CELL", flag)
        s, _ = make_pair(res, 0.55, bf.VelocitySet.D3Q19, density=rho, velocity=u,
                         storage=bf.FloatingPointAccuracy.fp16s, collision=1, esoteric=True)
        s.iterate_time(steps=33, save=True)
        out.append(s.get_populations())
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("vs,res,storage,collision", [
    (bf.VelocitySet.D3Q19, (24, 20, 16), bf.FloatingPointAccuracy.fp16s, 0),
    (bf.VelocitySet.D3Q19, (34, 6, 4), bf.FloatingPointAccuracy.fp16c, 0),
    (bf.VelocitySet.D2Q9, (40, 24, 1), bf.FloatingPointAccuracy.fp16s, 0),
    # three weight classes in the grouped stencil sum; TRT with the folded source term
    (bf.VelocitySet.D3Q27, (14, 8, 6), bf.FloatingPointAccuracy.fp16c, 0),
    (bf.VelocitySet.D3Q15, (16, 10, 8), bf.FloatingPointAccuracy.fp16s, 1),
    # rows of several blocks, the last one partly filled
    (bf.VelocitySet.D3Q19, (600, 3, 4), bf.FloatingPointAccuracy.fp16s, 1),
])
def test_two_cell_shan_chen_matches_oracle(vs, res, storage, collision, product_lib):
    """The pseudopotential force per cell of the pair: psi of the previous
    step at the neighbours, loaded once per pair, with the x wrap of each cell."""
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(31)
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    s, o = make_pair(res, 1.0, vs, density=rho, storage=storage, multiphase=True, G=-5.0, esoteric=True,
                     collision=collision)
    step_and_compare(s, o, [1, 2, 3, 8, 17])
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))


@pytest.mark.parametrize("storage,collision", [(bf.FloatingPointAccuracy.fp16s, 0), (bf.FloatingPointAccuracy.fp16c, 1)])
def test_shan_chen_16bit_generic_step_matches_oracle(storage, collision, product_lib):
    """16-bit Shan-Chen through the generic step (open y faces: out-of-domain
    neighbours take the cell's own psi) against the oracle, bit for bit."""
    res = (18, 12, 10)
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(34)
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    s, o = make_pair(res, 1.0, bf.VelocitySet.D3Q19, density=rho, storage=storage, multiphase=True, G=-5.0,
                     esoteric=True, collision=collision, periodic=(True, False, True))
    step_and_compare(s, o, [1, 2, 3, 8, 17])
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))


@pytest.mark.parametrize("storage,two_cell,periodic", [
    (bf.FloatingPointAccuracy.fp16s, "1", (True, True, True)),
    (bf.FloatingPointAccuracy.fp16c, "0", (True, True, True)),
    (bf.FloatingPointAccuracy.fp16c, "1", (True, False, True)),  # the generic step (open y faces)
])
def test_shan_chen_16bit_clamped_and_extreme_cells_match_oracle(storage, two_cell, periodic, monkeypatch,
                                                                product_lib):
    """The mass-conserving rounding where the density is clamped to 0.01 (the
    stored populations carry the clamped density's mass) and above the extreme
    velocity limit (the equilibrium), in the two-cell, one-cell and generic
    steps, against the oracle, bit for bit."""
    monkeypatch.setenv("BF_TWO_CELL", two_cell)
    res = (20, 12, 10)
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(35)
    # blocks, not single cells: a cell collides with what streams in from its
    # neighbours (27 cells clamped at step 1, 182 at the velocity limit)
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32).reshape(res[2], res[1], res[0])
    rho[2:7, 3:8, 2:7] = 0.004
    u = np.zeros((res[2], res[1], res[0], 3), np.float32)
    u[2:7, 3:8, 11:16, 0] = 0.4
    s, o = make_pair(res, 1.0, bf.VelocitySet.D3Q19, density=rho.reshape(-1), velocity=u.reshape(-1, 3),
                     storage=storage, multiphase=True, G=-5.0, esoteric=True, periodic=periodic)
    step_and_compare(s, o, [1, 2, 3])
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))


@pytest.mark.parametrize("storage,collision,tau", [(bf.FloatingPointAccuracy.fp16s, 0, 1.0),
                                                   (bf.FloatingPointAccuracy.fp16c, 1, 0.8)])
def test_shan_chen_16bit_with_objects_matches_oracle(storage, collision, tau, product_lib):
    """16-bit Shan-Chen with a velocity inlet and a density outlet (equilibrium
    objects: the rounding's target is the prescribed density's mass) and a
    solid obstacle under bounce-back, through the generic step, against the
    oracle, bit for bit."""
    nx, ny, nz = 24, 12, 10
    ids = np.zeros((nz, ny, nx), np.uint32)
    ids[:, :, 0] = 1
    ids[:, :, -1] = 2
    z, y, x = np.mgrid[0:nz, 0:ny, 0:nx]
    ids[(x - 9) ** 2 + (y - 6) ** 2 + (z - 5) ** 2 < 6] = 3
    objs = {1: dict(kind=1), 2: dict(kind=2), 3: dict()}
    n = nx * ny * nz
    rng = np.random.default_rng(36)
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    u = np.zeros((n, 3), np.float32)
    u[:, 0] = 0.02
    s, o = make_pair((nx, ny, nz), tau, bf.VelocitySet.D3Q19, density=rho, velocity=u, ids=ids.reshape(-1),
                     objects=objs, periodic=(False, True, True), boundary_mode=1, collision=collision,
                     storage=storage, multiphase=True, G=-5.0, esoteric=True)
    fluid = ids.reshape(-1) != 3
    step_and_compare(s, o, [1, 2, 3, 8, 17], mask=fluid)


def test_two_cell_shan_chen_equals_one_cell(monkeypatch, product_lib):
    res = (64, 12, 10)
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(32)
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("BF_TWO_CELL", flag)
        s, _ = make_pair(res, 1.0, bf.VelocitySet.D3Q19, density=rho, storage=bf.FloatingPointAccuracy.fp16s,
                         multiphase=True, G=-5.0, esoteric=True)
        s.iterate_time(steps=33, save=True)
        out.append((s.get_populations(), s.get_velocity_density_texture().copy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("vs,res,storage", [
    (bf.VelocitySet.D3Q19, (24, 20, 16), bf.FloatingPointAccuracy.fp16s),
    (bf.VelocitySet.D3Q19, (512, 3, 4), bf.FloatingPointAccuracy.fp16c),   # the widest row one block stages
    (bf.VelocitySet.D3Q15, (36, 6, 4), bf.FloatingPointAccuracy.fp16s),
    (bf.VelocitySet.D2Q9, (40, 24, 1), bf.FloatingPointAccuracy.fp16s),
    # rows the bulk copies cannot stage (several blocks; nx % 4 != 0): the cached-load kernel
    (bf.VelocitySet.D3Q19, (600, 3, 4), bf.FloatingPointAccuracy.fp16c),
    (bf.VelocitySet.D3Q15, (34, 6, 4), bf.FloatingPointAccuracy.fp16s),
])
def test_two_cell_shan_chen_psi_tile_matches_oracle(vs, res, storage, monkeypatch, product_lib):
    """The Shan-Chen step with the psi rows staged in shared memory by bulk
    copies (BF_PSI_TILE=1; the x wrap inside the staged row) against the
    oracle, bit for bit, and the fallback where a row cannot be staged."""
    monkeypatch.setenv("BF_PSI_TILE", "1")
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(33)
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    s, o = make_pair(res, 1.0, vs, density=rho, storage=storage, multiphase=True, G=-5.0, esoteric=True)
    step_and_compare(s, o, [1, 2, 3, 8, 17])
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))
