"""GPU parity: the sm_103a kernels (through the C ABI) against the CPU
oracle on the same seeded inputs.  Bar: max relative difference <= 1e-5 in
rho and u for the FP32 path (tests/gpu_helpers.py: RTOL, U_FLOOR)."""
import numpy as np
import pytest

from gpu_helpers import RTOL, make_pair, rel_errors, fields_of, seeded_fields, step_and_compare

pytestmark = pytest.mark.gpu

VS = {9: 2, 15: 3, 19: 4, 27: 5}


def grid(q):
    return (40, 24, 1) if q == 9 else (20, 14, 12)


@pytest.fixture(autouse=True)
def _lib(product_lib, oracle_mod):
    yield


@pytest.mark.parametrize("q", [9, 15, 19, 27])
def test_aa_periodic_fast_path(q):
    res = grid(q)
    rho, u = seeded_fields(res, seed=q, dims=2 if q == 9 else 3)
    s, o = make_pair(res, 0.6, VS[q], density=rho, velocity=u)
    step_and_compare(s, o, [1, 2, 3, 10, 60])


@pytest.mark.parametrize("q", [9, 19])
def test_aa_raw_lattice_after_one_and_two_steps(q):
    """The in-place AA slot layout itself matches the reference's addressing."""
    res = grid(q)
    rho, u = seeded_fields(res, seed=7, dims=2 if q == 9 else 3)
    s, o = make_pair(res, 0.7, VS[q], density=rho, velocity=u)
    for k in (1, 1, 5):
        s.iterate_time(steps=k)
        o.iterate(k)
        a = s.get_populations().astype(np.float64)
        b = o.lattice()
        assert np.array_equal(a, b)


@pytest.mark.parametrize("q", [9, 19])
def test_generic_path_equals_fast_path(q):
    """Defining an (unused) object moves the step onto the generic kernel;
    the result must not change by a single bit."""
    import boltzmannfluids_gb300 as bf
    res = grid(q)
    rho, u = seeded_fields(res, seed=11, dims=2 if q == 9 else 3)
    a, _ = make_pair(res, 0.6, VS[q], density=rho, velocity=u)
    b, _ = make_pair(res, 0.6, VS[q], density=rho, velocity=u, objects={1: dict(velocity=(0, 0, 0))})
    assert a.get_bits_per_boundry() == 0 and b.get_bits_per_boundry() == 1
    for n in (1, 1, 20):
        a.iterate_time(steps=n)
        b.iterate_time(steps=n)
        assert np.array_equal(a.get_velocity_density_texture(), b.get_velocity_density_texture())


def test_graph_batches_equal_single_steps():
    res = grid(19)
    rho, u = seeded_fields(res, seed=3)
    a, _ = make_pair(res, 0.6, 4, density=rho, velocity=u)
    b, _ = make_pair(res, 0.6, 4, density=rho, velocity=u)
    a.iterate_time(steps=41)          # captured graphs of 16 steps + direct steps
    for _ in range(41):
        b.iterate_time(steps=1)       # direct launches only
    assert a.get_total_ticks_elapsed() == b.get_total_ticks_elapsed() == 41
    assert np.array_equal(a.get_velocity_density_texture(), b.get_velocity_density_texture())
    assert np.array_equal(a.get_populations(), b.get_populations())


def cylinder_ids(nx, ny, cx, cy, r, wall_top=False):
    y, x = np.mgrid[0:ny, 0:nx]
    ids = np.zeros((ny, nx), np.uint32)
    ids[(x - cx) ** 2 + (y - cy) ** 2 < r * r] = 1
    if wall_top:
        ids[-1, :] = 2
    return ids


@pytest.mark.parametrize("mode", [0, 1])
def test_aa_solids_open_boundaries(mode):
    """Non-periodic x (0.01 open-boundary reads, dropped writes), a solid
    cylinder and a moving wall; mode 0 = skip as read, 1 = bounce-back."""
    nx, ny = 48, 32
    ids = cylinder_ids(nx, ny, 16, 16, 5, wall_top=True)
    rho, u = seeded_fields((nx, ny, 1), seed=5, rho_amp=0.001, u_amp=0.01, dims=2)
    u[:, 0] += 0.04
    objs = {1: dict(velocity=(0, 0, 0)), 2: dict(velocity=(0.05, 0, 0))}
    s, o = make_pair((nx, ny, 1), 0.62, 2, density=rho, velocity=u, ids=ids, objects=objs,
                     periodic=(False, True, True), boundary_mode=mode)
    fluid = ids.reshape(-1) == 0
    step_and_compare(s, o, [1, 2, 5, 40, 150], mask=fluid)
    assert np.array_equal(s.get_boundry_texture().reshape(-1), ids.reshape(-1).astype(np.uint8))


def lid_cavity(n):
    ids = np.zeros((n, n), np.uint32)
    ids[0, :] = 1
    ids[:, 0] = 1
    ids[:, -1] = 1
    ids[-1, :] = 2
    return ids, {1: dict(velocity=(0, 0, 0)), 2: dict(velocity=(0.1, 0, 0))}


def test_lid_driven_cavity_256_steps_1_100_10000():
    """D2Q9 BGK lid-driven cavity, 256x256, tau 0.6, lid u=(0.1,0) by
    moving-wall bounce-back: fields at steps 1, 100 and 10,000."""
    ids, objs = lid_cavity(256)
    s, o = make_pair((256, 256, 1), 0.6, 2, ids=ids, objects=objs, periodic=(False, False, True),
                     boundary_mode=1)
    fluid = ids.reshape(-1) == 0
    step_and_compare(s, o, [1, 100, 10000], mask=fluid)


def test_two_buffer_modes():
    ids, objs = lid_cavity(40)
    fluid = ids.reshape(-1) == 0
    for fixed in (False, True):
        s, o = make_pair((40, 40, 1), 0.6, 2, ids=ids, objects=objs, periodic=(False, False, True),
                         esoteric=False, two_buffer_fixed=fixed)
        step_and_compare(s, o, [1, 2, 7, 50], mask=fluid)


@pytest.mark.parametrize("field", [False, True])
def test_guo_forcing(field):
    res = (24, 16, 10)
    rho, u = seeded_fields(res, seed=21)
    n = res[0] * res[1] * res[2]
    f = np.zeros((n, 3), np.float32)
    f[:, 0] = 1e-5
    if field:
        f[:, 1] = np.linspace(-2e-5, 2e-5, n)
    s, o = make_pair(res, 0.58, 4, density=rho, velocity=u, force=f)
    assert s.get_is_forcing_scheme() and s.get_is_force_field_constant() == (not field)
    step_and_compare(s, o, [1, 3, 40])


def test_velocity_limiter_paths():
    """Cells above velocity_limit get u scaled; above the extreme limit the
    populations are reset to equilibrium (collide.comp:722-742)."""
    res = (32, 16, 1)
    rho, u = seeded_fields(res, seed=2, dims=2)
    u[:, 0] = np.linspace(0.0, 0.4, u.shape[0])
    s, o = make_pair(res, 0.7, 2, density=rho, velocity=u)
    step_and_compare(s, o, [1, 2, 10])


@pytest.mark.parametrize("storage,collision,q,res,field", [
    (2, 0, 2, (32, 16, 1), False), (3, 1, 4, (24, 10, 8), False), (2, 1, 4, (24, 10, 8), False),
    (3, 0, 4, (24, 10, 8), True), (2, 1, 2, (32, 16, 1), True)])
def test_velocity_limiter_paths_16bit_forced(storage, collision, q, res, field):
    """The limiter and the extreme-velocity equilibrium of the shifted 16-bit
    storages with a source term (the folded collision with omega = 1 and no
    source above the extreme limit): a uniform force (the two-cell kernel)
    and a force field (the generic kernel)."""
    n = res[0] * res[1] * res[2]
    rho, u = seeded_fields(res, seed=3, dims=2 if res[2] == 1 else 3)
    u[:, 0] = np.linspace(0.0, 0.4, n)
    force = np.zeros((n, 3), np.float32)
    force[:, 1] = 1e-5 * (1.0 + (np.arange(n) % 7 if field else 0))
    s, o = make_pair(res, 0.7, q, density=rho, velocity=u, force=force, storage=storage, collision=collision)
    step_and_compare(s, o, [1, 2, 10])
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))


def test_trt_collision():
    res = (20, 16, 12)
    rho, u = seeded_fields(res, seed=8)
    s, o = make_pair(res, 0.55, 4, density=rho, velocity=u, collision=1, trt_magic=0.25)
    step_and_compare(s, o, [1, 2, 30])


@pytest.mark.parametrize("bb", [0, 1])
@pytest.mark.parametrize("q", [9, 19])
def test_thermal_lattice(q, bb):
    """Thermal D2Q5/D3Q7 lattice with Dirichlet walls (stream_thermal.comp)
    and Boussinesq buoyancy; both the as-read zero start and the equilibrium
    start; walls skipped as read (bb 0) or under bounce-back (bb 1, where the
    thermal stream takes its sources from the flow lattice's masks)."""
    res = (32, 24, 1) if q == 9 else (16, 14, 10)
    nx, ny, nz = res
    ids = np.zeros((nz, ny, nx), np.uint32)
    ids[:, 0, :] = 1
    ids[:, -1, :] = 2
    objs = {1: dict(temperature=1.5), 2: dict(temperature=0.5)}
    f = np.zeros((nx * ny * nz, 3), np.float32)
    f[:, 1] = -1e-4
    fluid = ids.reshape(-1) == 0
    for eq in (False, True):
        s, o = make_pair(res, 0.6, VS[q], ids=ids, objects=objs, force=f, periodic=(True, False, True),
                         thermal_init_equilibrium=eq, tau_t=0.8, beta=0.5, boundary_mode=bb)
        assert s.get_is_flow_thermal()
        step_and_compare(s, o, [1, 2, 25, 80], mask=fluid, check_temperature=True)


@pytest.mark.parametrize("q", [9, 19])
def test_shan_chen(q):
    res = (32, 32, 1) if q == 9 else (16, 16, 16)
    rng = np.random.default_rng(4)
    n = res[0] * res[1] * res[2]
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    s, o = make_pair(res, 1.0, VS[q], density=rho, multiphase=True, G=-5.0)
    # psi = 1 - exp(-rho) uses the same hand-written exp on both sides
    step_and_compare(s, o, [1, 2, 20, 60])


@pytest.mark.parametrize("storage", [1, 2, 3])
def test_16bit_storage_matches_emulation(storage):
    """16-bit storage: the oracle emulates the same codecs (IEEE half RNE of
    f or of f - w, and the half of (f - w) * 2^12); with FP32
    arithmetic identical on both sides the stored lattices agree bit for bit."""
    res = (20, 14, 12)
    rho, u = seeded_fields(res, seed=31)
    s, o = make_pair(res, 0.6, 4, density=rho, velocity=u, storage=storage)
    a0 = s.get_populations().astype(np.float64)
    b0 = o.lattice()
    assert np.array_equal(a0, b0)  # identical encoding of the initial state
    for k in (1, 1, 10):
        s.iterate_time(steps=k)
        o.iterate(k)
        assert np.array_equal(s.get_populations().astype(np.float64), o.lattice())


def test_equilibrium_boundaries_inlet_outlet():
    """Extension: velocity inlet at x=0 and density outlet at x=nx-1 (objects
    of the equilibrium kinds), solid obstacle, TRT."""
    nx, ny, nz = 32, 16, 12
    ids = np.zeros((nz, ny, nx), np.uint32)
    ids[:, :, 0] = 1
    ids[:, :, -1] = 2
    z, y, x = np.mgrid[0:nz, 0:ny, 0:nx]
    ids[(x - 10) ** 2 + (y - 8) ** 2 + (z - 6) ** 2 < 9] = 3
    objs = {1: dict(kind=1), 2: dict(kind=2), 3: dict()}
    n = nx * ny * nz
    u = np.zeros((n, 3), np.float32)
    u[:, 0] = 0.05
    rho = np.ones(n, np.float32)
    s, o = make_pair((nx, ny, nz), 0.55, 4, density=rho, velocity=u, ids=ids, objects=objs,
                     periodic=(False, True, True), boundary_mode=1, collision=1)
    fluid = ids.reshape(-1) != 3
    step_and_compare(s, o, [1, 2, 30, 100], mask=fluid)


def test_reduction_matches_oracle():
    res = (24, 20, 16)
    rho, u = seeded_fields(res, seed=9)
    s, o = make_pair(res, 0.6, 4, density=rho, velocity=u)
    s.iterate_time(steps=5, save=True)
    o.iterate(5, True)
    got = s.reduce()
    # the oracle sums the saved fields in FP64; reduce() measures the state the
    # next step reads, so step the oracle's saved fields forward by a measure:
    o2_vd, _ = o.fields()
    vd, _ = fields_of(s)  # reduce() refreshed the saved fields
    n = vd.shape[0]
    exp = np.array([vd[:, 3].sum(), (vd[:, 3] * vd[:, 0]).sum(), (vd[:, 3] * vd[:, 1]).sum(),
                    (vd[:, 3] * vd[:, 2]).sum(), (0.5 * vd[:, 3] * (vd[:, :3] ** 2).sum(1)).sum()])
    assert np.allclose(got, exp, rtol=1e-6, atol=1e-9)
    assert abs(got[0] - o2_vd[:, 3].sum()) < 1e-4 * n
    again = s.reduce()
    assert np.array_equal(got, again)  # deterministic fixed-order FP64 sums


def test_snapshot_round_trip(tmp_path):
    res = (20, 14, 12)
    rho, u = seeded_fields(res, seed=12)
    s, _ = make_pair(res, 0.6, 4, density=rho, velocity=u)
    s.iterate_time(steps=7)
    p = tmp_path / "snap.bin"
    s.save_current_tick_mesoscropic(p)
    s.iterate_time(steps=9)
    ref = s.get_populations().copy()
    t9 = s.get_total_ticks_elapsed()
    s.load_tick_mesoscropic(p)
    assert s.get_total_ticks_elapsed() == 7
    s.iterate_time(steps=9)
    assert s.get_total_ticks_elapsed() == t9
    assert np.array_equal(s.get_populations(), ref)


def test_nan_density_reports_unstable_status():
    """A NaN planted in the host-side initial density surfaces as
    BF_ERR_UNSTABLE from synchronize (no device fault involved)."""
    import boltzmannfluids_gb300 as bf
    res = (16, 8, 1)
    rho = np.ones(res[0] * res[1], np.float32)
    rho[5] = np.nan
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.initialize_fields_from_arrays(res, 0.6, density=rho, velocity_set=bf.VelocitySet.D2Q9)
    s.iterate_time(steps=2)
    with pytest.raises(bf.LBMError) as e:
        s.synchronize()
    assert e.value.code == -5


def test_invalid_arguments_are_rejected():
    import boltzmannfluids_gb300 as bf
    s = bf.LBM()
    with pytest.raises(bf.LBMError):
        s.initialize_fields_from_arrays((8, 8, 2), 0.6, velocity_set=bf.VelocitySet.D2Q9)
    with pytest.raises(bf.LBMError):
        s.initialize_fields_from_arrays((0, 8, 1), 0.6)
    with pytest.raises(bf.LBMError):
        s.set_boundry_properties(0, (0, 0, 0))
    with pytest.raises(bf.LBMError):
        s.set_boundry_properties(256, (0, 0, 0))
    with pytest.raises(bf.LBMError):
        s.iterate_time(steps=1)  # not initialised


def test_lambda_initialisation_matches_arrays():
    """initialize_fields with a per-cell lambda, as the reference's API."""
    import boltzmannfluids_gb300 as bf
    res = (12, 10, 1)

    def init(c, p):
        x, y, _ = c
        p.velocity = (0.01 * np.sin(x), 0.0, 0.0)
        p.density = 1.0 + 0.001 * y
        if y == 0:
            p.boundry_id = 1

    a = bf.LBM()
    a.is_collide_esoteric = True
    a.set_boundry_properties(1, (0.0, 0.0, 0.0))
    a.initialize_fields(init, res, 0.6, True, False, True, bf.VelocitySet.D2Q9)
    b = bf.LBM()
    b.is_collide_esoteric = True
    b.set_boundry_properties(1, (0.0, 0.0, 0.0))
    y, x = np.mgrid[0:res[1], 0:res[0]]
    u = np.zeros((res[1], res[0], 3), np.float32)
    u[..., 0] = 0.01 * np.sin(x)
    ids = (y == 0).astype(np.uint32)
    b.initialize_fields_from_arrays(res, 0.6, density=1.0 + 0.001 * y, velocity=u, boundry_id=ids,
                                    periodic=(True, False, True), velocity_set=bf.VelocitySet.D2Q9)
    a.iterate_time(steps=5)
    b.iterate_time(steps=5)
    assert np.array_equal(a.get_velocity_density_texture(), b.get_velocity_density_texture())


def test_pseudopotential_exp_against_cuda_expf():
    """The kernels' hand-written exp in psi = 1 - exp(-rho): bit-exact with the
    oracle's, and within a few ulp of CUDA's expf (through torch) over the
    densities of a Shan-Chen flow, rho in [0.01, 10]."""
    import torch
    import boltzmannfluids_gb300 as bf
    from oracle import oracle as orc
    res = (256, 40, 1)
    n = res[0] * res[1]
    rho = np.linspace(0.01, 10.0, n).astype(np.float32)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.intermolecular_interaction_strength = -5.0
    s.initialize_fields_from_arrays(res, 1.0, density=rho, velocity_set=bf.VelocitySet.D2Q9, is_flow_multiphase=True)
    d = s.get_velocity_density_texture().reshape(-1, 4)[:, 3]  # the densities psi was formed from
    psi = s.get_pseudopotential().reshape(-1)
    lib = orc.load()
    e_orc = np.array([lib.orc32_exp_f32(float(-r)) for r in d], np.float32)
    assert np.array_equal(psi, (np.float32(1.0) - e_orc).astype(np.float32))
    dt = torch.from_numpy(d.copy()).cuda()
    e_cuda = torch.exp(-dt)
    psi_cuda = (1.0 - e_cuda).cpu().numpy()
    e_cuda = e_cuda.cpu().numpy()
    bound = 4 * np.spacing(e_cuda) + 2 * np.spacing(psi_cuda)
    assert (np.abs(psi - psi_cuda) <= bound).all()
    assert (np.abs(e_orc - e_cuda) <= 2 * np.spacing(e_cuda)).all()
