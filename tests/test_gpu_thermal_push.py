"""The thermal pull stream folded into the thermal collision as a push
(split boundary-aware step, bounce-back walls): the thermal populations after
each step against the oracle's (collision then stream), bit for bit, and
against the solver's own separate stream pass."""
import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from gpu_helpers import make_pair, step_and_compare

pytestmark = pytest.mark.gpu

VS = {9: bf.VelocitySet.D2Q9, 19: bf.VelocitySet.D3Q19}


def walls_case(q):
    """Hot floor and cold lid (solid walls at z = 0 / nz-1, or y in 2D), a
    solid block in the middle, open x faces, a temperature perturbation."""
    res = (36, 20, 1) if q == 9 else (28, 16, 14)
    nx, ny, nz = res
    ids = np.zeros((nz, ny, nx), np.uint32)
    if q == 9:
        ids[:, 0, :] = 1
        ids[:, -1, :] = 2
    else:
        ids[0] = 1
        ids[-1] = 2
    ids[:, ny // 2 - 2:ny // 2 + 2, nx // 2 - 2:nx // 2 + 2] = 3
    n = nx * ny * nz
    rng = np.random.default_rng(41)
    temp = (0.5 + 0.05 * rng.uniform(-1, 1, n)).astype(np.float32)
    u = np.zeros((n, 3), np.float32)
    u[:, 0] = 0.02
    f = np.zeros((n, 3), np.float32)
    f[:, 1 if q == 9 else 2] = -1e-4
    objs = {1: dict(temperature=1.0), 2: dict(temperature=0.0), 3: dict(temperature=0.7)}
    return res, ids.reshape(-1), temp, u, f, objs


@pytest.mark.parametrize("eq", [False, True])
@pytest.mark.parametrize("q", [9, 19])
def test_thermal_push_matches_oracle(q, eq):
    res, ids, temp, u, f, objs = walls_case(q)
    s, o = make_pair(res, 0.6, VS[q], ids=ids, objects=objs, force=f, temperature=temp, velocity=u,
                     periodic=(False, True, True) if q == 19 else (False, True, True), boundary_mode=1,
                     thermal_init_equilibrium=eq, tau_t=0.8, beta=0.5)
    assert s.get_is_flow_thermal()
    fluid = ids == 0
    step_and_compare(s, o, [1, 2, 7, 30], mask=fluid, check_temperature=True)
    qt = 5 if q == 9 else 7
    mine = s.get_thermal_populations()          # (Qt, N) in the solver's SoA layout
    ref = o.thermal_lattice().reshape(-1, qt).T  # the oracle's AoS (N, Qt)
    assert np.array_equal(mine[:, fluid], ref[:, fluid])


def test_thermal_push_equals_stream_pass(monkeypatch):
    res, ids, temp, u, f, objs = walls_case(19)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("BF_THERMAL_PUSH", flag)
        s, _ = make_pair(res, 0.6, VS[19], ids=ids, objects=objs, force=f, temperature=temp, velocity=u,
                         periodic=(False, True, True), boundary_mode=1, thermal_init_equilibrium=True,
                         tau_t=0.8, beta=0.5)
        s.iterate_time(steps=41, save=True)
        out.append((s.get_thermal_populations(), s.get_velocity_density_texture().copy(),
                    s.get_force_temperature_texture().copy()))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_thermal_push_with_reductions_saves_and_snapshots(monkeypatch, tmp_path):
    """Reductions (a measure pass reading the thermal state), save steps,
    graph-sized batches and a snapshot round trip between pushed steps give
    what the separate stream pass gives."""
    res, ids, temp, u, f, objs = walls_case(19)
    runs = []
    for flag in ("1", "0"):
        monkeypatch.setenv("BF_THERMAL_PUSH", flag)
        s, _ = make_pair(res, 0.6, VS[19], ids=ids, objects=objs, force=f, temperature=temp, velocity=u,
                         periodic=(False, True, True), boundary_mode=1, thermal_init_equilibrium=True,
                         tau_t=0.8, beta=0.5)
        rec = []
        s.iterate_time(steps=5, save=False)
        rec.append(s.reduce().copy())
        s.iterate_time(steps=3, save=True)
        rec.append(s.get_force_temperature_texture().copy())
        p = tmp_path / f"snap{flag}.bin"
        s.save_current_tick_mesoscropic(p)
        s.iterate_time(steps=20, save=True)  # includes a 16-step graph batch
        rec.append(s.get_thermal_populations().copy())
        s.load_tick_mesoscropic(p)
        s.iterate_time(steps=20, save=True)
        rec.append(s.get_thermal_populations().copy())
        rec.append(s.reduce().copy())
        runs.append(rec)
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)
    assert np.array_equal(runs[0][2], runs[0][3])  # the snapshot replays the same steps


@pytest.mark.parametrize("storage", [bf.FloatingPointAccuracy.fp16s, bf.FloatingPointAccuracy.fp16c])
def test_thermal_push_with_16bit_flow_storage(storage):
    """The thermal lattice (FP32) beside a 16-bit flow lattice in the split step."""
    res, ids, temp, u, f, objs = walls_case(19)
    s, o = make_pair(res, 0.6, VS[19], ids=ids, objects=objs, force=f, temperature=temp, velocity=u,
                     periodic=(False, True, True), boundary_mode=1, thermal_init_equilibrium=True,
                     tau_t=0.8, beta=0.5, storage=storage)
    fluid = ids == 0
    step_and_compare(s, o, [1, 2, 9], mask=fluid, check_temperature=True)
    mine = s.get_thermal_populations()
    ref = o.thermal_lattice().reshape(-1, 7).T
    assert np.array_equal(mine[:, fluid], ref[:, fluid])
