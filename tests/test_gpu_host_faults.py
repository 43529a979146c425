"""Host-side fault injection (no GPU fault): corrupted and truncated
snapshot files, a save into a missing directory, and a device allocation the
GPU cannot satisfy.  Each failure returns its status and leaves the solver
usable with its state unchanged."""
import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from boltzmannfluids_gb300.lbm import LBMError

pytestmark = pytest.mark.gpu

BF_ERR_OUT_OF_MEMORY = -3
BF_ERR_IO = -7


def small_solver():
    res = (24, 16, 12)
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(51)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.initialize_fields_from_arrays(res, 0.6, velocity=(0.02 * rng.uniform(-1, 1, (n, 3))).astype(np.float32),
                                    velocity_set=bf.VelocitySet.D3Q19)
    return s


def test_truncated_and_foreign_snapshots_leave_the_state(tmp_path):
    s = small_solver()
    s.iterate_time(steps=5)
    good = tmp_path / "good.bin"
    s.save_current_tick_mesoscropic(good)
    assert not (tmp_path / "good.bin.partial").exists()
    s.iterate_time(steps=7)
    before = s.get_populations().copy()
    ticks = s.get_total_ticks_elapsed()
    data = good.read_bytes()
    cut = tmp_path / "cut.bin"
    cut.write_bytes(data[: len(data) // 2])
    other = tmp_path / "other.bin"
    other.write_bytes(b"not a snapshot" + data[14:])
    for bad in (cut, other):
        with pytest.raises(LBMError) as e:
            s.load_tick_mesoscropic(bad)
        assert e.value.code == BF_ERR_IO
        assert np.array_equal(s.get_populations(), before)
        assert s.get_total_ticks_elapsed() == ticks
    s.load_tick_mesoscropic(good)  # the intact file still loads
    assert s.get_total_ticks_elapsed() == 5


def test_failed_save_leaves_no_file(tmp_path):
    s = small_solver()
    target = tmp_path / "missing_dir" / "snap.bin"
    with pytest.raises(LBMError) as e:
        s.save_current_tick_mesoscropic(target)
    assert e.value.code == BF_ERR_IO
    assert not target.exists() and not (tmp_path / "missing_dir").exists()
    s.iterate_time(steps=3)  # still usable


@pytest.mark.parametrize("after", [0, 3, 6])
def test_allocation_failure_reports_and_recovers(after):
    """The (after+1)-th device allocation of an initialisation fails (host-side
    injection through bf_debug_fail_allocation_after): the call reports
    out of memory and the same handle initialises afterwards."""
    lib = bf.load_library()
    s = bf.LBM()
    s.is_collide_esoteric = True
    lib.bf_debug_fail_allocation_after(after)
    try:
        with pytest.raises(LBMError) as e:
            s.initialize_fields_from_arrays((16, 12, 10), 0.6, velocity_set=bf.VelocitySet.D3Q19)
        assert e.value.code == BF_ERR_OUT_OF_MEMORY
    finally:
        lib.bf_debug_fail_allocation_after(-1)
    s.initialize_fields_from_arrays((16, 12, 10), 0.6, velocity_set=bf.VelocitySet.D3Q19)
    s.iterate_time(steps=4, save=True)
    assert np.isfinite(s.get_velocity_density_texture()).all()
