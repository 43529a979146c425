"""Forward/backward pair of the differentiable channel-flow model
(bf_adjoint_* in include/bf_lbm.h): partial-bounce-back solid fraction and
inlet profile in, drag + velocity-mismatch objective out, gradients by the
hand-written discrete adjoint on the GPU."""
import ctypes as C

import numpy as np

from .lbm import VelocitySet, _check, load_library


class AdjointDesc(C.Structure):
    _fields_ = [
        ("resolution", C.c_int32 * 3),
        ("relaxation_time", C.c_float),
        ("velocity_set", C.c_int32),
        ("steps", C.c_int32),
        ("checkpoint_interval", C.c_int32),
        ("drag_weight", C.c_float),
        ("mismatch_weight", C.c_float),
        ("resident_states", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]


# resident_states: let the library keep as many forward states in device
# memory as fit (bf_lbm.h, BF_ADJOINT_RESIDENT_AUTO)
RESIDENT_AUTO = -1


class AdjointChannel:
    """J(s, u_in) and its gradient.  Arrays are x-fastest: s (N,), u_in (ny*nz,), u_target (N, 3).

    resident_states: 0 for two segment buffers of checkpoint_interval states,
    R > 0 for a pool of R states kept from the forward (at least
    checkpoint_interval - 1), RESIDENT_AUTO for as many as device memory holds.
    The gradients do not depend on it."""

    def __init__(self, resolution=(512, 256, 1), relaxation_time=0.6, velocity_set=VelocitySet.D2Q9, steps=2000,
                 checkpoint_interval=100, drag_weight=1.0, mismatch_weight=1.0, resident_states=0):
        self._lib = load_library()
        d = AdjointDesc()
        self._lib.bf_adjoint_desc_default(C.byref(d))
        d.resolution[:] = [int(v) for v in resolution]
        d.relaxation_time = float(relaxation_time)
        d.velocity_set = int(velocity_set)
        d.steps = int(steps)
        d.checkpoint_interval = int(checkpoint_interval)
        d.drag_weight = float(drag_weight)
        d.mismatch_weight = float(mismatch_weight)
        d.resident_states = int(resident_states)
        h = C.c_void_p()
        _check(self._lib.bf_adjoint_create(C.byref(h), C.byref(d)))
        self._h = h
        self.res = tuple(int(v) for v in resolution)
        self.n = self.res[0] * self.res[1] * self.res[2]
        self.rows = self.res[1] * self.res[2]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.bf_adjoint_destroy(h)
            self._h = None

    def set_parameters(self, solid_fraction=None, inlet_velocity=None):
        s = None if solid_fraction is None else np.ascontiguousarray(np.asarray(solid_fraction, np.float32).reshape(-1))
        u = None if inlet_velocity is None else np.ascontiguousarray(np.asarray(inlet_velocity, np.float32).reshape(-1))
        _check(self._lib.bf_adjoint_set_parameters(self._h, None if s is None else s.ctypes.data_as(C.c_void_p),
                                                   None if u is None else u.ctypes.data_as(C.c_void_p)))

    def set_target(self, u_target):
        t = np.ascontiguousarray(np.asarray(u_target, np.float32).reshape(-1))
        _check(self._lib.bf_adjoint_set_target(self._h, t.ctypes.data_as(C.c_void_p)))

    def forward(self) -> float:
        j = C.c_double()
        _check(self._lib.bf_adjoint_forward(self._h, C.byref(j)))
        return j.value

    def backward(self):
        gs = np.zeros(self.n, np.float64)
        gu = np.zeros(self.rows, np.float64)
        _check(self._lib.bf_adjoint_backward(self._h, gs.ctypes.data_as(C.c_void_p), gu.ctypes.data_as(C.c_void_p)))
        return gs, gu

    @property
    def resident_states(self) -> int:
        """The schedule in use: 0 (segment buffers) or the pool's state count."""
        r = C.c_int32()
        _check(self._lib.bf_adjoint_get_resident_states(self._h, C.byref(r)))
        return r.value

    def time(self, repeats=3):
        f, b = C.c_float(), C.c_float()
        _check(self._lib.bf_adjoint_time(self._h, int(repeats), C.byref(f), C.byref(b)))
        return f.value, b.value


def channel_setup(resolution, u_max=0.05, box=64, seed_s=6, seed_t=7):
    """Config-5 inputs: Poiseuille inlet profile, a seeded smoothed random solid
    fraction ramped to [0,1] inside a central box x box region, and a seeded
    smooth target velocity field (x-fastest arrays)."""
    nx, ny, nz = resolution
    y = np.arange(ny) + 0.5
    prof = 4.0 * u_max * y * (ny - y) / ny ** 2
    u_in = np.tile(prof, nz).astype(np.float32)
    rng = np.random.default_rng(seed_s)
    raw = rng.uniform(0, 1, (nz, ny, nx))
    sm = raw.copy()
    for _ in range(3):  # separable 5-point box smoothing in x and y
        sm = sum(np.roll(sm, k, axis=2) for k in range(-2, 3)) / 5.0
        sm = sum(np.roll(sm, k, axis=1) for k in range(-2, 3)) / 5.0
    ramp = np.clip((sm - 0.5) * 8.0 + 0.5, 0.0, 1.0)
    s = np.zeros((nz, ny, nx))
    b = min(box, nx, ny)
    x0, y0 = (nx - b) // 2, (ny - b) // 2
    s[:, y0:y0 + b, x0:x0 + b] = ramp[:, y0:y0 + b, x0:x0 + b]
    rng_t = np.random.default_rng(seed_t)
    tgt = rng_t.standard_normal((nz, ny, nx, 3))
    for _ in range(3):
        tgt = sum(np.roll(tgt, k, axis=2) for k in range(-2, 3)) / 5.0
        tgt = sum(np.roll(tgt, k, axis=1) for k in range(-2, 3)) / 5.0
    tgt *= 0.01 / max(np.abs(tgt).max(), 1e-12)
    tgt[..., 0] += prof[None, :, None] if nz == 1 else prof[None, :, None]
    if nz == 1:
        tgt[..., 2] = 0.0
    return s.reshape(-1).astype(np.float32), u_in, tgt.reshape(-1, 3).astype(np.float32)


def main(argv=None):
    """Command line: one gradient of the channel model and, with --repeats,
    the device time of forward and backward.

    python -m boltzmannfluids_gb300.adjoint --resolution 128 128 128 --steps 2000 --interval 100 --resident auto --repeats 2
    """
    import argparse
    ap = argparse.ArgumentParser(description=main.__doc__.splitlines()[0])
    ap.add_argument("--resolution", type=int, nargs=3, default=(512, 256, 1))
    ap.add_argument("--relaxation-time", type=float, default=0.6)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--interval", type=int, default=100, help="checkpoint interval K")
    ap.add_argument("--resident", default="0", help="0, a state count, or 'auto'")
    ap.add_argument("--repeats", type=int, default=0)
    a = ap.parse_args(argv)
    res = tuple(a.resolution)
    vs = VelocitySet.D2Q9 if res[2] == 1 else VelocitySet.D3Q19
    resident = RESIDENT_AUTO if a.resident == "auto" else int(a.resident)
    s, u_in, tgt = channel_setup(res)
    g = AdjointChannel(res, a.relaxation_time, vs, a.steps, a.interval, resident_states=resident)
    g.set_parameters(s, u_in)
    g.set_target(tgt)
    J = g.forward()
    gs, gu = g.backward()
    out = {"J": J, "grad_s_norm": float(np.linalg.norm(gs)), "grad_u_in_norm": float(np.linalg.norm(gu)),
           "resident_states": g.resident_states}
    if a.repeats > 0:
        f, b = g.time(a.repeats)
        out.update(forward_ms=f, backward_ms=b, gradient_over_forward=(f + b) / f)
    print(out)


if __name__ == "__main__":
    main()
