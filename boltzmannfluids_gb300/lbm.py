"""Python mirror of BoltzmannFluids' solver class `LBM` over the C ABI.

Method names, argument meaning and defaults follow
BoltzmannFluids/Source/LBM/LBM.h:26-145.  The compute path is the sm_103a
library libbfgb300.so (include/bf_lbm.h); this module only marshals
arguments.  There is no CPU fallback: constructing an `LBM` without the
built library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
import time
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbfgb300.so")


class VelocitySet(enum.IntEnum):
    """VelocitySet.h:18-23 (same numeric values)."""
    D2Q9 = 2
    D3Q15 = 3
    D3Q19 = 4
    D3Q27 = 5


class FloatingPointAccuracy(enum.IntEnum):
    """DDF storage.  fp32/fp16 are the reference's FloatingPointAccuracy
    (FloatingPointAccuracy.h:6-9, fp16 = R16F lattice); fp16s (shifted IEEE
    half of f-w) and fp16c (custom-scaled: IEEE half of (f-w)*2^12) are extensions; fp64 is
    the FP64 accuracy reference stepper (every esoteric-pull configuration)."""
    fp32 = 0
    fp16 = 1
    fp16s = 2
    fp16c = 3
    fp64 = 4


class BoundaryMode(enum.IntEnum):
    skip = 0          # as the reference's collide.comp reads it
    bounce_back = 1   # halfway bounce-back with moving walls, folded into AA


class Collision(enum.IntEnum):
    bgk = 0
    trt = 1


class ObjectKind(enum.IntEnum):
    solid = 0
    eq_velocity = 1
    eq_density = 2


class Field(enum.IntEnum):
    velocity_density = 0
    boundary = 1
    force_temperature = 2
    populations = 3
    thermal_populations = 4
    pseudopotential = 5


class LBMError(RuntimeError):
    """Raised for a non-zero bf_status; `.code` holds the status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[LBM Error] {message} (status {code})")
        self.code = code


class _InitDesc(C.Structure):
    _fields_ = [
        ("resolution", C.c_int32 * 3),
        ("relaxation_time", C.c_float),
        ("periodic", C.c_int32 * 3),
        ("velocity_set", C.c_int32),
        ("storage", C.c_int32),
        ("multiphase", C.c_int32),
        ("esoteric", C.c_int32),
        ("boundary_mode", C.c_int32),
        ("collision", C.c_int32),
        ("trt_magic", C.c_float),
        ("velocity_limit", C.c_float),
        ("velocity_limit_extreme", C.c_float),
        ("intermolecular_interaction_strength", C.c_float),
        ("thermal_relaxation_time", C.c_float),
        ("thermal_expansion_coefficient", C.c_float),
        ("thermal_init_equilibrium", C.c_int32),
        ("two_buffer_fixed", C.c_int32),
        ("reserved", C.c_int32 * 8),
    ]


class _Object(C.Structure):
    _fields_ = [
        ("velocity_translational", C.c_float * 3),
        ("temperature", C.c_float),
        ("velocity_angular", C.c_float * 3),
        ("center_of_mass", C.c_float * 3),
        ("effective_density", C.c_float),
        ("kind", C.c_int32),
    ]


class _Field(C.Structure):
    _fields_ = [
        ("device_ptr", C.c_void_p),
        ("kind", C.c_int32),
        ("resolution", C.c_int32 * 3),
        ("components", C.c_int32),
        ("bytes_per_component", C.c_int32),
        ("bytes", C.c_size_t),
    ]


# every entry point of include/bf_lbm.h with its ctypes signature
ABI = {
    "bf_init_desc_default": (None, [C.POINTER(_InitDesc)]),
    "bf_last_error": (C.c_char_p, []),
    "bf_abi_version": (C.c_int, []),
    "bf_debug_fail_allocation_after": (C.c_int, [C.c_int32]),
    "bf_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "bf_destroy": (C.c_int, [C.c_void_p]),
    "bf_set_boundry_properties": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(_Object)]),
    "bf_clear_boundry_properties": (C.c_int, [C.c_void_p]),
    "bf_initialize_fields": (C.c_int, [C.c_void_p, C.POINTER(_InitDesc), C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]),
    "bf_iterate_time": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "bf_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "bf_synchronize": (C.c_int, [C.c_void_p, C.c_int32]),
    "bf_get_total_ticks_elapsed": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "bf_get_resolution": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "bf_get_velocity_set_vector_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "bf_get_relaxation_time": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "bf_set_relaxation_time": (C.c_int, [C.c_void_p, C.c_float]),
    "bf_get_constant_force": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "bf_set_constant_force": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "bf_get_intermolecular_interaction_strength": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "bf_set_intermolecular_interaction_strength": (C.c_int, [C.c_void_p, C.c_float]),
    "bf_set_velocity_limits": (C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    "bf_set_thermal_parameters": (C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    "bf_get_scheme_flags": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "bf_get_field": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(_Field)]),
    "bf_copy_field_to_host": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    "bf_copy_boundry_bits_to_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bf_reduce": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "bf_save_snapshot": (C.c_int, [C.c_void_p, C.c_char_p]),
    "bf_load_snapshot": (C.c_int, [C.c_void_p, C.c_char_p]),
    "bf_save_macroscopic": (C.c_int, [C.c_void_p, C.c_char_p]),
    "bf_load_macroscopic": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "bf_benchmark_steps": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "bf_get_velosity_vectors": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_int32)]),
    "bf_bits_per_boundry": (C.c_int, [C.c_int32, C.POINTER(C.c_int32)]),
    "bf_pack_boundries": (C.c_int, [C.c_void_p, C.c_size_t, C.c_int32, C.c_void_p, C.c_size_t,
                                    C.POINTER(C.c_size_t)]),
    "bf_reduce_field_noalloc": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.POINTER(C.c_double)]),
    "bf_adjoint_desc_default": (None, [C.c_void_p]),
    "bf_adjoint_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p]),
    "bf_adjoint_destroy": (C.c_int, [C.c_void_p]),
    "bf_adjoint_set_parameters": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "bf_adjoint_set_target": (C.c_int, [C.c_void_p, C.c_void_p]),
    "bf_adjoint_forward": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "bf_adjoint_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "bf_adjoint_time": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "bf_adjoint_get_resident_states": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "bf_mc_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "bf_mc_destroy": (C.c_int, [C.c_void_p]),
    "bf_mc_compute": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.c_float,
                                C.POINTER(C.c_float), C.c_void_p, C.POINTER(C.c_uint64)]),
    "bf_mc_get_vertices": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64)]),
    "bf_mc_copy_vertices_to_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "bf_mc_case_table": (C.c_int, [C.c_void_p, C.c_void_p]),
    "bf_voxelize_mesh": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_void_p]),
    "bf_render3d": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                              C.c_void_p, C.c_void_p]),
}

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads libbfgb300.so and binds every C-ABI symbol.  Raises when the
    library has not been built (there is deliberately no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libbfgb300.so is not built ({path}); run boltzmannfluids_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in ABI.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(code: int):
    if code != 0:
        raise LBMError(code, _lib.bf_last_error().decode(errors="replace"))


def get_velosity_vectors(velocity_set, thermal: bool = False) -> np.ndarray:
    """(count, 4) float32 rows (c.x, c.y, c.z, w): VelocitySet.cpp:53-142 / :180-204."""
    lib = load_library()
    n = C.c_int32()
    _check(lib.bf_get_velosity_vectors(int(velocity_set), int(bool(thermal)), None, C.byref(n)))
    out = np.zeros((n.value, 4), np.float32)
    _check(lib.bf_get_velosity_vectors(int(velocity_set), int(bool(thermal)), out.ctypes.data_as(C.c_void_p),
                                       C.byref(n)))
    return out


def bits_per_boundry(object_count: int) -> int:
    lib = load_library()
    b = C.c_int32()
    _check(lib.bf_bits_per_boundry(int(object_count), C.byref(b)))
    return b.value


def pack_boundries(ids, bits: int) -> np.ndarray:
    """Packed boundary words of LBM.cpp:634-659."""
    lib = load_library()
    ids = np.ascontiguousarray(np.asarray(ids, np.uint32).reshape(-1))
    w = C.c_size_t()
    _check(lib.bf_pack_boundries(None, ids.size, int(bits), None, 0, C.byref(w)))
    out = np.zeros(w.value, np.uint32)
    _check(lib.bf_pack_boundries(ids.ctypes.data_as(C.c_void_p), ids.size, int(bits), out.ctypes.data_as(C.c_void_p),
                                 out.size, C.byref(w)))
    return out


@dataclass
class FluidProperties:
    """LBM::FluidProperties (LBM.h:41-47)."""
    velocity: Sequence[float] = (0.0, 0.0, 0.0)
    force: Sequence[float] = (0.0, 0.0, 0.0)
    density: float = 1.0
    temperature: float = 1.0
    boundry_id: int = 0


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class LBM:
    """The reference's LBM solver API on the GB300 kernels."""

    not_a_boundry = 0
    max_boundry_count = 255
    referance_temperature = 1.0
    referance_boundry_density = 1.0

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.bf_create(C.byref(h)))
        self._h = h
        # public knobs of LBM.h:139-145 plus the extensions
        self.is_lattice_texture3d = False  # layout detail of the GL path; no effect here
        self.is_collide_esoteric = False
        self.velocity_limit = 0.25
        self.velocity_limit_extreme = 0.30
        self.boundary_mode = BoundaryMode.skip
        self.collision = Collision.bgk
        self.trt_magic = 0.25
        self.thermal_relaxation_time = 2.0
        self.thermal_expansion_coefficient = 0.5
        self.intermolecular_interaction_strength = -6.0
        self.thermal_init_equilibrium = False
        self.two_buffer_fixed = False
        self._res = (0, 0, 0)
        self._vs = VelocitySet.D2Q9
        # knob values the solver holds (sent at initialisation, then when changed)
        self._sent = None
        # LBM::iterate_time's wall-clock state (LBM.cpp:220-240): epoch before the first call
        self._first_iteration = True
        self._simulation_begin = 0.0
        self._last_visual_update = 0.0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.bf_destroy(h)
            self._h = None

    # ---- boundary objects (LBM.h:60-82) -------------------------------
    def set_boundry_properties(self, boundry_id: int, *args, velocity_translational=None, velocity_angular=None,
                               center_of_mass=None, temperature: float = 1.0, effective_density: float = 1.0,
                               kind: ObjectKind = ObjectKind.solid):
        """Overloads of LBM.cpp:1015-1065:
        (id, u_trans, omega, com[, T[, rho_eff]]), (id, u_trans[, T[, rho_eff]]), (id, T[, rho_eff])."""
        vt, va, com = (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)
        a = list(args)
        if a and np.ndim(a[0]) == 1:
            vt = a.pop(0)
            if a and np.ndim(a[0]) == 1:
                va = a.pop(0)
                com = a.pop(0)
        if a:
            temperature = a.pop(0)
        if a:
            effective_density = a.pop(0)
        if velocity_translational is not None:
            vt = velocity_translational
        if velocity_angular is not None:
            va = velocity_angular
        if center_of_mass is not None:
            com = center_of_mass
        o = _Object()
        o.velocity_translational[:] = [float(v) for v in vt]
        o.velocity_angular[:] = [float(v) for v in va]
        o.center_of_mass[:] = [float(v) for v in com]
        o.temperature = float(temperature)
        o.effective_density = float(effective_density)
        o.kind = int(kind)
        _check(self._lib.bf_set_boundry_properties(self._h, int(boundry_id), C.byref(o)))

    def clear_boundry_properties(self):
        _check(self._lib.bf_clear_boundry_properties(self._h))

    # ---- initialisation (LBM.h:48-58) ---------------------------------
    def _desc(self, resolution, relaxation_time, periodic, velocity_set, fp_accuracy, multiphase):
        d = _InitDesc()
        self._lib.bf_init_desc_default(C.byref(d))
        d.resolution[:] = [int(v) for v in resolution]
        d.relaxation_time = float(relaxation_time)
        d.periodic[:] = [int(bool(p)) for p in periodic]
        d.velocity_set = int(velocity_set)
        d.storage = int(fp_accuracy)
        d.multiphase = int(bool(multiphase))
        d.esoteric = int(bool(self.is_collide_esoteric))
        d.boundary_mode = int(self.boundary_mode)
        d.collision = int(self.collision)
        d.trt_magic = float(self.trt_magic)
        d.velocity_limit = float(self.velocity_limit)
        d.velocity_limit_extreme = float(self.velocity_limit_extreme)
        d.intermolecular_interaction_strength = float(self.intermolecular_interaction_strength)
        d.thermal_relaxation_time = float(self.thermal_relaxation_time)
        d.thermal_expansion_coefficient = float(self.thermal_expansion_coefficient)
        d.thermal_init_equilibrium = int(bool(self.thermal_init_equilibrium))
        d.two_buffer_fixed = int(bool(self.two_buffer_fixed))
        return d

    def initialize_fields(self, initialization_lambda: Callable, resolution, relaxation_time: float,
                          periodic_x=True, periodic_y=True, periodic_z=True,
                          velocity_set=VelocitySet.D2Q9, fp_accuracy=FloatingPointAccuracy.fp32,
                          is_flow_multiphase=False):
        """LBM::initialize_fields: calls `initialization_lambda((x, y, z), props)` once per cell
        (x fastest) on a fresh FluidProperties, then uploads.  Use
        initialize_fields_from_arrays for large grids."""
        rx, ry, rz = (int(v) for v in resolution)
        n = rx * ry * rz
        rho = np.empty(n, np.float32)
        u = np.empty((n, 3), np.float32)
        f = np.empty((n, 3), np.float32)
        t = np.empty(n, np.float32)
        ids = np.empty(n, np.uint32)
        k = 0
        for z in range(rz):
            for y in range(ry):
                for x in range(rx):
                    p = FluidProperties()
                    initialization_lambda((x, y, z), p)
                    rho[k] = p.density
                    u[k] = p.velocity
                    f[k] = p.force
                    t[k] = p.temperature
                    ids[k] = int(p.boundry_id)
                    k += 1
        self.initialize_fields_from_arrays((rx, ry, rz), relaxation_time, density=rho, velocity=u, force=f,
                                           temperature=t, boundry_id=ids, periodic=(periodic_x, periodic_y, periodic_z),
                                           velocity_set=velocity_set, fp_accuracy=fp_accuracy,
                                           is_flow_multiphase=is_flow_multiphase)

    def initialize_fields_from_arrays(self, resolution, relaxation_time: float, density=None, velocity=None,
                                      force=None, temperature=None, boundry_id=None, periodic=(True, True, True),
                                      velocity_set=VelocitySet.D2Q9, fp_accuracy=FloatingPointAccuracy.fp32,
                                      is_flow_multiphase=False):
        """Array form of initialize_fields: per-cell arrays in x-fastest order."""
        rx, ry, rz = (int(v) for v in resolution)
        n = rx * ry * rz

        def prep(a, comps, dtype):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=dtype).reshape(n * comps))
            return a

        arrs = (prep(density, 1, np.float32), prep(velocity, 3, np.float32), prep(force, 3, np.float32),
                prep(temperature, 1, np.float32), prep(boundry_id, 1, np.uint32))
        # initialize_fields resets the thermal relaxation time to 2 (LBM.cpp:461);
        # a value set afterwards reaches the solver before the next step
        self.thermal_relaxation_time = 2.0
        d = self._desc((rx, ry, rz), relaxation_time, periodic, velocity_set, fp_accuracy, is_flow_multiphase)
        _check(self._lib.bf_initialize_fields(self._h, C.byref(d), *[_ptr(a) for a in arrs]))
        self._res = (rx, ry, rz)
        self._vs = VelocitySet(int(velocity_set))
        self._sent = self._knobs()

    def _knobs(self):
        return (float(self.velocity_limit), float(self.velocity_limit_extreme), float(self.thermal_relaxation_time),
                float(self.thermal_expansion_coefficient))

    def _sync_knobs(self):
        """The public knobs are uniforms the reference sets at every dispatch
        (LBM.cpp:1590-1591, :1612-1613): changed values reach the solver
        before the next step.  An invalid thermal relaxation time (<= 0.5)
        raises here, and again at every later step until it is fixed."""
        if self._sent is None:
            return
        k = self._knobs()
        if k[:2] != self._sent[:2]:
            _check(self._lib.bf_set_velocity_limits(self._h, k[0], k[1]))
            self._sent = k[:2] + self._sent[2:]
        if k[2:] != self._sent[2:]:
            _check(self._lib.bf_set_thermal_parameters(self._h, k[2], k[3]))
            self._sent = self._sent[:2] + k[2:]

    # ---- time (LBM.h:34-38) -------------------------------------------
    def iterate_time(self, target_tick_per_second: float = 0, steps: Optional[int] = None,
                     save: Optional[bool] = None):
        """LBM::iterate_time (LBM.cpp:220-240) when called without `steps` and
        `save`: one tick, unless a positive target_tick_per_second is already
        met by the ticks run since the first call; the macroscopic fields are
        saved on the first tick and then only when more than 1000/60 ms (whole
        milliseconds) have passed since the last save.  With `steps` and/or
        `save`: that many ticks (default 1) at once, saving the fields on the
        last one when `save` (default True)."""
        self._sync_knobs()
        if steps is None and save is None:
            now = time.time()
            if self._first_iteration:
                self._simulation_begin = now
                self._last_visual_update = now
            targeted = int(target_tick_per_second * self.get_total_time_elapsed() / 1000.0)
            if target_tick_per_second <= 0 or self.get_total_ticks_elapsed() < targeted or self._first_iteration:
                since_ms = int((time.time() - self._last_visual_update) * 1000.0)
                do_save = self._first_iteration or since_ms > 1000.0 / 60
                if do_save:
                    self._last_visual_update = time.time()
                _check(self._lib.bf_iterate_time(self._h, 1, int(do_save)))
            self._first_iteration = False
            return
        _check(self._lib.bf_iterate_time(self._h, int(1 if steps is None else steps),
                                         int(True if save is None else bool(save))))

    def get_total_time_elapsed(self) -> float:
        """Milliseconds since the first LBM-style iterate_time call (LBM.cpp:247-250)."""
        return (time.time() - self._simulation_begin) * 1000.0

    def get_stream(self) -> int:
        """The solver's CUDA stream handle (a cudaStream_t as an integer)."""
        v = C.c_void_p()
        _check(self._lib.bf_get_stream(self._h, C.byref(v)))
        return v.value or 0

    def synchronize(self, timeout_ms: int = 0):
        _check(self._lib.bf_synchronize(self._h, int(timeout_ms)))

    def get_total_ticks_elapsed(self) -> int:
        v = C.c_int64()
        _check(self._lib.bf_get_total_ticks_elapsed(self._h, C.byref(v)))
        return v.value

    def get_resolution(self):
        r = (C.c_int32 * 3)()
        _check(self._lib.bf_get_resolution(self._h, r))
        return tuple(r)

    def get_velocity_set_vector_count(self) -> int:
        v = C.c_int32()
        _check(self._lib.bf_get_velocity_set_vector_count(self._h, C.byref(v)))
        return v.value

    def get_velocity_set(self):
        return self._vs

    def get_dimentionality(self):
        return 2 if self._vs == VelocitySet.D2Q9 else 3

    def get_relaxation_time(self) -> float:
        v = C.c_float()
        _check(self._lib.bf_get_relaxation_time(self._h, C.byref(v)))
        return v.value

    def set_relaxation_time(self, tau: float):
        _check(self._lib.bf_set_relaxation_time(self._h, float(tau)))

    def get_constant_force(self):
        v = (C.c_float * 3)()
        _check(self._lib.bf_get_constant_force(self._h, v))
        return tuple(v)

    def set_constant_force(self, force):
        v = (C.c_float * 3)(*[float(x) for x in force])
        _check(self._lib.bf_set_constant_force(self._h, v))

    def get_intermolecular_interaction_strength(self) -> float:
        v = C.c_float()
        _check(self._lib.bf_get_intermolecular_interaction_strength(self._h, C.byref(v)))
        return v.value

    def set_intermolecular_interaction_strength(self, g: float):
        self.intermolecular_interaction_strength = float(g)
        _check(self._lib.bf_set_intermolecular_interaction_strength(self._h, float(g)))

    def _flags(self):
        f, b = C.c_int32(), C.c_int32()
        _check(self._lib.bf_get_scheme_flags(self._h, C.byref(f), C.byref(b)))
        return f.value, b.value

    def get_is_forcing_scheme(self):
        return bool(self._flags()[0] & 1)

    def get_is_force_field_constant(self):
        return bool(self._flags()[0] & 2)

    def get_is_flow_thermal(self):
        return bool(self._flags()[0] & 4)

    def get_is_flow_multiphase(self):
        return bool(self._flags()[0] & 8)

    def get_bits_per_boundry(self):
        return self._flags()[1]

    # ---- readback (LBM.h:97-99) ---------------------------------------
    def _copy(self, kind: Field, dtype, comps):
        rx, ry, rz = self._res
        n = rx * ry * rz
        if kind == Field.populations:
            comps = self.get_velocity_set_vector_count()
        if kind == Field.thermal_populations:
            comps = 5 if self._vs == VelocitySet.D2Q9 else 7
        out = np.empty(n * comps, dtype)
        _check(self._lib.bf_copy_field_to_host(self._h, int(kind), out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def get_velocity_density_texture(self) -> np.ndarray:
        """(nz, ny, nx, 4) float32: u.xyz, rho of the last saved step."""
        rx, ry, rz = self._res
        return self._copy(Field.velocity_density, np.float32, 4).reshape(rz, ry, rx, 4)

    def get_boundry_texture(self) -> np.ndarray:
        rx, ry, rz = self._res
        return self._copy(Field.boundary, np.uint8, 1).reshape(rz, ry, rx)

    def get_force_temperature_texture(self) -> np.ndarray:
        rx, ry, rz = self._res
        return self._copy(Field.force_temperature, np.float32, 4).reshape(rz, ry, rx, 4)

    def get_populations(self) -> np.ndarray:
        """Raw DDF decoded to FP32, SoA (Q, N) in the solver's slot layout."""
        q = self.get_velocity_set_vector_count()
        return self._copy(Field.populations, np.float32, q).reshape(q, -1)

    def get_pseudopotential(self) -> np.ndarray:
        """(nz, ny, nx) float32 psi = 1 - exp(-rho_eff) that the next Shan-Chen step reads."""
        rx, ry, rz = self._res
        return self._copy(Field.pseudopotential, np.float32, 1).reshape(rz, ry, rx)

    def get_thermal_populations(self) -> np.ndarray:
        q = 5 if self._vs == VelocitySet.D2Q9 else 7
        return self._copy(Field.thermal_populations, np.float32, q).reshape(q, -1)

    def get_field_device(self, kind: Field):
        f = _Field()
        _check(self._lib.bf_get_field(self._h, int(kind), C.byref(f)))
        return f.device_ptr, f.bytes

    def get_boundry_bits(self) -> np.ndarray:
        words = C.c_size_t()
        _check(self._lib.bf_copy_boundry_bits_to_host(self._h, None, 0, C.byref(words)))
        out = np.zeros(words.value, np.uint32)
        if words.value:
            _check(self._lib.bf_copy_boundry_bits_to_host(self._h, out.ctypes.data_as(C.c_void_p), words.value,
                                                          C.byref(words)))
        return out

    # ---- reductions / snapshots ---------------------------------------
    def reduce(self) -> np.ndarray:
        """FP64 (mass, momentum x/y/z, kinetic energy) of the current state."""
        out = (C.c_double * 5)()
        _check(self._lib.bf_reduce(self._h, out))
        return np.array(out[:], np.float64)

    def save_current_tick_mesoscropic(self, path):
        _check(self._lib.bf_save_snapshot(self._h, os.fsencode(str(path))))

    def load_tick_mesoscropic(self, path, target_tick: int = -1):
        _check(self._lib.bf_load_snapshot(self._h, os.fsencode(str(path))))

    def save_current_tick_macroscopic(self, path):
        """u/rho, F/T and boundary ids of the last saved tick, with that tick (bf_save_macroscopic)."""
        _check(self._lib.bf_save_macroscopic(self._h, os.fsencode(str(path))))

    def load_tick_macroscopic(self, path, target_tick: int = -1):
        """Restarts from a macroscopic file: equilibrium populations of its
        fields, the tick counter at its tick (bf_load_macroscopic)."""
        self._sync_knobs()
        _check(self._lib.bf_load_macroscopic(self._h, os.fsencode(str(path)), int(target_tick)))

    def benchmark_steps(self, steps: int) -> float:
        """Runs `steps` steps bracketed by CUDA events on the solver's stream; returns milliseconds."""
        ms = C.c_float()
        self._sync_knobs()
        _check(self._lib.bf_benchmark_steps(self._h, int(steps), C.byref(ms)))
        return ms.value


class RenderMode(enum.IntEnum):
    """bf_render_mode: the five LBM::render3d_* views (LBM.cpp:1207-1376)."""
    density = 0
    velocity = 1
    boundries = 2
    forces = 3
    temperature = 4


def render3d(lbm: "LBM", mode: RenderMode, view, projection, width: int, height: int, sample_count: int = 64):
    """Headless LBM::render3d_<mode>(camera, sample_count): view/projection are
    column-major 4x4 matrices (glm layout); -> float32 (height, width, 4)
    straight RGBA, row 0 at the bottom (bf_render3d)."""
    import torch  # device buffer for the image
    lib = load_library()
    v = np.ascontiguousarray(np.asarray(view, np.float32).reshape(16))
    p = np.ascontiguousarray(np.asarray(projection, np.float32).reshape(16))
    img = torch.empty((int(height), int(width), 4), dtype=torch.float32, device="cuda")
    _check(lib.bf_render3d(lbm._h, int(mode), v.ctypes.data_as(C.c_void_p), p.ctypes.data_as(C.c_void_p), int(width),
                           int(height), int(sample_count), C.c_void_p(img.data_ptr()), None))
    return img.cpu().numpy()
