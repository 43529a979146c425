"""ctypes loader for the CPU oracle (oracle/lbm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product package never
imports this module.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class OrcDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("velocity_set", C.c_int), ("storage", C.c_int),
        ("multiphase", C.c_int), ("esoteric", C.c_int), ("periodic", C.c_int * 3), ("tau", C.c_float),
        ("boundary_mode", C.c_int), ("collision", C.c_int), ("trt_magic", C.c_float),
        ("velocity_limit", C.c_float), ("velocity_limit_extreme", C.c_float), ("G", C.c_float),
        ("tau_t", C.c_float), ("beta", C.c_float), ("thermal_init_equilibrium", C.c_int),
        ("two_buffer_fixed", C.c_int),
    ]


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _b  # noqa: F401  (package-relative when imported as oracle.oracle)
    so = _b.build()
    lib = C.CDLL(so)
    for p in ("orc32_", "orc64_"):
        f = getattr(lib, p + "create")
        f.restype = C.c_void_p
        f.argtypes = [C.POINTER(OrcDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                      C.c_void_p, C.c_void_p]
        getattr(lib, p + "destroy").argtypes = [C.c_void_p]
        getattr(lib, p + "iterate").argtypes = [C.c_void_p, C.c_int, C.c_int]
        getattr(lib, p + "get_fields").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        getattr(lib, p + "get_lattice").argtypes = [C.c_void_p, C.c_void_p]
        getattr(lib, p + "set_lattice").argtypes = [C.c_void_p, C.c_void_p]
        getattr(lib, p + "get_thermal").argtypes = [C.c_void_p, C.c_void_p]
        getattr(lib, p + "get_boundries").argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        getattr(lib, p + "reduce").argtypes = [C.c_void_p, C.c_void_p]
        getattr(lib, p + "set_thermal").argtypes = [C.c_void_p, C.c_float, C.c_float]
        for n in ("thermal", "forcing", "constant_force", "bits", "q"):
            getattr(lib, p + n).argtypes = [C.c_void_p]
            getattr(lib, p + n).restype = C.c_int
        getattr(lib, p + "ticks").argtypes = [C.c_void_p]
        getattr(lib, p + "ticks").restype = C.c_long
        getattr(lib, p + "bits_per_boundry").argtypes = [C.c_int]
        getattr(lib, p + "bits_per_boundry").restype = C.c_int
        getattr(lib, p + "pack_boundries").argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p, C.c_size_t]
        getattr(lib, p + "pack_boundries").restype = C.c_size_t
    lib.adj_create.restype = C.c_void_p
    lib.adj_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_double, C.c_double]
    lib.adj_destroy.argtypes = [C.c_void_p]
    lib.adj_set_params.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.adj_forward.argtypes = [C.c_void_p]
    lib.adj_forward.restype = C.c_double
    lib.adj_backward.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.orc32_f32_to_f16.argtypes = [C.c_float]
    lib.orc32_f32_to_f16.restype = C.c_uint16
    lib.orc32_f16_to_f32.argtypes = [C.c_uint16]
    lib.orc32_f16_to_f32.restype = C.c_float
    lib.orc32_exp_f32.argtypes = [C.c_float]
    lib.orc32_exp_f32.restype = C.c_float
    lib.orc64_exp_f64.argtypes = [C.c_double]
    lib.orc64_exp_f64.restype = C.c_double
    lib.orc32_fp16c_round.argtypes = [C.c_float]
    lib.orc32_fp16c_round.restype = C.c_float
    _lib = lib
    return lib


Q_OF = {2: 9, 3: 15, 4: 19, 5: 27}


class Oracle:
    """CPU stepper with the same inputs as LBM.initialize_fields_from_arrays.

    precision=32: ref-literal FP32 restatement; precision=64: FP64 oracle.
    objects: dict id -> dict(velocity=(3), temperature, effective_density, kind).
    """

    def __init__(self, resolution, tau, density=None, velocity=None, force=None, temperature=None,
                 boundry_id=None, periodic=(True, True, True), velocity_set=2, storage=0, multiphase=False,
                 esoteric=False, boundary_mode=0, collision=0, trt_magic=0.25, velocity_limit=0.25,
                 velocity_limit_extreme=0.30, G=-6.0, tau_t=2.0, beta=0.5, thermal_init_equilibrium=False,
                 two_buffer_fixed=False, objects=None, precision=32):
        self.lib = load()
        self.p = "orc32_" if precision == 32 else "orc64_"
        rx, ry, rz = (int(v) for v in resolution)
        self.res = (rx, ry, rz)
        self.n = rx * ry * rz
        self.q = Q_OF[int(velocity_set)]
        self.qt = 5 if int(velocity_set) == 2 else 7
        d = OrcDesc()
        d.nx, d.ny, d.nz = rx, ry, rz
        d.velocity_set = int(velocity_set)
        d.storage = int(storage)
        d.multiphase = int(bool(multiphase))
        d.esoteric = int(bool(esoteric))
        d.periodic[:] = [int(bool(p)) for p in periodic]
        d.tau = float(tau)
        d.boundary_mode = int(boundary_mode)
        d.collision = int(collision)
        d.trt_magic = float(trt_magic)
        d.velocity_limit = float(velocity_limit)
        d.velocity_limit_extreme = float(velocity_limit_extreme)
        d.G = float(G)
        # initialize_fields resets the thermal relaxation time to 2
        # (LBM.cpp:461): the initial pass runs with 2, the given value applies
        # from the first step on (set after initialisation, as a caller of the
        # reference must)
        d.tau_t = 2.0
        d.beta = float(beta)
        d.thermal_init_equilibrium = int(bool(thermal_init_equilibrium))
        d.two_buffer_fixed = int(bool(two_buffer_fixed))
        n = self.n

        def prep(a, comps, dtype):
            if a is None:
                return None
            return np.ascontiguousarray(np.asarray(a, dtype=dtype).reshape(n * comps))

        self._keep = [prep(density, 1, np.float32), prep(velocity, 3, np.float32), prep(force, 3, np.float32),
                      prep(temperature, 1, np.float32), prep(boundry_id, 1, np.uint32)]
        nobj = 0
        objs = kinds = None
        if objects:
            nobj = max(objects) + 1
            objs = np.zeros(nobj * 12, np.float32)
            kinds = np.zeros(nobj, np.int32)
            for k in range(nobj):
                objs[k * 12 + 3] = 1.0
                objs[k * 12 + 11] = 1.0
            for k, o in objects.items():
                v = o.get("velocity", (0, 0, 0))
                objs[k * 12:k * 12 + 3] = v
                objs[k * 12 + 3] = o.get("temperature", 1.0)
                objs[k * 12 + 4:k * 12 + 7] = o.get("velocity_angular", (0, 0, 0))
                objs[k * 12 + 8:k * 12 + 11] = o.get("center_of_mass", (0, 0, 0))
                objs[k * 12 + 11] = o.get("effective_density", 1.0)
                kinds[k] = int(o.get("kind", 0))
        self._keep += [objs, kinds]
        ptrs = [None if a is None else a.ctypes.data_as(C.c_void_p) for a in self._keep]
        self.h = getattr(self.lib, self.p + "create")(C.byref(d), ptrs[0], ptrs[1], ptrs[2], ptrs[3], ptrs[4],
                                                     nobj, ptrs[5], ptrs[6])
        if not self.h:
            raise ValueError("oracle: bad description")
        if float(tau_t) != 2.0:
            self.set_thermal(tau_t, beta)

    def __del__(self):
        if getattr(self, "h", None):
            getattr(self.lib, self.p + "destroy")(self.h)
            self.h = None

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def set_thermal(self, tau_t, beta):
        self._f("set_thermal")(self.h, C.c_float(float(tau_t)), C.c_float(float(beta)))

    def iterate(self, n=1, save=True):
        self._f("iterate")(self.h, int(n), int(bool(save)))

    def fields(self):
        """(vel_den (N,4), force_temp (N,4)) as float64 of the last saved step."""
        vd = np.zeros(self.n * 4, np.float64)
        ft = np.zeros(self.n * 4, np.float64)
        self._f("get_fields")(self.h, vd.ctypes.data_as(C.c_void_p), ft.ctypes.data_as(C.c_void_p), None)
        return vd.reshape(self.n, 4), ft.reshape(self.n, 4)

    def lattice(self):
        out = np.zeros(self.n * self.q, np.float64)
        self._f("get_lattice")(self.h, out.ctypes.data_as(C.c_void_p))
        return out.reshape(self.q, self.n)

    def set_lattice(self, a):
        a = np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1))
        self._f("set_lattice")(self.h, a.ctypes.data_as(C.c_void_p))

    def thermal_lattice(self):
        """thermal populations in the reference's AoS order (cell*Qt + i), as (N, Qt)."""
        out = np.zeros(self.n * self.qt, np.float64)
        self._f("get_thermal")(self.h, out.ctypes.data_as(C.c_void_p))
        return out.reshape(self.n, self.qt)

    def boundary_words(self):
        words = (self.n * max(self.bits, 0) + 31) // 32
        out = np.zeros(words + 1, np.uint32)
        self._f("get_boundries")(self.h, out.ctypes.data_as(C.c_void_p), words)
        return out[:words]

    def reduce(self):
        out = np.zeros(5, np.float64)
        self._f("reduce")(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    @property
    def ticks(self):
        return self._f("ticks")(self.h)

    @property
    def thermal(self):
        return bool(self._f("thermal")(self.h))

    @property
    def forcing(self):
        return bool(self._f("forcing")(self.h))

    @property
    def constant_force(self):
        return bool(self._f("constant_force")(self.h))

    @property
    def bits(self):
        return self._f("bits")(self.h)


def bits_per_boundry(count):
    return load().orc32_bits_per_boundry(int(count))


def pack_boundries(ids, bits):
    ids = np.ascontiguousarray(np.asarray(ids, np.uint32))
    lib = load()
    words = lib.orc32_pack_boundries(None, ids.size, int(bits), None, 0)
    out = np.zeros(words + 1, np.uint32)
    lib.orc32_pack_boundries(ids.ctypes.data_as(C.c_void_p), ids.size, int(bits), out.ctypes.data_as(C.c_void_p),
                             words + 1)
    return out[:words]


class AdjointOracle:
    """FP64 reference of the differentiable channel model and its adjoint
    (oracle/adjoint_oracle.c).  Arrays: s (N,), u_in (ny*nz,), u_target (N, 3)."""

    def __init__(self, resolution, tau, steps, q, s, u_in, u_target, drag_weight=1.0, mismatch_weight=1.0):
        self.lib = load()
        nx, ny, nz = (int(v) for v in resolution)
        self.res = (nx, ny, nz)
        self.n = nx * ny * nz
        self._s = np.ascontiguousarray(np.asarray(s, np.float64).reshape(-1))
        self._u = np.ascontiguousarray(np.asarray(u_in, np.float64).reshape(-1))
        self._t = np.ascontiguousarray(np.asarray(u_target, np.float64).reshape(-1))
        self.h = self.lib.adj_create(nx, ny, nz, int(q), float(tau), int(steps), self._s.ctypes.data_as(C.c_void_p),
                                     self._u.ctypes.data_as(C.c_void_p), self._t.ctypes.data_as(C.c_void_p),
                                     float(drag_weight), float(mismatch_weight))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.adj_destroy(self.h)
            self.h = None

    def set_params(self, s, u_in):
        self._s = np.ascontiguousarray(np.asarray(s, np.float64).reshape(-1))
        self._u = np.ascontiguousarray(np.asarray(u_in, np.float64).reshape(-1))
        self.lib.adj_set_params(self.h, self._s.ctypes.data_as(C.c_void_p), self._u.ctypes.data_as(C.c_void_p))

    def forward(self):
        return self.lib.adj_forward(self.h)

    def backward(self):
        gs = np.zeros(self.n, np.float64)
        gu = np.zeros(self.res[1] * self.res[2], np.float64)
        self.lib.adj_backward(self.h, gs.ctypes.data_as(C.c_void_p), gu.ctypes.data_as(C.c_void_p))
        return gs, gu
