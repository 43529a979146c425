"""Loader of the reference-built checker (oracle/_ref/libref_<config>.so,
built by oracle/build_ref.py from the reference's own shader sources).
TEST INFRASTRUCTURE ONLY; present only where the reference sources are."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def available(config):
    return os.path.exists(os.path.join(REF_DIR, f"libref_{config}.so"))


class RefShaders:
    """The reference's compute shaders (compiled as C++) behind a restatement
    of LBM.cpp's driver.  Same inputs as LBM.initialize_fields_from_arrays;
    objects: {id: dict(velocity, temperature, effective_density)}."""

    def __init__(self, config, resolution, tau, density=None, velocity=None, force=None, temperature=None,
                 boundry_id=None, objects=None, G=-6.0, velocity_limit=0.25, velocity_limit_extreme=0.30,
                 tau_t=2.0, beta=0.5):
        self.lib = C.CDLL(os.path.join(REF_DIR, f"libref_{config}.so"))
        self.lib.ref_create.restype = C.c_void_p
        self.lib.ref_create.argtypes = [C.c_int] * 3 + [C.c_float] + [C.c_void_p] * 5 + [C.c_int, C.c_void_p] + \
                                       [C.c_float] * 5 + [C.POINTER(C.c_int)]
        self.lib.ref_iterate.argtypes = [C.c_void_p, C.c_int, C.c_int]
        self.lib.ref_fields.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        self.lib.ref_lattice.argtypes = [C.c_void_p, C.c_void_p]
        self.lib.ref_destroy.argtypes = [C.c_void_p]
        self.q = self.lib.ref_q()
        nx, ny, nz = (int(v) for v in resolution)
        n = nx * ny * nz
        self.n = n

        def arr(a, comps, default, dtype=np.float32):
            if a is None:
                return np.full(n * comps, default, dtype)
            return np.ascontiguousarray(np.asarray(a, dtype).reshape(n * comps))

        self._keep = [arr(density, 1, 1.0), arr(velocity, 3, 0.0), arr(force, 3, 0.0), arr(temperature, 1, 1.0),
                      arr(boundry_id, 1, 0, np.uint32)]
        nobj = 0
        ob = None
        if objects:
            nobj = max(objects) + 1
            ob = np.zeros(nobj * 12, np.float32)
            for k in range(nobj):
                ob[k * 12 + 3] = 1.0
                ob[k * 12 + 11] = 1.0
            for k, o in objects.items():
                ob[k * 12:k * 12 + 3] = o.get("velocity", (0, 0, 0))
                ob[k * 12 + 3] = o.get("temperature", 1.0)
                ob[k * 12 + 11] = o.get("effective_density", 1.0)
        self._keep.append(ob)
        p = [None if a is None else a.ctypes.data_as(C.c_void_p) for a in self._keep]
        st = C.c_int(0)
        self.h = self.lib.ref_create(nx, ny, nz, float(tau), p[0], p[1], p[2], p[3], p[4], nobj, p[5], float(G),
                                     float(velocity_limit), float(velocity_limit_extreme), float(tau_t), float(beta),
                                     C.byref(st))
        if not self.h:
            raise ValueError(f"inputs do not match the compiled configuration {config} (status {st.value})")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def iterate(self, n=1, save=True):
        self.lib.ref_iterate(self.h, int(n), int(bool(save)))

    def fields(self):
        vd = np.zeros(self.n * 4, np.float32)
        ft = np.zeros(self.n * 4, np.float32)
        self.lib.ref_fields(self.h, vd.ctypes.data_as(C.c_void_p), ft.ctypes.data_as(C.c_void_p))
        return vd.reshape(self.n, 4).astype(np.float64), ft.reshape(self.n, 4).astype(np.float64)

    def lattice(self):
        out = np.zeros(self.n * self.q, np.float32)
        self.lib.ref_lattice(self.h, out.ctypes.data_as(C.c_void_p))
        return out.reshape(self.q, self.n).astype(np.float64)
