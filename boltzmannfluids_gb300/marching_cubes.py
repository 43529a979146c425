"""Marching cubes on the GPU over the C ABI (bf_mc_*): the mesh that
BoltzmannFluids' MarchingCubes (MarchingCubes.h:13-39) builds from a 3D
field, as a triangle list."""
import ctypes as C

import numpy as np

from .lbm import LBM, Field, _check, load_library


def case_table():
    """(triangles (256, 15) int8 edge numbers, -1 padded; counts (256,) uint8)."""
    lib = load_library()
    tri = np.zeros((256, 15), np.int8)
    cnt = np.zeros(256, np.uint8)
    _check(lib.bf_mc_case_table(tri.ctypes.data_as(C.c_void_p), cnt.ctypes.data_as(C.c_void_p)))
    return tri, cnt


class MarchingCubes:
    """MarchingCubes::compute(source_texture, mipmap) of the reference with the
    threshold and mesh_scale it sets as uniforms (1.0 and vec3(1) there,
    MarchingCubes.cpp:44-46) exposed as arguments."""

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.bf_mc_create(C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.bf_mc_destroy(self._h)
            self._h = C.c_void_p()

    def compute_device(self, field_ptr: int, resolution, components: int = 1, component: int = 0,
                       threshold: float = 1.0, mesh_scale=(1.0, 1.0, 1.0), stream: int = 0) -> int:
        """Mesh of a device field; returns the triangle count (the vertices stay on the device)."""
        res = (C.c_int32 * 3)(*[int(v) for v in resolution])
        sc = (C.c_float * 3)(*[float(v) for v in mesh_scale])
        n = C.c_uint64()
        _check(self._lib.bf_mc_compute(self._h, C.c_void_p(int(field_ptr)), int(components), int(component), res,
                                       float(threshold), sc, C.c_void_p(int(stream)), C.byref(n)))
        return n.value

    def compute(self, lbm: LBM, threshold: float = 1.0, mesh_scale=(1.0, 1.0, 1.0)) -> np.ndarray:
        """Mesh of the solver's density (the w component of its velocity/density field);
        -> float32 (T, 3, 3) triangle vertices."""
        ptr, _ = lbm.get_field_device(Field.velocity_density)
        self.compute_device(ptr, lbm.get_resolution(), 4, 3, threshold, mesh_scale)
        return self.vertices()

    def vertices(self) -> np.ndarray:
        dev = C.c_void_p()
        n = C.c_uint64()
        _check(self._lib.bf_mc_get_vertices(self._h, C.byref(dev), C.byref(n)))
        out = np.zeros((n.value, 3, 3), np.float32)
        w = C.c_uint64()
        _check(self._lib.bf_mc_copy_vertices_to_host(self._h, out.ctypes.data_as(C.c_void_p), n.value, C.byref(w)))
        return out


def voxelize_mesh(triangles, resolution, samples_per_voxel: int = 64, model=None) -> np.ndarray:
    """MeshRasterizer3D::rasterize(mesh, target_texture, model_matrix) of the
    reference as a GPU ray-parity voxeliser (bf_voxelize_mesh): triangles
    (T, 3, 3) float32 mapped by `model` (4x4, column-major as glm; None =
    identity) into the cube [-1, 1]^3 spanning the volume -> uint8 mask
    (nz, ny, nx), 1 = solid."""
    lib = load_library()
    tri = np.ascontiguousarray(np.asarray(triangles, np.float32).reshape(-1))
    nx, ny, nz = (int(v) for v in resolution)
    mask = np.zeros(nx * ny * nz, np.uint8)
    res = (C.c_int32 * 3)(nx, ny, nz)
    m = None
    if model is not None:
        m = np.ascontiguousarray(np.asarray(model, np.float32).reshape(16))
    _check(lib.bf_voxelize_mesh(tri.ctypes.data_as(C.c_void_p), tri.size // 9,
                                None if m is None else m.ctypes.data_as(C.c_void_p), res, int(samples_per_voxel),
                                mask.ctypes.data_as(C.c_void_p)))
    return mask.reshape(nz, ny, nx)
