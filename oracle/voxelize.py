"""CPU restatement of the solid-voxel rasterisation of a closed triangle mesh
that BoltzmannFluids' MeshRasterizer3D performs through OpenGL
(BoltzmannFluids/Source/MeshRasterizer3D/MeshRasterizer3D.cpp:7-113: 64 depth
slabs per voxel layer, raster_unifier.comp:18-35 toggling a per-pixel
inside/outside parity, copy_to_3d.comp:18-26 writing the layer), for the
product's CUDA voxeliser to be checked against.  TEST INFRASTRUCTURE ONLY.

Restated as rays: one ray per voxel column through its centre along z; the
sorted depths where it crosses the mesh bound the inside intervals (an odd
count leaves the rest of the column inside); voxel k is solid when one of its
`samples` depth samples lies strictly inside.  A column centre on an edge is
owned by one triangle by the top-left rule after each triangle is made
counter-clockwise, and edge functions are evaluated from the lexicographically
smaller endpoint, so shared edges count once.  Coordinates: the model matrix
(column-major) maps the mesh into [-1, 1]^3, column i has its centre at
-1 + (2i+1)/nx, sample s of voxel k sits at -1 + 2(k + (s + 1/2)/samples)/nz.
Every arithmetic step is one float32 operation in the kernels' order."""
import math

import numpy as np

f32 = np.float32


def _edge_raw(ax, ay, bx, by, px, py):
    return f32(f32(f32(bx - ax) * f32(py - ay)) - f32(f32(by - ay) * f32(px - ax)))


def _edge(ax, ay, bx, by, px, py):
    if ax < bx or (ax == bx and ay < by):
        return _edge_raw(ax, ay, bx, by, px, py)
    return -_edge_raw(bx, by, ax, ay, px, py)


def _owns(ax, ay, bx, by):
    dx, dy = f32(bx - ax), f32(by - ay)
    return dy < 0 or (dy == 0 and dx < 0)


def transform(vertices, model=None):
    v = np.asarray(vertices, np.float32).reshape(-1, 3)
    m = np.eye(4, dtype=np.float32) if model is None else np.asarray(model, np.float32).reshape(4, 4).T  # column-major
    out = np.zeros_like(v)
    for n in range(len(v)):
        x, y, z = v[n]
        r = [f32(f32(f32(f32(m[row, 0] * x) + f32(m[row, 1] * y)) + f32(m[row, 2] * z)) + m[row, 3]) for row in range(4)]
        out[n] = [f32(r[0] / r[3]), f32(r[1] / r[3]), f32(r[2] / r[3])]
    return out.reshape(-1, 3, 3)


def voxelize(vertices, res, samples=64, model=None):
    nx, ny, nz = (int(v) for v in res)
    tris = transform(vertices, model)
    cols = [[] for _ in range(nx * ny)]
    hx, hy = f32(0.5 * nx), f32(0.5 * ny)
    for t in tris:
        (ax, ay, az), (bx, by, bz), (cx, cy, cz) = t
        area = _edge(ax, ay, bx, by, cx, cy)
        if not (area > 0 or area < 0):
            continue
        if area < 0:
            bx, by, bz, cx, cy, cz = cx, cy, cz, bx, by, bz
            area = -area
        minx, maxx = min(ax, bx, cx), max(ax, bx, cx)
        miny, maxy = min(ay, by, cy), max(ay, by, cy)
        i0 = max(math.ceil(f32(f32(f32(minx + f32(1)) * hx) - f32(0.5))), 0)
        i1 = min(math.floor(f32(f32(f32(maxx + f32(1)) * hx) - f32(0.5))), nx - 1)
        j0 = max(math.ceil(f32(f32(f32(miny + f32(1)) * hy) - f32(0.5))), 0)
        j1 = min(math.floor(f32(f32(f32(maxy + f32(1)) * hy) - f32(0.5))), ny - 1)
        oa, ob, oc = _owns(bx, by, cx, cy), _owns(cx, cy, ax, ay), _owns(ax, ay, bx, by)
        for j in range(j0, j1 + 1):
            py = f32(f32(f32(2 * j + 1) / f32(ny)) - f32(1))
            for i in range(i0, i1 + 1):
                px = f32(f32(f32(2 * i + 1) / f32(nx)) - f32(1))
                wa = _edge(bx, by, cx, cy, px, py)
                wb = _edge(cx, cy, ax, ay, px, py)
                wc = _edge(ax, ay, bx, by, px, py)
                if (wa > 0 or (wa == 0 and oa)) and (wb > 0 or (wb == 0 and ob)) and (wc > 0 or (wc == 0 and oc)):
                    z = f32(f32(f32(f32(wa * az) + f32(wb * bz)) + f32(wc * cz)) / area)
                    cols[i + nx * j].append(z)
    mask = np.zeros(nz * ny * nx, np.uint8)
    total = nz * samples
    hz = f32(0.5 * total)
    for col, ds in enumerate(cols):
        ds = sorted(ds)
        for a in range(0, len(ds), 2):
            lo = ds[a]
            hi = ds[a + 1] if a + 1 < len(ds) else f32(3)
            t0 = max(math.floor(f32(f32(f32(lo + f32(1)) * hz) - f32(0.5))) + 1, 0)
            t1 = min(math.ceil(f32(f32(f32(hi + f32(1)) * hz) - f32(0.5))) - 1, total - 1)
            if t0 > t1:
                continue
            for k in range(t0 // samples, t1 // samples + 1):
                mask[col + k * nx * ny] = 1
    return mask


def icosphere(subdivisions=2, radius=1.0, center=(0.0, 0.0, 0.0)):
    """Closed, consistently oriented triangle mesh of a sphere -> float32 (T, 3, 3)."""
    t = (1.0 + 5 ** 0.5) / 2
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, float) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
             (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache, nf = {}, []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    v = np.array(verts) * radius + np.asarray(center)
    return v[np.array(faces)].astype(np.float32)
