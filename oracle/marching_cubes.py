"""CPU restatement of the marching-cubes mesh extraction that
BoltzmannFluids' MarchingCubes (BoltzmannFluids/Source/MarchingCubes/
MarchingCubes.cpp:3-64, GLSL/MarchingCubes/marching_cubes.comp:41-97) sets out
to compute, for the product's CUDA kernels to be checked against.  TEST
INFRASTRUCTURE ONLY: the tests load this module as the checker; the product
never imports it.

The reference's shader cannot produce a mesh as written: MarchingCubes::compute
binds its uniforms but never dispatches (MarchingCubes.cpp:27-46), the shader
reads look_up_table[case_code] for every triangle instead of entry
case_code*5 + i and writes edge numbers as vertex indices
(marching_cubes.comp:88-96), and its corner bit order (:70-77) does not match
the corner numbering of its own table.  What it sets out to do is restated
here: a voxel between lattice nodes is classified by which of its eight corner
values are >= threshold, and the iso-surface crosses each edge whose corners
disagree, at the linearly interpolated position.  Vertex coordinates follow
the shader's mapping -0.5 + node / resolution, times mesh_scale (:52-53).

The case table is derived, not transcribed: corners k = (k&1, k>>1&1, k>>2&1);
edge 4d + j joins the j-th corner with bit d clear to its neighbour along d;
on each face the cut edges pair into segments, a face with two diagonal
inside corners cuts each inside corner off (the rule depends on the face
alone, so neighbouring voxels agree and the surface is closed); the segments
chain into loops, each loop is oriented so its normal points from the inside
corners to the outside ones, and is fanned into triangles from its first
edge.  Output order: voxels in x-fastest order, triangles in table order,
three vertices per triangle."""
import numpy as np

CORNERS = [(k & 1, (k >> 1) & 1, (k >> 2) & 1) for k in range(8)]
EDGES = [(c, c | (1 << d)) for d in range(3) for c in range(8) if not (c >> d) & 1]
_EDGE_ID = {e: i for i, e in enumerate(EDGES)}


def _edge(a, b):
    return _EDGE_ID[(min(a, b), max(a, b))]


def _faces():
    out = []
    for d in range(3):
        a, b = [x for x in range(3) if x != d]
        for side in (0, 1):
            base = side << d
            out.append([base, base | (1 << a), base | (1 << a) | (1 << b), base | (1 << b)])
    return out


def case_table():
    """-> list of 256 lists of (e0, e1, e2) edge triples."""
    faces = _faces()
    table = []
    for case in range(256):
        inside = [(case >> k) & 1 for k in range(8)]
        adj = {}
        for cyc in faces:
            ins = [inside[c] for c in cyc]
            es = [_edge(cyc[i], cyc[(i + 1) % 4]) for i in range(4)]
            cuts = [i for i in range(4) if ins[i] != ins[(i + 1) % 4]]
            if len(cuts) == 2:
                segs = [(es[cuts[0]], es[cuts[1]])]
            elif len(cuts) == 4:
                segs = [(es[(i - 1) % 4], es[i]) for i in range(4) if ins[i]]
            else:
                segs = []
            for a, b in segs:
                adj.setdefault(a, []).append(b)
                adj.setdefault(b, []).append(a)
        seen, tris = set(), []
        for start in sorted(adj):
            if start in seen:
                continue
            loop, prev, cur = [start], None, start
            seen.add(start)
            while True:
                nxt = adj[cur][0] if adj[cur][0] != prev else adj[cur][1]
                if nxt == start:
                    break
                loop.append(nxt)
                seen.add(nxt)
                prev, cur = cur, nxt
            # orientation: Newell normal of the edge midpoints against inside -> outside
            mid = [np.add(CORNERS[EDGES[e][0]], CORNERS[EDGES[e][1]]) / 2.0 for e in loop]
            nrm = sum(np.cross(mid[i], mid[(i + 1) % len(mid)]) for i in range(len(mid)))
            out_dir = np.zeros(3)
            for e in loop:
                a, b = EDGES[e]
                ia, ib = (a, b) if inside[a] else (b, a)
                out_dir += np.subtract(CORNERS[ib], CORNERS[ia])
            if float(np.dot(nrm, out_dir)) < 0:
                loop = loop[::-1]
            for i in range(1, len(loop) - 1):
                tris.append((loop[0], loop[i], loop[i + 1]))
        table.append(tris)
    return table


def extract(field, res, threshold, mesh_scale=(1.0, 1.0, 1.0)):
    """field: float32 array of nx*ny*nz node values (x fastest).
    -> float32 array (T, 3, 3) of triangle vertices."""
    nx, ny, nz = (int(v) for v in res)
    v = np.asarray(field, np.float32).reshape(nz, ny, nx)
    table = case_table()
    thr = np.float32(threshold)
    scale = np.asarray(mesh_scale, np.float32)
    resf = np.array([nx, ny, nz], np.float32)
    out = []
    for z in range(nz - 1):
        for y in range(ny - 1):
            for x in range(nx - 1):
                vals = [v[z + c[2], y + c[1], x + c[0]] for c in CORNERS]
                case = sum(1 << k for k in range(8) if vals[k] >= thr)
                for tri in table[case]:
                    tv = []
                    for e in tri:
                        a, b = EDGES[e]
                        d = (a ^ b).bit_length() - 1
                        t = np.float32(thr - vals[a]) / np.float32(vals[b] - vals[a])
                        p = np.array([x + CORNERS[a][0], y + CORNERS[a][1], z + CORNERS[a][2]], np.float32)
                        p[d] = np.float32(p[d] + t)
                        tv.append((np.float32(-0.5) + p / resf) * scale)
                    out.append(tv)
    return np.array(out, np.float32).reshape(-1, 3, 3)
