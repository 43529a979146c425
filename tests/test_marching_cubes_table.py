"""Marching-cubes case table and the oracle's mesh properties (CPU only):
the library's derived table equals the oracle's independent derivation, and
the oracle's surface of a sphere is closed, outward oriented and encloses the
sphere's volume."""
from collections import Counter

import numpy as np

from oracle.marching_cubes import case_table, extract


def sphere_field(n, r):
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    c = (n - 1) / 2.0
    return (r - np.sqrt((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2)).astype(np.float32).reshape(-1)


def test_library_table_matches_oracle_derivation(product_lib):
    from boltzmannfluids_gb300.marching_cubes import case_table as lib_table
    tri, cnt = lib_table()
    ref = case_table()
    for cs in range(256):
        assert cnt[cs] == len(ref[cs]), cs
        got = [tuple(int(v) for v in tri[cs, 3 * t:3 * t + 3]) for t in range(cnt[cs])]
        assert got == [tuple(t) for t in ref[cs]], cs
        assert np.all(tri[cs, 3 * cnt[cs]:] == -1)


def test_table_shape():
    t = case_table()
    assert len(t[0]) == 0 and len(t[255]) == 0
    assert max(len(x) for x in t) == 5
    # complementary cases cut the same edges
    for cs in range(256):
        e1 = sorted({e for tri in t[cs] for e in tri})
        e2 = sorted({e for tri in t[255 - cs] for e in tri})
        assert e1 == e2, cs


def test_oracle_sphere_is_closed_oriented_and_has_the_sphere_volume():
    n, r = 24, 7.0
    tris = extract(sphere_field(n, r), (n, n, n), 0.0)
    p = (tris.astype(np.float64) + 0.5) * n  # back to lattice units
    vol = np.sum(np.einsum("ij,ij->i", p[:, 0], np.cross(p[:, 1], p[:, 2]))) / 6.0
    assert abs(vol - 4.0 / 3.0 * np.pi * r ** 3) / (4.0 / 3.0 * np.pi * r ** 3) < 0.03
    edges = Counter()
    for t in np.round(p, 5):
        for i in range(3):
            edges[(tuple(t[i]), tuple(t[(i + 1) % 3]))] += 1
    for (a, b), c in edges.items():
        assert c == 1 and edges.get((b, a)) == 1
