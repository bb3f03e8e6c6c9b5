"""Shared test matrices (small, seeded)."""
from __future__ import annotations

import numpy as np

from openph_gb300 import complexes as cx
from openph_gb300.complexes import BoundaryMatrix


def triangle():
    """The filled triangle: v1 v2 v3, e12 e13 e23, t (1-based low 0 0 0 2 3 0 6)."""
    return BoundaryMatrix.from_columns([[], [], [], [0, 1], [0, 2], [1, 2], [3, 4, 5]])


def empty_columns(m=5):
    return BoundaryMatrix.from_columns([[] for _ in range(m)])


def random_complex(n_vertices, p_edge, p_tri, seed):
    """A random filtered 2-complex (flag-free): random edges, random triangles
    whose three edges exist, in a random valid filtration order."""
    rng = np.random.default_rng(seed)
    V = list(range(n_vertices))
    edges = [(a, b) for a in V for b in V if a < b and rng.random() < p_edge]
    es = set(edges)
    tris = [(a, b, c) for a in V for b in V for c in V if a < b < c and (a, b) in es and (a, c) in es
            and (b, c) in es and rng.random() < p_tri]
    # filtration value: random for vertices/edges, then cofaces after faces
    val = {}
    for v in V:
        val[(v,)] = rng.random() * 0.1
    for e in edges:
        val[e] = max(val[(e[0],)], val[(e[1],)]) + rng.random()
    for t in tris:
        val[t] = max(val[(t[0], t[1])], val[(t[0], t[2])], val[(t[1], t[2])]) + rng.random()
    simplices = sorted(val, key=lambda s: (val[s], len(s), s))
    pos = {s: i for i, s in enumerate(simplices)}
    cols = []
    for s in simplices:
        if len(s) == 1:
            cols.append([])
        else:
            cols.append(sorted(pos[f] for f in (tuple(x for x in s if x != y) for y in s)))
    return BoundaryMatrix.from_columns(cols)


def simplex_skeleton(n_vertices, seed, max_dim=None):
    """Every face of the (n_vertices - 1)-simplex up to max_dim (all of them by
    default), in a lower-star order: a random value per vertex, a simplex
    valued by its largest vertex, ties by dimension then vertex tuple.
    Columns have up to max_dim + 1 rows."""
    from itertools import combinations
    rng = np.random.default_rng(seed)
    vv = rng.random(n_vertices)
    top = n_vertices if max_dim is None else max_dim + 1
    simplices = [c for k in range(1, top + 1) for c in combinations(range(n_vertices), k)]
    simplices.sort(key=lambda s: (max(vv[list(s)]), len(s), s))
    pos = {s: i for i, s in enumerate(simplices)}
    cols = []
    for s in simplices:
        cols.append([] if len(s) == 1 else sorted(pos[s[:y] + s[y + 1:]] for y in range(len(s))))
    return BoundaryMatrix.from_columns(cols)


def small_cases():
    out = {
        "triangle": triangle(),
        "empty5": empty_columns(5),
        "rips_cube_12": cx.rips_cube(12, seed=3),
        "rips_circle_16": cx.rips_mixed(16, seed=7),
        "lower_star_8x8": cx.lower_star_image(8, 8, seed=4, sigma=1.0),
    }
    for s in range(3):
        out[f"random_{s}"] = random_complex(14, 0.5, 0.6, seed=100 + s)
    out["simplex_6d"] = simplex_skeleton(7, seed=11)          # columns of up to 7 rows
    out["skeleton_4d_of_9"] = simplex_skeleton(9, seed=12, max_dim=4)
    return out


def anti_transpose(bm):
    """D' with entry (m-1-j, m-1-i) for every entry (i, j) of D, rows
    ascending (column m-1-i of D' lists the columns of D holding row i)."""
    m = bm.m
    cols = [[] for _ in range(m)]
    for j in range(m - 1, -1, -1):
        for i in bm.column(j):
            cols[m - 1 - int(i)].append(m - 1 - j)
    return BoundaryMatrix.from_columns(cols)


def mixed_buckets():
    """A matrix whose columns of three rows take them from two buckets (the
    triangle's edges, and three vertices), so its buckets are not graded."""
    return BoundaryMatrix.from_columns([[], [], [], [0, 1], [0, 2], [1, 2], [3, 4, 5], [0, 1, 2]])


def lower_star_volume(n, seed, sigma=1.5):
    """The lower-star filtration of a smoothed random n x n x n volume on its
    Freudenthal triangulation (each grid cube cut into six tetrahedra along
    its main diagonal): a simplex valued by its largest vertex, ties by
    dimension then vertex tuple.  Every triangle has at most two
    tetrahedra, edges and triangles have many cofaces."""
    from itertools import combinations, permutations
    rng = np.random.default_rng(seed)
    f = rng.standard_normal((n, n, n))
    if sigma > 0:  # separable box-blur passes, a cheap smoothing
        for ax in range(3):
            for _ in range(int(sigma * 2)):
                f = (f + np.roll(f, 1, axis=ax) + np.roll(f, -1, axis=ax)) / 3.0
    val = f.ravel() + rng.random(n ** 3) * 1e-9
    vid = lambda x, y, z: (x * n + y) * n + z
    tets = set()
    for x in range(n - 1):
        for y in range(n - 1):
            for z in range(n - 1):
                for perm in permutations(range(3)):
                    p = [x, y, z]
                    vs = [vid(*p)]
                    for ax in perm:
                        p[ax] += 1
                        vs.append(vid(*p))
                    tets.add(tuple(sorted(vs)))
    simplices = set((v,) for v in range(n ** 3))
    for t in tets:
        for k in (2, 3, 4):
            simplices.update(combinations(t, k))
    simplices = sorted(simplices, key=lambda s: (max(val[list(s)]), len(s), s))
    pos = {s: i for i, s in enumerate(simplices)}
    cols = [[] if len(s) == 1 else sorted(pos[s[:y] + s[y + 1:]] for y in range(len(s))) for s in simplices]
    return BoundaryMatrix.from_columns(cols)
