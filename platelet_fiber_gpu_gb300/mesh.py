"""Membrane meshes and the reference driver's topology build.

`build_topology` restates the host-side mesh preprocessing of the reference
driver (gpuSEM_LB.c:846-1055): edge-midpoint virtual nodes appended to each
triangle, the node -> triangle table, ring-ordered vertex neighbours, the
reference normals and the rest areas / volume.  `edge_rest_lengths` restates
the bond table the mesh reader fills (gpuSEM_LB.c:346-404, NEUReader).

The mesh generators are this package's own: an ellipsoidal icosphere for
small test cases and a Fibonacci-lattice ellipsoid (convex hull) with a chosen
vertex count for the benchmark platelets.
"""
from __future__ import annotations

import numpy as np


def orient_inward(verts: np.ndarray, tris: np.ndarray) -> np.ndarray:
    """Orders every triangle so (v1-v0)x(v2-v0) points towards the centroid.

    The reference's element normal is -(e12 x e13)/|e12 x e13|
    (sem_kernel.cu:797-803) and its volume sum is positive for closed meshes
    wound this way (gpuSEM_LB.c:1037-1050)."""
    tris = np.array(tris, dtype=np.int32, copy=True)
    c = verts.mean(axis=0)
    v0, v1, v2 = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
    n = np.cross(v1 - v0, v2 - v0)
    out = np.einsum("ij,ij->i", n, (v0 + v1 + v2) / 3.0 - c) > 0
    tris[out, 1], tris[out, 2] = tris[out, 2].copy(), tris[out, 1].copy()
    return tris


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere with `level` loop subdivisions."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
         (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int32)


def ellipsoid_icosphere(level: int, axes=(1.0, 1.0, 0.5)) -> tuple[np.ndarray, np.ndarray]:
    v, f = icosphere(level)
    v = v * np.asarray(axes, dtype=np.float64)
    return v, orient_inward(v, f)


def ellipsoid_fibonacci(n: int, axes=(1.0, 1.0, 0.5), seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """`n` quasi-uniform vertices on an ellipsoid (golden-angle spiral on the
    unit sphere under a seeded random rotation, scaled by the semi-axes),
    triangulated as their convex hull."""
    from scipy.spatial import ConvexHull

    rng = np.random.default_rng(seed)
    k = np.arange(n) + 0.5
    zc = 1.0 - 2.0 * k / n
    r = np.sqrt(1.0 - zc * zc)
    phi = np.pi * (3.0 - 5 ** 0.5) * k
    p = np.stack([r * np.cos(phi), r * np.sin(phi), zc], axis=1)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    p = p @ q.T
    hull = ConvexHull(p)
    v = p * np.asarray(axes, dtype=np.float64)
    return v, orient_inward(v, hull.simplices.astype(np.int32))


def edge_rest_lengths(verts: np.ndarray, tris: np.ndarray, n_elem: int):
    """CSR of the membrane springs: for every triangle edge (a,b) the rest
    length |x_a - x_b| (the bond table of NEUReader, gpuSEM_LB.c:381-403),
    rows ordered by ascending neighbour like the dense-table scan of
    sem_kernel.cu:355-389.  Elements beyond the mesh (cytoplasm) have none."""
    nb: list[dict[int, float]] = [dict() for _ in range(n_elem)]
    for a, b, c in tris[:, :3]:
        for u, w in ((a, b), (b, c), (c, a)):
            d = verts[u] - verts[w]
            dr = float(np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))
            nb[u][int(w)] = dr
            nb[w][int(u)] = dr
    ptr = np.zeros(n_elem + 1, dtype=np.int32)
    cols, vals = [], []
    for e in range(n_elem):
        items = sorted(nb[e].items())
        ptr[e + 1] = ptr[e] + len(items)
        cols += [k for k, _ in items]
        vals += [v for _, v in items]
    return ptr, np.array(cols, dtype=np.int32), np.array(vals, dtype=np.float64)


def dense_bond_lengths(ptr, cols, vals, n_elem: int) -> np.ndarray:
    b = np.zeros((n_elem, n_elem), dtype=np.float64)
    for e in range(n_elem):
        b[e, cols[ptr[e]:ptr[e + 1]]] = vals[ptr[e]:ptr[e + 1]]
    return b


class Topology:
    """Output of `build_topology` (field names follow the reference driver)."""

    def __init__(self, tri6, node_ntri, node_share, ring, newnode, N):
        self.tri6 = tri6
        self.node_ntri = node_ntri
        self.node_share = node_share
        self.ring = ring
        self.newnode = newnode
        self.N = N


def build_topology(tris: np.ndarray, n_vert: int, ref_xyz: np.ndarray) -> Topology:
    """Restates gpuSEM_LB.c:846-1020 (virtual nodes, node->triangle table,
    ring ordering, reference normals)."""
    T = len(tris)
    tri6 = -np.ones((T, 6), dtype=np.int32)
    tri6[:, :3] = tris[:, :3]
    newnode = n_vert
    # triangle pairs sharing an edge, in (i, j>i) order, numbered in that order
    edge_owner: dict[tuple[int, int], list[int]] = {}
    for i in range(T):
        a, b, c = (int(x) for x in tri6[i, :3])
        for u, w in ((a, b), (a, c), (b, c)):
            edge_owner.setdefault((min(u, w), max(u, w)), []).append(i)
    pairs: dict[int, list[int]] = {}
    for owners in edge_owner.values():
        if len(owners) == 2:
            i, j = sorted(owners)
            pairs.setdefault(i, []).append(j)
    slot_of = {1: 3, 2: 4, 3: 5}
    for i in range(T):
        for j in sorted(pairs.get(i, [])):
            f1 = f2 = match = 0
            for k in range(3):
                for l in range(3):
                    if tri6[i, k] == tri6[j, l]:
                        f1 += k
                        f2 += l
                        match += 1
            if match == 2:
                if f1 in slot_of:
                    tri6[i, slot_of[f1]] = newnode
                if f2 in slot_of:
                    tri6[j, slot_of[f2]] = newnode
                newnode += 1
    if T == 1:
        newnode += 3
        tri6[0, 3:6] = (3, 4, 5)
    share = -np.ones((newnode, 10), dtype=np.int32)
    ntri = np.zeros(newnode, dtype=np.int32)
    for i in range(T):
        for j in range(6):
            nd = int(tri6[i, j])
            if nd == -1:
                break
            if ntri[nd] >= 10:
                raise ValueError("more than 10 triangles share a node")
            share[nd, ntri[nd]] = i
            ntri[nd] += 1
    ring = -np.ones((n_vert, 10), dtype=np.int32)
    for i in range(n_vert):
        elem = share[i, 0]
        node_idx = -1
        for j in range(3):
            if tri6[elem, j] == i:
                node_idx = tri6[elem, 0] if j == 2 else tri6[elem, j + 1]
                ring[i, 0] = node_idx
        for j in range(1, ntri[i]):
            for k in range(j, ntri[i]):
                elem = share[i, k]
                hit = False
                for l in range(3):
                    if tri6[elem, l] == node_idx:
                        hit = True
                        node_idx = tri6[elem, 2] if l == 0 else tri6[elem, l - 1]
                        ring[i, j] = node_idx
                        break
                if hit:
                    share[i, j], share[i, k] = share[i, k], share[i, j]
                    break
    # reference normals (gpuSEM_LB.c:986-1020); only the vertex columns of
    # ref_xyz are read
    N = np.zeros((newnode, 3), dtype=np.float64)
    for i in range(newnode):
        for j in range(10):
            e = share[i, j]
            if e == -1:
                break
            c = ref_xyz[tri6[e, :3]]
            e12, e13 = c[1] - c[0], c[2] - c[0]
            n = np.array([e12[1] * e13[2] - e12[2] * e13[1], e12[2] * e13[0] - e12[0] * e13[2],
                          e12[0] * e13[1] - e12[1] * e13[0]])
            N[i] += n / np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
        if ntri[i]:
            N[i] /= ntri[i]
            N[i] /= -np.sqrt(N[i, 0] ** 2 + N[i, 1] ** 2 + N[i, 2] ** 2)
    return Topology(tri6, ntri, share, ring, newnode, N)


def rest_area_volume(tris: np.ndarray, xyz: np.ndarray):
    """Per-triangle rest area S0, total S0_all and volume V0
    (gpuSEM_LB.c:1021-1055, normal E13 x E12 and centroid-weighted volume)."""
    T = len(tris)
    S0 = np.zeros(T)
    S0_all = 0.0
    V0 = 0.0
    for i in range(T):
        c = xyz[tris[i, :3]]
        e12, e13 = c[1] - c[0], c[2] - c[0]
        cc = 1 / 3.0 * (c[0] + c[1] + c[2])
        n = np.array([e13[1] * e12[2] - e13[2] * e12[1], e13[2] * e12[0] - e13[0] * e12[2],
                      e13[0] * e12[1] - e13[1] * e12[0]])
        nn = np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
        n = n / nn
        S0[i] = 0.5 * nn
        S0_all += S0[i]
        V0 += 1 / 3.0 * (cc[0] * n[0] + cc[1] * n[1] + cc[2] * n[2]) * S0[i]
    return S0, S0_all, V0


def mean_bond_length(vals: np.ndarray, ptr: np.ndarray, cols: np.ndarray) -> float:
    """Mean over unordered bonded pairs (gpuSEM_LB.c:829-839)."""
    tot, cnt = 0.0, 0
    for e in range(len(ptr) - 1):
        for q in range(ptr[e], ptr[e + 1]):
            if cols[q] > e:
                tot += vals[q]
                cnt += 1
    return tot / max(cnt, 1)
