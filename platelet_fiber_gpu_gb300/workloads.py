"""Seeded synthetic workloads.

* `reference_case`   -- the reference's own setting at test size: one
  triangulated platelet, Bell-model receptor bonds, Zou/He shear walls on z,
  periodic x/y lattice, IBM periodic in y only (LB_kernel.cu:1483-1518).
* `plain_small`      -- 64x32x32 body-force Poiseuille channel with half-way
  bounce-back walls on y and z, one platelet of 400 membrane + 200 cytoplasm
  elements, Morse pairs, a 200-node / 400-link Hookean fibrin mesh.
* `single_large`     -- 256x128x128 shear channel (1000 1/s through the
  reference's unit chain), 50 platelets x 600 elements placed by seeded
  dart-throwing Poisson-disk sampling, a 20k-node / 40k-link fibrin mesh on
  the bottom wall, 200 receptors per platelet with constant per-step bond
  probabilities 1e-2 / 1e-3.
* `mixed_small`      -- a scaled-down single_large for GPU parity tests.

Lengths are in microns with the reference's lattice spacing dx = 0.2 um
(Input/parameter.dat DELTA_X); the platelet ellipsoid has semi-axes
1.0 x 1.0 x 0.5 um.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import mesh as M
from .scene import (BC_BOUNCEBACK, BC_INOUT, BC_PERIODIC, BC_ZOUHE_SHEAR, BOND_BELL, BOND_CONSTANT, FIB_HOOKE,
                    MEM_ALL, P_KF0, P_KR0, P_NUMRECEPTORS, Scene, force_to_lattice, reference_params)

REF_DX = 0.2
REF_DT = 1e-8


class PlateletTemplate:
    """One platelet in local coordinates: mesh vertices first, cytoplasm after."""

    def __init__(self, verts, tris, n_cyto: int, seed: int, axes):
        self.verts = np.asarray(verts, dtype=np.float64)
        self.tris = np.asarray(tris, dtype=np.int32)
        self.n_membrane = len(self.verts)
        rng = np.random.default_rng(seed)
        pts = []
        a = np.asarray(axes, dtype=np.float64) * 0.85
        while len(pts) < n_cyto:
            q = rng.uniform(-1, 1, size=3)
            if q @ q <= 1.0:
                pts.append(q * a)
        self.cyto = np.array(pts, dtype=np.float64).reshape(-1, 3)
        self.n_elem = self.n_membrane + len(self.cyto)
        self.local = np.vstack([self.verts, self.cyto]) if len(self.cyto) else self.verts.copy()
        self.sp_ptr, self.sp_nbr, self.sp_L0 = M.edge_rest_lengths(self.verts, self.tris, self.n_elem)
        self.mean_bond = M.mean_bond_length(self.sp_L0, self.sp_ptr, self.sp_nbr)

    @classmethod
    def from_neu(cls, path, n_cyto: int, seed: int, axes):
        """A template whose membrane is the reference's NEU surface mesh (read
        by libpfgpu's NEU reader); `axes` bound the cytoplasm sampling."""
        from .gpu import read_neu
        m = read_neu(path)
        return cls(np.stack([m["X"], m["Y"], m["Z"]], 1), m["tri"], n_cyto, seed, axes)


def _place(scene: Scene, tpl: PlateletTemplate, centers: np.ndarray, ly_um: float):
    P = len(centers)
    E = tpl.n_elem
    X = np.zeros((P, E))
    Y = np.zeros((P, E))
    Z = np.zeros((P, E))
    for p, c in enumerate(centers):
        X[p] = tpl.local[:, 0] + c[0]
        Y[p] = tpl.local[:, 1] + c[1]
        Z[p] = tpl.local[:, 2] + c[2]
    RY = Y.copy()
    if scene.ibm_wrap[1]:
        Y = np.where(Y > ly_um, Y - ly_um, Y)
        Y = np.where(Y < 0, Y + ly_um, Y)
    topo = M.build_topology(tpl.tris, tpl.n_membrane, np.stack([X[0], RY[0], Z[0]], 1))
    S0 = np.zeros((P, len(tpl.tris)))
    S0_all = np.zeros(P)
    V0 = np.zeros(P)
    for p in range(P):
        S0[p], S0_all[p], V0[p] = M.rest_area_volume(tpl.tris, np.stack([X[p], RY[p], Z[p]], 1))
    scene.n_platelets, scene.n_elem, scene.n_membrane = P, E, tpl.n_membrane
    scene.tri, scene.node_ntri, scene.ring = topo.tri6, topo.node_ntri, topo.ring
    scene.spring_ptr, scene.spring_nbr, scene.spring_L0 = tpl.sp_ptr, tpl.sp_nbr, tpl.sp_L0
    scene.S0, scene.S0_all, scene.V0 = S0, S0_all, V0
    scene.X, scene.Y, scene.RY, scene.Z = X, Y, RY, Z
    scene.meta["topology"] = topo
    return topo


def _receptors_per_triangle(scene: Scene, R: int, rng):
    """R receptors on every triangle, tri-major (the reference's
    [SurfElem][numReceptorsPerElem] layout, gpuSEM_LB.c:732-747)."""
    T = scene.n_tri
    P = scene.n_platelets
    scene.n_rec = T * R
    scene.rec_tri = np.tile(np.repeat(np.arange(T, dtype=np.int32), R), (P, 1))
    scene.rec_r1 = rng.uniform(size=(P, T * R)).astype(np.float32)
    scene.rec_r2 = rng.uniform(size=(P, T * R)).astype(np.float32)


def _receptors_random(scene: Scene, n_rec: int, rng):
    P, T = scene.n_platelets, scene.n_tri
    scene.n_rec = n_rec
    tri = rng.integers(0, T, size=(P, n_rec)).astype(np.int32)
    scene.rec_tri = np.sort(tri, axis=1)
    scene.rec_r1 = rng.uniform(size=(P, n_rec)).astype(np.float32)
    scene.rec_r2 = rng.uniform(size=(P, n_rec)).astype(np.float32)


def _fibrin(scene: Scene, n_nodes: int, n_links: int, slab: float, rng, k: float):
    """Nodes uniform in the wall slab z in [0, slab); links by nearest-neighbour
    pairing (the n_links shortest distinct pairs among each node's 6 nearest
    neighbours); rest length = initial length; nodes within one dx of the
    wall are fixed (the rule of fiber.cpp:380-384 on the wall-normal axis)."""
    from scipy.spatial import cKDTree

    if n_nodes == 0:
        scene.n_fib = 0
        return
    Lx, Ly = scene.nx * scene.dx, scene.ny * scene.dx
    pts = np.stack([rng.uniform(0, Lx, n_nodes), rng.uniform(0, Ly, n_nodes),
                    rng.uniform(0, slab, n_nodes)], 1)
    tree = cKDTree(pts)
    kk = min(7, n_nodes)
    d, idx = tree.query(pts, k=kk)
    pairs = {}
    for i in range(n_nodes):
        for q in range(1, kk):
            j = int(idx[i, q])
            key = (min(i, j), max(i, j))
            if key not in pairs:
                pairs[key] = float(d[i, q])
    items = sorted(pairs.items(), key=lambda t: (t[1], t[0]))[:n_links]
    links = np.array([p for p, _ in items], dtype=np.int32).reshape(-1, 2)
    nbr = [[] for _ in range(n_nodes)]
    for a, b in links:
        nbr[a].append(int(b))
        nbr[b].append(int(a))
    ptr = np.zeros(n_nodes + 1, dtype=np.int32)
    cols, L0 = [], []
    for i in range(n_nodes):
        ptr[i + 1] = ptr[i] + len(nbr[i])
        for j in nbr[i]:
            cols.append(j)
            dd = pts[i] - pts[j]
            L0.append(float(np.sqrt(dd @ dd)))
    scene.n_fib = n_nodes
    scene.fib_X, scene.fib_Y, scene.fib_Z = pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy()
    scene.fib_fixed = (pts[:, 2] < scene.dx).astype(np.int32)
    scene.fib_ptr = ptr
    scene.fib_nbr = np.array(cols, dtype=np.int32)
    scene.fib_L0 = np.array(L0, dtype=np.float64)
    scene.fib_law = FIB_HOOKE
    scene.fib_k = k
    scene.meta["fib_links"] = links


def poisson_disk(n: int, lo, hi, rmin: float, rng, fixed_z=None, n_fixed=0, max_tries=200000):
    """Dart-throwing Poisson-disk sampling of `n` centres in the box [lo, hi)
    with pairwise distance >= rmin; the first `n_fixed` darts have z=fixed_z."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    pts = []
    tries = 0
    while len(pts) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("poisson_disk: domain too small for the requested count")
        c = rng.uniform(lo, hi)
        if len(pts) < n_fixed:
            c[2] = fixed_z
        if all(np.linalg.norm(c - q) >= rmin for q in pts):
            pts.append(c)
    return np.array(pts)


# ---------------------------------------------------------------- workloads
def reference_case(seed: int = 7, nx=16, ny=20, nz=10, level=1, R=2, center=None,
                   kf0=3.0e4, kr0=1.5e4, mesh=None) -> Scene:
    """The reference's own path at test size (bond rates stressed so that
    binding happens within tens of steps).  `mesh`: (vertices, triangles)
    of the platelet surface, e.g. the reference's own NEU mesh; default a
    level-`level` icosphere ellipsoid 0.6 x 0.6 x 0.3 um."""
    rng = np.random.default_rng(seed)
    if mesh is None:
        v, t = M.ellipsoid_icosphere(level, axes=(0.6, 0.6, 0.3))
        half_z = 0.3
    else:
        v, t = np.asarray(mesh[0], dtype=np.float64), np.asarray(mesh[1], dtype=np.int32)
        half_z = float(0.5 * (v[:, 2].max() - v[:, 2].min()))
    axes = tuple(float(a) for a in 0.5 * (v.max(0) - v.min(0)))
    tpl = PlateletTemplate(v, t, 0, seed, axes)
    T = len(t)
    params = reference_params(dx=REF_DX, dt=REF_DT, nz=nz, shear=300.0, receptors=2 * R * T,
                              mean_bond=tpl.mean_bond, kf0=kf0, kr0=kr0)
    sc = Scene(nx=nx, ny=ny, nz=nz, dx=REF_DX, dt=REF_DT, params=params,
               bc=(BC_PERIODIC, BC_PERIODIC, BC_ZOUHE_SHEAR), ibm_wrap=(0, 1, 0))
    if center is None:
        center = (nx * REF_DX / 2, ny * REF_DX / 2, half_z + 0.05)
    _place(sc, tpl, np.array([center]), ny * REF_DX)
    _receptors_per_triangle(sc, R, rng)
    sc.bond_model = BOND_BELL
    sc.membrane_forces = MEM_ALL
    sc.seed = seed
    sc.meta["R"] = R
    return sc


def plain_small(seed: int = 1, n_membrane=400, n_cyto=200, n_fib=200, n_links=400,
                nx=64, ny=32, nz=32, g_lattice=2e-5) -> Scene:
    rng = np.random.default_rng(seed)
    axes = (1.0, 1.0, 0.5)
    v, t = M.ellipsoid_fibonacci(n_membrane, axes, seed)
    tpl = PlateletTemplate(v, t, n_cyto, seed, axes)
    tau = 0.8
    nu = 1.2e6 / 1.0239
    dt = float(np.float32((tau - 0.5) * REF_DX * REF_DX / (3 * nu)))
    umax = float(np.float32(REF_DX) / np.float32(dt))
    params = reference_params(dx=REF_DX, dt=dt, nz=nz, shear=0.0, mean_bond=tpl.mean_bond, umax=umax,
                              tau=tau, receptors=0.0)
    sc = Scene(nx=nx, ny=ny, nz=nz, dx=REF_DX, dt=dt, params=params,
               bc=(BC_PERIODIC, BC_BOUNCEBACK, BC_BOUNCEBACK), ibm_wrap=(1, 0, 0))
    fx = g_lattice / force_to_lattice(params, REF_DX, dt)
    sc.body_force = (fx, 0.0, 0.0)
    _place(sc, tpl, np.array([(nx * REF_DX / 2, ny * REF_DX / 2, nz * REF_DX / 2)]), ny * REF_DX)
    sc.morse = 1
    sc.n_rec = 0
    _fibrin(sc, n_fib, n_links, 3 * REF_DX, rng, 0.5)
    sc.seed = seed
    sc.meta.update(workload="plain_small", tau=tau, g_lattice=g_lattice)
    return sc


def single_large(seed: int = 2, nx=256, ny=128, nz=128, n_platelets=50, n_membrane=400, n_cyto=200,
                 n_fib=20000, n_links=40000, n_rec=200, shear=1000.0, n_wall=10) -> Scene:
    rng = np.random.default_rng(seed)
    axes = (1.0, 1.0, 0.5)
    v, t = M.ellipsoid_fibonacci(n_membrane, axes, seed)
    tpl = PlateletTemplate(v, t, n_cyto, seed, axes)
    params = reference_params(dx=REF_DX, dt=REF_DT, nz=nz, shear=shear, mean_bond=tpl.mean_bond)
    sc = Scene(nx=nx, ny=ny, nz=nz, dx=REF_DX, dt=REF_DT, params=params,
               bc=(BC_PERIODIC, BC_PERIODIC, BC_ZOUHE_SHEAR), ibm_wrap=(1, 1, 0))
    L = np.array([nx, ny, nz]) * REF_DX
    rmin = 2 * axes[0] + 2 * REF_DX
    centers = poisson_disk(n_platelets, (axes[0], axes[1], axes[2] + 0.05),
                           (L[0] - axes[0], L[1] - axes[1], L[2] - axes[2] - 0.6), rmin, rng,
                           fixed_z=axes[2] + 0.05, n_fixed=min(n_wall, n_platelets))
    _place(sc, tpl, centers, L[1])
    _receptors_random(sc, n_rec, rng)
    sc.params[P_NUMRECEPTORS] = n_rec * n_platelets
    sc.bond_model = BOND_CONSTANT
    sc.p_on, sc.p_off = 1e-2, 1e-3
    sc.morse = 1
    _fibrin(sc, n_fib, n_links, 3 * REF_DX, rng, 0.5)
    sc.seed = seed
    sc.meta.update(workload="single_large", shear=shear)
    return sc


def from_reference_inputs(parameter_file, nx: int, ny: int, nz: int, neu_path=None, centers=None,
                          n_fib: int = 0, n_links: int = 0, n_wall: int = 0) -> Scene:
    """A scene from the reference driver's own inputs: `Input/parameter.dat`
    (read by libpfgpu's ParReader restatement) and the NEU surface mesh it
    names (NEUReader restatement).  The file sets dx, dt, the shear rate, the
    initial density, the spring constant, Kr0, the receptor total and the seed
    of the parameter table (gpuSEM_LB.c:1206-1233), the cell count
    (MAX_CELL) and the elements per cell (MAX_ELEM: the mesh's vertices, then
    cytoplasm).  Cell positions: `centers` (um, shape [MAX_CELL][3], added to
    the mesh coordinates), else for one cell the driver's own offset of the
    mesh, (8.0, 1.5, 0.32) um (gpuSEM_LB.c:811-820; its PDB and PSF readers
    are commented out at :810, :1060), else a seeded Poisson-disk placement
    above the bottom wall.  `neu_path` defaults to the file's NEU_PATH,
    relative to the directory holding Input/."""
    from .gpu import read_neu, read_parameter_file
    par = Path(parameter_file)
    p = read_parameter_file(par)
    neu = Path(neu_path) if neu_path is not None else Path(p["neu_path"])
    if not neu.is_absolute() and not neu.exists():
        neu = par.resolve().parent.parent / neu
    hp = p["host_param"]
    seed = int(hp[1])
    n_cells = int(p["max_cell"])
    m = read_neu(neu)
    verts = np.stack([m["X"], m["Y"], m["Z"]], 1)
    n_cyto = max(0, int(p["max_elem"]) - len(verts))
    axes = tuple(float(a) for a in 0.5 * (verts.max(0) - verts.min(0)))
    tpl = PlateletTemplate(verts, m["tri"], n_cyto, seed, axes)
    dx, dt = float(p["dx"]), float(p["dt"])
    params = reference_params(dx=dx, dt=dt, nz=nz, shear=float(hp[5]), rho0=float(hp[6]), k_spring=float(hp[2]),
                              kr0=float(hp[4]), receptors=float(hp[0]), seed=float(hp[1]),
                              mean_bond=tpl.mean_bond)
    sc = Scene(nx=nx, ny=ny, nz=nz, dx=dx, dt=dt, params=params,
               bc=(BC_PERIODIC, BC_PERIODIC, BC_ZOUHE_SHEAR), ibm_wrap=(1, 1, 0))
    rng = np.random.default_rng(seed)
    L = np.array([nx, ny, nz]) * dx
    if centers is None and n_cells == 1:
        centers = [(8.0, 1.5, 0.32)]
    if centers is None:
        rmin = 2 * max(axes[0], axes[1]) + 2 * dx
        centers = poisson_disk(n_cells, (axes[0], axes[1], axes[2] + 0.05),
                               (L[0] - axes[0], L[1] - axes[1], L[2] - axes[2] - 0.6), rmin, rng,
                               fixed_z=axes[2] + 0.05, n_fixed=min(n_wall, n_cells))
    centers = np.asarray(centers, dtype=np.float64).reshape(-1, 3)
    if len(centers) != n_cells:
        raise ValueError(f"{len(centers)} centers for MAX_CELL = {n_cells}")
    _place(sc, tpl, centers, L[1])
    n_rec = int(round(float(hp[0]))) // max(1, n_cells)
    _receptors_random(sc, n_rec, rng)
    sc.params[P_NUMRECEPTORS] = n_rec * n_cells
    sc.morse = 1
    if n_fib:
        _fibrin(sc, n_fib, n_links, 3 * dx, rng, 0.5)
    sc.seed = seed
    sc.meta.update(workload="reference_inputs", parameter_file=str(par), neu=str(neu))
    return sc


def mixed_large(seed: int = 5) -> Scene:
    """The mixed-precision large case: single_large's scene scaled to a
    512x256x256 channel with 500 platelets and a 100k-node / 200k-link fibrin
    mesh on the bottom wall."""
    sc = single_large(seed=seed, nx=512, ny=256, nz=256, n_platelets=500, n_fib=100000, n_links=200000)
    sc.meta.update(workload="mixed_large")
    return sc


def mixed_small(seed: int = 3, nx=40, ny=32, nz=20, n_platelets=3, level=1, n_cyto=12, n_fib=300,
                n_links=600, n_rec=40, bell=False, wall_gap=0.05) -> Scene:
    """Every feature of single_large on a lattice the oracle steps in seconds.
    Two platelets sit `wall_gap` um above the bottom wall (receptors within
    the 0.078 um bond range of it can bind)."""
    rng = np.random.default_rng(seed)
    axes = (0.6, 0.6, 0.3)
    v, t = M.ellipsoid_icosphere(level, axes)
    tpl = PlateletTemplate(v, t, n_cyto, seed, axes)
    params = reference_params(dx=REF_DX, dt=REF_DT, nz=nz, shear=1000.0, mean_bond=tpl.mean_bond,
                              kf0=3.0e4 if bell else None, kr0=1.5e4 if bell else 3.21,
                              receptors=float(n_rec * n_platelets))
    sc = Scene(nx=nx, ny=ny, nz=nz, dx=REF_DX, dt=REF_DT, params=params,
               bc=(BC_PERIODIC, BC_PERIODIC, BC_ZOUHE_SHEAR), ibm_wrap=(1, 1, 0))
    L = np.array([nx, ny, nz]) * REF_DX
    centers = poisson_disk(n_platelets, (axes[0], axes[1], axes[2] + 0.05),
                           (L[0] - axes[0], L[1] - axes[1], L[2] - axes[2] - 0.3), 2 * axes[0] + 2 * REF_DX,
                           rng, fixed_z=axes[2] + wall_gap, n_fixed=min(2, n_platelets))
    _place(sc, tpl, centers, L[1])
    _receptors_random(sc, n_rec, rng)
    if bell:
        sc.bond_model = BOND_BELL
    else:
        sc.bond_model = BOND_CONSTANT
        sc.p_on, sc.p_off = 0.2, 0.05
    sc.morse = 1
    sc.morse_intra = (1.0, 2.0, 0.3, 0.6)
    sc.morse_inter = (1.0, 2.0, 0.3, 0.6)
    _fibrin(sc, n_fib, n_links, 3 * REF_DX, rng, 0.5)
    sc.seed = seed
    sc.meta.update(workload="mixed_small")
    return sc


def inflow_small(seed: int = 3, **kw) -> Scene:
    """mixed_small with the y axis open: the velocity inlet at y=0 and outlet
    at y=ny-1 (BC_INOUT, the reference's in/out-flow planes) carrying the
    same shear profile as the initial flow, and no IBM wrap across them."""
    sc = mixed_small(seed=seed, **kw)
    sc.bc = (BC_PERIODIC, BC_INOUT, BC_ZOUHE_SHEAR)
    sc.ibm_wrap = (1, 0, 0)
    sc.meta.update(workload="inflow_small")
    return sc


_BATCH_TEMPLATE = {}


def _batch_template(seed: int):
    if seed not in _BATCH_TEMPLATE:
        axes = (1.0, 1.0, 0.5)
        v, t = M.ellipsoid_fibonacci(400, axes, seed)
        _BATCH_TEMPLATE[seed] = PlateletTemplate(v, t, 200, seed, axes)
    return _BATCH_TEMPLATE[seed]


def batch_job(seed: int, index: int, steps_range=None) -> Scene:
    """One job of the many-job workload: node count log-uniform in
    [32^3, 128*64*64] with aspect 2:1:1 rounded to multiples of 8, 1-8
    platelets (as many as fit) of the single_large template, 1k-5k fibrin
    nodes on the bottom wall, shear uniform in [100, 2000] 1/s, 200 receptors
    per platelet with constant per-step probabilities 1e-2 / 1e-3.  The job's
    own stream of draws is seeded by (seed, index)."""
    rng = np.random.default_rng([seed, index])
    nodes = float(np.exp(rng.uniform(np.log(32 ** 3), np.log(128 * 64 * 64))))
    a = max(16, int(round((nodes / 2) ** (1 / 3) / 8)) * 8)
    nx, ny, nz = 2 * a, a, a
    tpl = _batch_template(seed)
    axes = (1.0, 1.0, 0.5)
    shear = float(rng.uniform(100.0, 2000.0))
    params = reference_params(dx=REF_DX, dt=REF_DT, nz=nz, shear=shear, mean_bond=tpl.mean_bond)
    sc = Scene(nx=nx, ny=ny, nz=nz, dx=REF_DX, dt=REF_DT, params=params,
               bc=(BC_PERIODIC, BC_PERIODIC, BC_ZOUHE_SHEAR), ibm_wrap=(1, 1, 0))
    L = np.array([nx, ny, nz]) * REF_DX
    rmin = 2 * axes[0] + 2 * REF_DX
    want = int(rng.integers(1, 9))
    fit = max(1, int(np.prod(L - np.array([2 * axes[0], 2 * axes[1], 2 * axes[2] + 0.65])) / rmin ** 3 // 2))
    n_pl = min(want, fit)
    centers = poisson_disk(n_pl, (axes[0], axes[1], axes[2] + 0.05),
                           (L[0] - axes[0], L[1] - axes[1], L[2] - axes[2] - 0.6), rmin, rng,
                           fixed_z=axes[2] + 0.05, n_fixed=1)
    _place(sc, tpl, centers, L[1])
    _receptors_random(sc, 200, rng)
    sc.params[P_NUMRECEPTORS] = 200 * len(centers)
    sc.bond_model = BOND_CONSTANT
    sc.p_on, sc.p_off = 1e-2, 1e-3
    sc.morse = 1
    n_fib = int(rng.integers(1000, 5001))
    _fibrin(sc, n_fib, 2 * n_fib, 3 * REF_DX, rng, 0.5)
    sc.seed = (seed << 20) + index
    sc.meta.update(workload="batch_job", shear=shear, index=index)
    if steps_range is not None:
        sc.meta["steps"] = int(rng.integers(steps_range[0], steps_range[1] + 1))
    return sc
