"""Generates the golden vectors of tests/golden/*.npz from the reference itself.

The reference's own CUDA kernel sources (LB_kernel.cu + sem_kernel.cu) are
compiled with g++ through the serial CUDA emulation of oracle/refemu and run
in the per-step launch order of semLB.cu (see oracle/refemu/refemu.cpp for
the three documented substitutions).  Each fixture stores the complete input
scene and the reference's state after `nsteps` coupled steps, so the tests
can rebuild the case without the reference tree.

Run in a checkout with the reference tree beside it (or at $PF_REFERENCE_DIR):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import binding as ob  # noqa: E402
from platelet_fiber_gpu_gb300 import mesh as M  # noqa: E402
from platelet_fiber_gpu_gb300 import workloads as W  # noqa: E402
from platelet_fiber_gpu_gb300.scene import MEM_ALL, MEM_FEMBEND, P_SHEAR, scene_to_dict  # noqa: E402

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0], dtype=np.float64)
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1], dtype=np.float64)
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1], dtype=np.float64)
W19 = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)

dp, ip, fp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_float)


class RefCase(C.Structure):
    _fields_ = [("lx", C.c_int), ("ly", C.c_int), ("lz", C.c_int), ("dx", C.c_float), ("dt", C.c_float),
                ("params", C.c_float * 100),
                ("fIN", dp), ("fOUT", dp), ("ux", dp), ("uy", dp), ("uz", dp), ("rho", dp), ("obst", fp),
                ("Fx", dp), ("Fy", dp), ("Fz", dp), ("vWF", ip),
                ("maxE", C.c_int), ("surf", C.c_int), ("newnode", C.c_int), ("R", C.c_int),
                ("X", dp), ("Y", dp), ("RY", dp), ("Z", dp), ("VX", dp), ("VY", dp), ("VZ", dp),
                ("FX", dp), ("FY", dp), ("FZ", dp), ("bondLengths", dp), ("triElem", ip),
                ("r1", fp), ("r2", fp), ("node_nbrElemNum", ip), ("node_nbr_nodes", ip), ("Nref", dp),
                ("S0", dp), ("S0_all", C.c_double), ("V0", C.c_double), ("receptBond", ip),
                ("nsteps", C.c_int), ("uniforms", dp), ("totalBond_per_step", ip), ("traj", dp),
                ("km_out", dp), ("S_all_V_out", dp), ("first_lost_site_step", C.c_int),
                ("fem_bend", C.c_int)]


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def reference_initial_lattice(sc):
    """Initial shear-flow equilibrium exactly as gpuSEM_LB.c:1206-1258 forms it."""
    nx, ny, nz = sc.nx, sc.ny, sc.nz
    shear = float(sc.params[P_SHEAR])
    dxf, dtf = np.float32(sc.dx), np.float32(sc.dt)
    umax = shear * (nz - 1) * float(dxf)
    c = float(np.float32(dxf / dtf)) / umax
    c2 = c * c
    k = np.arange(nz, dtype=np.float64)[:, None, None] * np.ones((nz, ny, nx))
    ux = np.zeros((nz, ny, nx))
    uy = shear * k * float(dxf) / umax
    uz = np.zeros((nz, ny, nx))
    rho = np.ones((nz, ny, nx))
    f = np.zeros((19, nz, ny, nx))
    for d in range(19):
        cu = 3.0 * (CX[d] * ux + CY[d] * uy + CZ[d] * uz)
        f[d] = rho * W19[d] * (1.0 + cu / c + 0.5 * cu * cu / c2 - 1.5 * (ux * ux + uy * uy + uz * uz) / c2)
    return f.reshape(19, -1), ux.ravel(), uy.ravel(), uz.ravel(), rho.ravel()


def run_reference(sc, nsteps: int):
    lib = C.CDLL(str(ob.build_refemu()))
    lib.refemu_run.argtypes = [C.POINTER(RefCase)]
    lib.refemu_run.restype = C.c_int
    N = sc.n_nodes
    E, T, NN = sc.n_elem, sc.n_tri, sc.n_node
    R = sc.n_rec // T
    f, ux, uy, uz, rho = reference_initial_lattice(sc)
    fIN = f.copy()
    fOUT = np.zeros_like(fIN)
    ux0, uy0, uz0, rho0 = ux.copy(), uy.copy(), uz.copy(), rho.copy()
    obst = np.zeros((sc.nz, sc.ny, sc.nx), dtype=np.float32)
    obst[0] = 1.0
    obst[-1] = 1.0
    Fx, Fy, Fz = np.zeros(N), np.zeros(N), np.zeros(N)
    vwf = -np.ones((4, sc.ny, sc.nx), dtype=np.int32)
    X, Y, RY, Z = (np.array(a[0], dtype=np.float64) for a in (sc.X, sc.Y, sc.RY, sc.Z))
    VX, VY, VZ, FX, FY, FZ = (np.zeros(E) for _ in range(6))
    bonds = M.dense_bond_lengths(sc.spring_ptr, sc.spring_nbr, sc.spring_L0, E)
    tri = np.ascontiguousarray(sc.tri, dtype=np.int32)
    r1 = np.ascontiguousarray(sc.rec_r1[0].reshape(T, R), dtype=np.float32)
    r2 = np.ascontiguousarray(sc.rec_r2[0].reshape(T, R), dtype=np.float32)
    ntri = np.ascontiguousarray(sc.node_ntri, dtype=np.int32)
    ring = np.ascontiguousarray(sc.ring, dtype=np.int32)
    Nref = np.ascontiguousarray(sc.meta["topology"].N if "topology" in sc.meta else np.zeros((NN, 3)))
    S0 = np.ascontiguousarray(sc.S0[0], dtype=np.float64)
    rb = np.empty((3, R, T), dtype=np.int32)
    rb[0] = -1
    rb[1] = -1
    rb[2] = 0
    uni = np.zeros((nsteps, 2, R, T))
    for t in range(nsteps):
        for tr in range(T):
            for r in range(R):
                u = ob.receptor_uniforms(sc.seed, t, tr * R + r)
                uni[t, 0, r, tr] = u[0]
                uni[t, 1, r, tr] = u[1]
    tb = np.zeros(nsteps, dtype=np.int32)
    traj = np.zeros((nsteps, 3, E))
    km = np.zeros(NN)
    sv = np.zeros((nsteps, 2))
    c = RefCase()
    c.lx, c.ly, c.lz, c.dx, c.dt = sc.nx, sc.ny, sc.nz, sc.dx, sc.dt
    c.params[:] = [float(v) for v in sc.params]
    c.fIN, c.fOUT, c.ux, c.uy, c.uz, c.rho = _p(fIN), _p(fOUT), _p(ux), _p(uy), _p(uz), _p(rho)
    c.obst = _p(obst, C.c_float)
    c.Fx, c.Fy, c.Fz, c.vWF = _p(Fx), _p(Fy), _p(Fz), _p(vwf, C.c_int)
    c.maxE, c.surf, c.newnode, c.R = E, T, NN, R
    c.X, c.Y, c.RY, c.Z = _p(X), _p(Y), _p(RY), _p(Z)
    c.VX, c.VY, c.VZ, c.FX, c.FY, c.FZ = _p(VX), _p(VY), _p(VZ), _p(FX), _p(FY), _p(FZ)
    c.bondLengths, c.triElem = _p(bonds), _p(tri, C.c_int)
    c.r1, c.r2 = _p(r1, C.c_float), _p(r2, C.c_float)
    c.node_nbrElemNum, c.node_nbr_nodes, c.Nref = _p(ntri, C.c_int), _p(ring, C.c_int), _p(Nref)
    c.S0, c.S0_all, c.V0 = _p(S0), float(sc.S0_all[0]), float(sc.V0[0])
    c.receptBond = _p(rb, C.c_int)
    c.nsteps, c.uniforms = nsteps, _p(uni)
    c.totalBond_per_step, c.traj, c.km_out, c.S_all_V_out = _p(tb, C.c_int), _p(traj), _p(km), _p(sv)
    c.fem_bend = 1 if int(sc.membrane_forces) & MEM_FEMBEND else 0
    if lib.refemu_run(C.byref(c)) != 0:
        raise RuntimeError("refemu_run failed")
    rec_state = np.stack([rb[0].T.reshape(-1), rb[1].T.reshape(-1), rb[2].T.reshape(-1)], 1)[None]
    lost = c.first_lost_site_step
    return dict(lost_site_step=np.asarray(lost), fIN=fIN, fOUT=fOUT, rho=rho, ux=ux, uy=uy, uz=uz, Fx=Fx, Fy=Fy, Fz=Fz, vwf=vwf,
                X=X, Y=Y, RY=RY, Z=Z, VX=VX, VY=VY, VZ=VZ, FX=FX, FY=FY, FZ=FZ, rec_state=rec_state,
                total_bond=tb, traj=traj, km=km, S_V=sv, f_init=f,
                u_init=np.stack([ux0, uy0, uz0]), rho_init=rho0)


CASES = {
    # platelet resting near the no-slip wall in the middle of the box
    "ref_wall": dict(seed=7, nx=16, ny=20, nz=10, level=1, R=2, nsteps=40),
    # platelet straddling the periodic y seam's stencils and the bounded low-x edge
    "ref_edges": dict(seed=11, nx=14, ny=16, nz=9, level=1, R=1, nsteps=30,
                      center=(0.45, 0.62, 0.35)),
    # the reference's own 958-vertex platelet mesh 0.02 um above the wall:
    # about 150 receptors bind in the first step, some of them to two vWF
    # sites (the two-bond branch of the bond kernel); no unbinding (Kr0 = 0),
    # so no receptor drops from two bonds to one (the stored-site path whose
    # out-of-bounds read the CUDA path fixes)
    "ref_mesh958": dict(seed=5, nx=16, ny=16, nz=8, level=1, R=1, nsteps=25, mesh="958", two_bonds=True,
                        gap=0.02, kr0=0.0),
    # the FEM bending chain the reference comments out (semLB.cu:518-520),
    # launched in its slot on top of the membrane chain it runs
    "ref_fembend": dict(seed=13, nx=16, ny=20, nz=10, level=1, R=2, nsteps=20, mem=MEM_ALL | MEM_FEMBEND),
    # the same chain on the reference's own 958-vertex mesh; four steps: the
    # chain makes this mesh's motion grow step by step (0.04 um in the first
    # step, 15 um by the eighth), after which rounding differences grow with it
    "ref_fembend958": dict(seed=17, nx=16, ny=16, nz=8, level=1, R=1, nsteps=4, mesh="958", gap=0.02,
                           kr0=0.0, mem=MEM_ALL | MEM_FEMBEND),
}


def reference_mesh958():
    """The reference's own 958-vertex / 1912-triangle platelet surface
    (Input/Platelet_Mesh_958.neu of its archive), read by libpfgpu's NEU
    reader from a temporary extraction."""
    import tarfile
    import tempfile
    from platelet_fiber_gpu_gb300 import build, gpu
    build.build()
    with tarfile.open(ob.reference_dir() / "gpu_20151203.tar.gz") as tf, tempfile.TemporaryDirectory() as d:
        path = Path(d) / "mesh.neu"
        path.write_bytes(tf.extractfile(tf.getmember("./Input/Platelet_Mesh_958.neu")).read())
        m = gpu.read_neu(path)
    return np.stack([m["X"], m["Y"], m["Z"]], 1), m["tri"]


def make(name: str, seed, nx, ny, nz, level, R, nsteps, center=None, mesh=None, two_bonds=False, gap=None,
         kf0=3.0e4, kr0=1.5e4, mem=MEM_ALL):
    msh = reference_mesh958() if mesh == "958" else None
    for attempt in range(50):
        s = seed + 1000 * attempt
        c = center
        if c is None and gap is not None:
            c = (nx * W.REF_DX / 2, ny * W.REF_DX / 2, 0.5 * (msh[0][:, 2].max() - msh[0][:, 2].min()) + gap)
        sc = W.reference_case(seed=s, nx=nx, ny=ny, nz=nz, level=level, R=R, center=c, mesh=msh, kf0=kf0, kr0=kr0)
        sc.membrane_forces = mem
        out = run_reference(sc, nsteps)
        # a receptor that drops from 2 bonds to 1 leaves the reference's stored
        # site at -1 (sem_kernel.cu:1937-1942); pick a seed whose run never does
        if int(out["lost_site_step"]) >= 0:
            continue
        if out["total_bond"].max() == 0:
            continue
        # the two-bond branch of sem_kernel.cu:1999-2030 must be taken
        if two_bonds and not (out["rec_state"][..., 2] > 1).any():
            continue
        break
    else:
        raise RuntimeError(f"{name}: no admissible seed")
    sc.f_init = out["f_init"]
    sc.u_init, sc.rho_init = out["u_init"], out["rho_init"]
    st0 = np.empty((1, sc.n_rec, 3), dtype=np.int32)
    st0[..., 0] = -1
    st0[..., 1] = -1
    st0[..., 2] = 0
    sc.rec_state = st0
    d = scene_to_dict(sc)
    d.update({"out." + k: v for k, v in out.items() if k not in ("f_init", "u_init", "rho_init")})
    d["nsteps"] = np.asarray(nsteps)
    path = ROOT / "tests" / "golden" / f"{name}.npz"
    np.savez_compressed(path, **d)
    print(f"{name}: seed {s}, bonds per step {out['total_bond'].tolist()}, wrote {path.name} "
          f"({path.stat().st_size // 1024} KB)")


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for n in names:
        make(n, **CASES[n])
