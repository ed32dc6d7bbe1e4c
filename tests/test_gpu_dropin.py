"""The reference-named C entry points (fluid_* / sem_* / fiber_*GPUKernel)
driven the way the reference driver drives them (gpuSEM_LB.c:1285-1304,
1433-1454): host arrays in the reference's layouts, per step
sem_invokeGPUKernel_Force then fluid_invokeGPUKernel, then the copy calls.
The result must match the golden vectors of the reference kernels as
closely as the job API does (FP64)."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden"
vp = C.c_void_p


class UniformSource(C.Structure):
    _fields_ = [("seed", C.c_uint64)]


@pytest.fixture(scope="module")
def lib():
    from platelet_fiber_gpu_gb300 import build, gpu
    build.build()
    L = gpu.lib()
    L.fluid_allocGPUKernel.restype = vp
    L.fluid_allocGPUKernel.argtypes = [vp, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int]
    L.fluid_initGPUKernel.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_float), C.POINTER(vp), C.POINTER(vp)] + [vp] * 9
    L.fluid_invokeGPUKernel.argtypes = [vp, vp, vp, vp, vp, C.c_int]
    L.fluid_releaseGPUKernel.argtypes = [vp, vp]
    L.sem_allocGPUKernel.restype = vp
    L.sem_allocGPUKernel.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_double,
                                     C.POINTER(C.c_float)]
    L.sem_initGPUKernel.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_int] + [vp] * 23 + [C.c_double, vp, vp]
    L.sem_invokeGPUKernel_Force.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), vp, C.c_double]
    L.sem_copyGPUKernel.argtypes = [vp, vp] + [vp] * 10 + [C.c_int]
    L.sem_releaseGPUKernel.argtypes = [vp, vp]
    return L


def _ptr(a):
    return a.ctypes.data_as(vp)


def test_reference_api_reproduces_golden(lib):
    from platelet_fiber_gpu_gb300 import mesh as M
    from platelet_fiber_gpu_gb300.scene import scene_from_dict
    d = np.load(GOLDEN / "ref_wall.npz")
    sc = scene_from_dict(d)
    n = int(d["nsteps"])
    N, E, T, NN = sc.n_nodes, sc.n_elem, sc.n_tri, sc.n_node
    R = sc.n_rec // T
    params = np.ascontiguousarray(sc.params, dtype=np.float32)
    pf = params.ctypes.data_as(C.POINTER(C.c_float))
    # fluid handle: fIN/fOUT as 19 separate [lz][ly][lx] buffers
    f = np.ascontiguousarray(np.asarray(sc.f_init, dtype=np.float64).reshape(19, N))
    fin = [np.ascontiguousarray(f[k]) for k in range(19)]
    fout = [np.zeros(N) for _ in range(19)]
    fin_p = (vp * 19)(*[_ptr(a) for a in fin])
    fout_p = (vp * 19)(*[_ptr(a) for a in fout])
    u = np.asarray(sc.u_init, dtype=np.float64).reshape(3, N)
    ux, uy, uz = (np.ascontiguousarray(u[k]) for k in range(3))
    rho = np.ascontiguousarray(np.asarray(sc.rho_init, dtype=np.float64).reshape(N))
    obst = np.zeros(N, dtype=np.float32)
    Fx, Fy, Fz = np.zeros(N), np.zeros(N), np.zeros(N)
    vwf = -np.ones((4, sc.ny, sc.nx), dtype=np.int32)
    g = lib.fluid_allocGPUKernel(None, sc.dt, sc.dx, sc.nx, sc.ny, sc.nz)
    assert g
    lib.fluid_initGPUKernel(None, g, 1, pf, fin_p, fout_p, _ptr(ux), _ptr(uy), _ptr(uz), _ptr(rho), _ptr(obst),
                            _ptr(Fx), _ptr(Fy), _ptr(Fz), _ptr(vwf))
    # SEM handle: element arrays [maxElements][maxCells] with one cell
    s = lib.sem_allocGPUKernel(None, 1, E, T, NN, R, sc.dt, float(sc.S0_all[0]), pf)
    assert s
    X, Y, Z = (np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(E)) for a in (sc.X, sc.Y, sc.Z))
    zeros = [np.zeros(E) for _ in range(6)]
    etype = np.zeros(E, dtype=np.int32)
    bonds = M.dense_bond_lengths(sc.spring_ptr, sc.spring_nbr, sc.spring_L0, E)
    tri = np.ascontiguousarray(sc.tri, dtype=np.int32)
    r1 = np.ascontiguousarray(np.asarray(sc.rec_r1, dtype=np.float32).reshape(T, R))
    r2 = np.ascontiguousarray(np.asarray(sc.rec_r2, dtype=np.float32).reshape(T, R))
    share = -np.ones((NN, 10), dtype=np.int32)
    Nn = np.zeros((NN, 3))
    ntri = np.ascontiguousarray(sc.node_ntri, dtype=np.int32)
    ring = np.zeros((E, 10), dtype=np.int32)
    ring[:sc.n_membrane] = sc.ring
    S0 = np.ascontiguousarray(np.asarray(sc.S0, dtype=np.float64).reshape(-1)[:T])
    st = np.asarray(sc.rec_state, dtype=np.int32).reshape(T, R, 3)
    rb = np.ascontiguousarray(np.transpose(st, (2, 1, 0)))  # [3][R][T]
    rnd = np.zeros((2, R, T))
    ncell = np.array([E], dtype=np.int32)
    lib.sem_initGPUKernel(None, s, 1, _ptr(ncell), T, R, _ptr(X), _ptr(Y), _ptr(Z), _ptr(X), _ptr(Y), _ptr(Y),
                          _ptr(Z), *[_ptr(a) for a in zeros], _ptr(etype), _ptr(bonds), _ptr(tri), _ptr(r1),
                          _ptr(r2), _ptr(share), _ptr(Nn), _ptr(ntri), _ptr(ring), _ptr(S0), float(sc.V0[0]),
                          _ptr(rb), _ptr(rnd))
    src = UniformSource(sc.seed)
    done, totalT = C.c_int(0), C.c_int(0)
    for _ in range(n):
        lib.sem_invokeGPUKernel_Force(None, s, 1, C.byref(done), C.byref(totalT), C.byref(src), 0.0)
        lib.fluid_invokeGPUKernel(None, g, s, _ptr(rnd), C.byref(src), 1)
    assert totalT.value == n and done.value == 0
    lib.fluid_initGPUKernel(None, g, 0, pf, fin_p, fout_p, _ptr(ux), _ptr(uy), _ptr(uz), _ptr(rho), _ptr(obst),
                            _ptr(Fx), _ptr(Fy), _ptr(Fz), _ptr(vwf))
    out = [np.zeros(E) for _ in range(10)]
    lib.sem_copyGPUKernel(None, s, *[_ptr(a) for a in out], n)
    fIN = np.stack(fin).reshape(d["out.fIN"].shape)
    rel = np.abs(fIN - d["out.fIN"]).max() / np.abs(d["out.fIN"]).max()
    assert rel < 1e-13
    u_ref = np.stack([d["out.ux"], d["out.uy"], d["out.uz"]]).reshape(3, -1)
    u_got = np.stack([ux, uy, uz])
    assert np.linalg.norm(u_got - u_ref) / np.linalg.norm(u_ref) < 1e-10
    for got, key in zip(out[:4], ("X", "Y", "RY", "Z")):
        assert np.abs(got - d[f"out.{key}"].reshape(-1)).max() < 1e-13
    np.testing.assert_array_equal(vwf, d["out.vwf"])
    lib.sem_releaseGPUKernel(None, s)
    lib.fluid_releaseGPUKernel(None, g)
