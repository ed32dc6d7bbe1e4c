"""The reference-named C entry points (fluid_* / sem_* / fiber_*GPUKernel)
driven the way the reference driver drives them (gpuSEM_LB.c:1285-1304,
1433-1454): host arrays in the reference's layouts, per step
sem_invokeGPUKernel_Force then fluid_invokeGPUKernel, then the copy calls.

- FP64 (the default): the golden vectors of the reference kernels to 1e-13,
  as closely as the job API.
- node_share_Elem and N are accepted and not read (the reference uploads
  them, semLB.cu:939-943, but its kernels use neither outside commented-out
  code, sem_kernel.cu:743,856,1513): poisoned arrays give the same result.
- FP32 handles (pfgpu_set_default_precision): the golden vectors within the
  FP32 tolerances of the job API's own golden test.
- A fibrin handle in the reference's tmp_fiber_GPUgrids layouts
  (GPUDefines.h:170-200: NodeType, N_Conn_at_Node, Link_at_Node padded with
  -100, lAdjVer, linkLengths0), attached to the fluid handle: fibrin and
  element positions equal the job API's and the oracle's for the same scene.
"""
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
    L.fiber_allocGPUKernel.restype = vp
    L.fiber_allocGPUKernel.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, vp]
    L.fiber_init_GPUKernel.argtypes = [vp, vp] + [vp] * 19
    L.fiber_copy_GPUKernel.argtypes = [vp, vp] + [vp] * 12
    L.fiber_release_GPUKernel.argtypes = [vp, vp]
    L.pfgpu_fluid_attach_fiber.argtypes = [vp, vp, C.c_int, C.c_double, C.c_double]
    L.pfgpu_set_default_precision.argtypes = [C.c_int, C.c_double]
    return L


def _ptr(a):
    return a.ctypes.data_as(vp)


def _fiber_arrays(sc):
    """The scene's fibrin mesh in tmp_fiber_GPUgrids host layouts; each
    node's links in the order of the scene's own neighbour lists."""
    links = np.asarray(sc.meta["fib_links"], dtype=np.int32)
    M, L = sc.n_fib, len(links)
    per = [[] for _ in range(M)]
    for l, (a, b) in enumerate(links):
        per[a].append(l)
        per[b].append(l)
    K = max(len(p) for p in per)
    lan = np.full((M, K), -100, dtype=np.int32)
    for m, p in enumerate(per):
        lan[m, :len(p)] = p
    nconn = np.array([len(p) for p in per], dtype=np.int32)
    l0 = np.zeros(L)
    ptr, nbr, csr_l0 = sc.fib_ptr, sc.fib_nbr, sc.fib_L0
    for m in range(M):
        for q, l in zip(range(ptr[m], ptr[m + 1]), per[m]):
            a, b = links[l]
            assert nbr[q] == (b if a == m else a)
            l0[l] = csr_l0[q]
    return dict(M=M, L=L, K=K, type=np.ascontiguousarray(sc.fib_fixed, dtype=np.int32), nconn=nconn, lan=lan,
                adj=np.ascontiguousarray(links), l0=l0)


def drive(lib, sc, n, poison=False, fiber=False):
    """Runs `sc` for n steps through the reference entry points; returns
    the downloaded lattice, elements and (with fiber) fibrin state."""
    from platelet_fiber_gpu_gb300 import mesh as M
    N, E, T, NN = sc.n_nodes, sc.n_elem, sc.n_tri, sc.n_node
    R = sc.n_rec // T
    params = np.ascontiguousarray(sc.params, dtype=np.float32)
    pf = params.ctypes.data_as(C.POINTER(C.c_float))
    # fluid handle: fIN/fOUT as 19 separate [lz][ly][lx] buffers
    # the caller's own arrays (copies: the download writes into them)
    f = np.array(np.asarray(sc.f_init, dtype=np.float64).reshape(19, N))
    fin = [np.array(f[k]) for k in range(19)]
    fout = [np.zeros(N) for _ in range(19)]
    fin_p = (vp * 19)(*[_ptr(a) for a in fin])
    fout_p = (vp * 19)(*[_ptr(a) for a in fout])
    u = np.asarray(sc.u_init, dtype=np.float64).reshape(3, N)
    ux, uy, uz = (np.array(u[k]) for k in range(3))
    rho = np.array(np.asarray(sc.rho_init, dtype=np.float64).reshape(N))
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
    if poison:
        share = np.full((NN, 10), 123456789, dtype=np.int32)
        Nn = np.full((NN, 3), np.nan)
    else:
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
    fg = None
    if fiber:
        fa = _fiber_arrays(sc)
        Mf = fa["M"]
        fx, fy, fz = (np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in (sc.fib_X, sc.fib_Y, sc.fib_Z))
        z3 = [np.zeros(Mf) for _ in range(9)]
        fg = lib.fiber_allocGPUKernel(None, Mf, fa["L"], fa["K"], float(sc.dt), None)
        assert fg
        lib.fiber_init_GPUKernel(None, fg, _ptr(fa["type"]), _ptr(fa["nconn"]), _ptr(fa["lan"]), _ptr(fa["adj"]),
                                 _ptr(fa["l0"]), _ptr(fa["l0"]), _ptr(fa["l0"]), _ptr(fx), _ptr(z3[0]), _ptr(fx),
                                 _ptr(z3[1]), _ptr(fy), _ptr(fy), _ptr(z3[2]), _ptr(z3[3]), _ptr(fz), _ptr(fz),
                                 _ptr(z3[4]), _ptr(z3[5]))
        assert lib.pfgpu_fluid_attach_fiber(g, fg, int(sc.fib_law), float(sc.fib_k), float(sc.fib_mass)) == 0
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
    res = dict(fIN=np.stack(fin), u=np.stack([ux, uy, uz]), rho=rho, X=out[0], Y=out[1], RY=out[2], Z=out[3],
               vwf=vwf)
    if fiber:
        fo = [np.zeros(Mf) for _ in range(12)]
        lib.fiber_copy_GPUKernel(None, fg, *[_ptr(a) for a in fo])
        res["fib"] = dict(X=fo[0], VX=fo[1], FX=fo[3], Y=fo[4], Z=fo[8], FY=fo[7], FZ=fo[11])
        lib.fiber_release_GPUKernel(None, fg)
    lib.sem_releaseGPUKernel(None, s)
    lib.fluid_releaseGPUKernel(None, g)
    return res


def _golden():
    from platelet_fiber_gpu_gb300.scene import scene_from_dict
    d = np.load(GOLDEN / "ref_wall.npz")
    return scene_from_dict(d), int(d["nsteps"]), d


@pytest.mark.parametrize("poison", [False, True], ids=["plain", "poisoned_share_and_N"])
def test_reference_api_reproduces_golden(lib, poison):
    sc, n, d = _golden()
    r = drive(lib, sc, n, poison=poison)
    fIN = r["fIN"].reshape(d["out.fIN"].shape)
    assert np.abs(fIN - d["out.fIN"]).max() / np.abs(d["out.fIN"]).max() < 1e-13
    u_ref = np.stack([d["out.ux"], d["out.uy"], d["out.uz"]]).reshape(3, -1)
    assert np.linalg.norm(r["u"] - u_ref) / np.linalg.norm(u_ref) < 1e-10
    for key in ("X", "Y", "RY", "Z"):
        assert np.abs(r[key] - d[f"out.{key}"].reshape(-1)).max() < 1e-13
    np.testing.assert_array_equal(r["vwf"], d["out.vwf"])


def test_reference_api_fp32_handles(lib):
    """pfgpu_set_default_precision(PF_PREC_FP32): later fluid handles run the
    FP32 store; the golden vectors within the FP32 tolerances (velocity
    relative L2 1e-4 after the fixture's steps, positions 1e-7), vWF slots
    bit for bit."""
    sc, n, d = _golden()
    assert lib.pfgpu_set_default_precision(1, 0.0) == 0
    try:
        r = drive(lib, sc, n)
    finally:
        lib.pfgpu_set_default_precision(0, 0.0)
    u_ref = np.stack([d["out.ux"], d["out.uy"], d["out.uz"]]).reshape(3, -1)
    assert np.linalg.norm(r["u"] - u_ref) / np.linalg.norm(u_ref) < 1e-4
    pos = np.stack([r["X"], r["Y"], r["Z"]])
    pos_ref = np.stack([d["out.X"], d["out.Y"], d["out.Z"]]).reshape(3, -1)
    assert np.linalg.norm(pos - pos_ref) / np.linalg.norm(pos_ref) < 1e-7
    np.testing.assert_array_equal(r["vwf"], d["out.vwf"])


def test_reference_api_with_fibrin_handle(lib):
    """The golden channel with a 60-node / 120-link Hookean fibrin mesh on
    the bottom wall, driven through fiber_allocGPUKernel ->
    fiber_init_GPUKernel -> pfgpu_fluid_attach_fiber -> per-step invokes ->
    fiber_copy_GPUKernel: the same state as the job API and the oracle."""
    from oracle import binding as ob
    from platelet_fiber_gpu_gb300 import gpu
    from platelet_fiber_gpu_gb300 import workloads as W
    sc, _, _ = _golden()
    W._fibrin(sc, 60, 120, 3 * sc.dx, np.random.default_rng(11), 0.5)
    n = 12
    r = drive(lib, sc, n, fiber=True)
    j = gpu.Job(sc, 0)
    j.step(n)
    Fj, Ej, Lj = j.fibrin(), j.elements(), j.lattice()
    j.close()
    o = ob.Oracle(sc)
    o.step(n)
    Fo, Eo = o.fibrin(), o.elements()
    o.close()
    assert sc.fib_fixed.any() and not sc.fib_fixed.all()
    for ref in (Fj, Fo):
        for k in ("X", "Y", "Z"):
            assert np.abs(r["fib"][k] - ref[k]).max() < 1e-12
    assert np.abs(r["fib"]["X"] - sc.fib_X).max() > 0  # the free nodes moved
    for k in ("X", "Y", "Z"):
        assert np.abs(r[k] - Ej[k]).max() < 1e-12
        assert np.abs(r[k] - Eo[k]).max() < 1e-12
    assert np.abs(r["fIN"] - Lj["fIN"]).max() / np.abs(Lj["fIN"]).max() < 1e-12
    fF = np.stack([r["fib"]["FX"], r["fib"]["FY"], r["fib"]["FZ"]])
    assert np.linalg.norm(fF - Fj["F"]) <= 1e-9 * np.linalg.norm(Fj["F"])
