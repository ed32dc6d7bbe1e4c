"""Host restatements pinned to the reference's own code, compiled here from
the reference tree (oracle/refemu: refhost_driver.c runs gpuSEM_LB.c's host
code with stub GPU entry points; refhost_fiber.cpp exposes fiber.cpp's
worm-like-chain law), on the reference's own inputs (Input/parameter.dat and
Input/Platelet_Mesh_958.neu from its archive, extracted at test time):

- ParReader and NEUReader against pfgpu_read_parameter_file / pfgpu_read_neu;
- the topology the driver builds and hands to sem_initGPUKernel (virtual edge
  nodes of triElem, node -> triangle lists, vertex rings, normals, rest areas
  and volume) against pfgpu_build_topology;
- the element dumps the driver's step loop writes (seven files, byte for
  byte) against pfgpu_output_* fed the same arrays;
- writeVTK against pfgpu_write_vti (byte for byte);
- the worm-like-chain law against the oracle's.
Skipped where the reference tree is absent (it never is in the development
container, where these CPU tests run)."""
import ctypes as C
import shutil
import tarfile

import numpy as np
import pytest

from oracle import binding as ob

REF = ob.reference_dir()
ARCHIVE = REF / "gpu_20151203.tar.gz"
pytestmark = pytest.mark.skipif(not (REF / "gpuSEM_LB.c").exists() or not ARCHIVE.exists(),
                                reason="reference tree not present")
INPUTS = ("parameter.dat", "Platelet_Mesh_958.neu", "1ellip.pdb", "1ellip.psf")
STEPS, OUT_FREQ, SEED = 7, 3, 1101


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    d = tmp_path_factory.mktemp("refinput")
    with tarfile.open(ARCHIVE) as tf:
        for name in INPUTS:
            m = tf.getmember(f"./Input/{name}")
            (d / name).write_bytes(tf.extractfile(m).read())
    return d


@pytest.fixture(scope="module")
def driver(inputs, tmp_path_factory):
    """The driver run: Input/ as archived except OUT_FREQ (3), STEPS steps."""
    ob.build_refemu()
    L = C.CDLL(str(ob.HERE / "_ref" / "librefhost_driver.so"))
    L.refhost_run.argtypes = [C.c_char_p, C.c_int, C.c_int]
    L.refhost_pattern.restype = C.c_double
    L.refhost_pattern.argtypes = [C.c_int] * 4
    for f in ("refhost_tri", "refhost_node_share", "refhost_ring_count", "refhost_ring"):
        getattr(L, f).restype = C.POINTER(C.c_int)
    for f in ("refhost_normals", "refhost_S0", "refhost_bond_lengths"):
        getattr(L, f).restype = C.POINTER(C.c_double)
    L.refhost_elem.restype = C.POINTER(C.c_double)
    L.refhost_elem.argtypes = [C.c_int]
    L.refhost_S0_all.restype = C.c_double
    L.refhost_V0.restype = C.c_double
    L.ParReader.argtypes = [C.c_char_p] + [C.c_void_p] * 11
    L.NEUReader.argtypes = [C.c_char_p] + [C.c_void_p] * 5
    L.refhost_write_vtk.argtypes = [C.c_int] * 4 + [C.c_void_p] * 4 + [C.c_char_p, C.c_char_p]
    work = tmp_path_factory.mktemp("refrun")
    (work / "Input").mkdir()
    (work / "Output").mkdir()
    for name in INPUTS:
        shutil.copy(inputs / name, work / "Input" / name)
    par = (work / "Input" / "parameter.dat").read_text().splitlines()
    par = [f"OUT_FREQ      {OUT_FREQ}" if ln.startswith("OUT_FREQ") else ln for ln in par]
    (work / "Input" / "parameter.dat").write_text("\n".join(par) + "\n")
    assert L.refhost_run(str(work).encode(), SEED, STEPS) == STEPS
    dims = (C.c_int * 6)()
    L.refhost_dims(dims)
    return L, work, list(dims)


def _arr(ptr, n, dtype):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype).copy()


def test_parameter_reader(gpu, driver, inputs):
    L = driver[0]
    f = (inputs / "parameter.dat")
    dt, st, dx = C.c_float(), C.c_float(), C.c_float()
    of, mc, me, se = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    pdb, psf, neu = (C.create_string_buffer(256) for _ in range(3))
    hp = (C.c_float * 100)()
    L.ParReader(str(f).encode(), C.byref(dt), C.byref(st), C.byref(of), C.byref(mc), C.byref(me), C.byref(se), pdb,
                psf, neu, C.byref(dx), hp)
    p = gpu.read_parameter_file(f)
    assert (p["dt"], p["sim_time"], p["dx"]) == (dt.value, st.value, dx.value)
    assert (p["out_freq"], p["max_cell"], p["max_elem"], p["surf_elem"]) == (of.value, mc.value, me.value, se.value)
    assert (p["pdb_path"], p["psf_path"], p["neu_path"]) == (pdb.value.decode(), psf.value.decode(), neu.value.decode())
    for k in (0, 1, 2, 4, 5, 6):
        assert np.float32(p["host_param"][k]) == np.float32(hp[k]), k


def test_neu_reader(gpu, driver, inputs):
    L = driver[0]
    f = inputs / "Platelet_Mesh_958.neu"
    m = gpu.read_neu(f)
    n, t = len(m["X"]), len(m["tri"])
    X, Y, Z = np.zeros(n), np.zeros(n), np.zeros(n)
    bonds = np.zeros(n * n)
    tri = np.zeros((t, 6), dtype=np.int32)
    L.NEUReader(str(f).encode(), X.ctypes.data, Y.ctypes.data, Z.ctypes.data, bonds.ctypes.data, tri.ctypes.data)
    np.testing.assert_array_equal(m["X"], X)
    np.testing.assert_array_equal(m["Y"], Y)
    np.testing.assert_array_equal(m["Z"], Z)
    np.testing.assert_array_equal(m["tri"], tri[:, :3])
    dense = np.zeros((n, n))
    for i in range(n):
        for q in range(m["bond_ptr"][i], m["bond_ptr"][i + 1]):
            dense[i, m["bond_nbr"][q]] = m["bond_len"][q]
    np.testing.assert_array_equal(dense, bonds.reshape(n, n).T)


def test_topology_matches_the_driver(gpu, driver, inputs):
    L, _, (C_, E, T, NN, R, P) = driver
    X = _arr(L.refhost_elem(0), E * C_, np.float64).reshape(E, C_)[:, 0]
    Y = _arr(L.refhost_elem(1), E * C_, np.float64).reshape(E, C_)[:, 0]
    Z = _arr(L.refhost_elem(3), E * C_, np.float64).reshape(E, C_)[:, 0]
    tri_ref = _arr(L.refhost_tri(), T * 6, np.int32).reshape(T, 6)
    nv = int(tri_ref[:, :3].max()) + 1
    topo = gpu.build_topology(tri_ref[:, :3], X[:nv], Y[:nv], Z[:nv])
    assert topo["n_nodes"] == NN
    np.testing.assert_array_equal(topo["tri6"], tri_ref)
    share = _arr(L.refhost_node_share(), NN * 10, np.int32).reshape(NN, 10)
    ptr = topo["node_ptr"]
    for q in range(NN):
        ours = sorted(topo["node_tri"][ptr[q]:ptr[q + 1]].tolist())
        theirs = sorted(v for v in share[q].tolist() if v >= 0)
        assert ours == theirs, q
    cnt = _arr(L.refhost_ring_count(), E, np.int32)
    ring = _arr(L.refhost_ring(), E * 10, np.int32).reshape(E, 10)
    for v in range(nv):
        k = ptr[v + 1] - ptr[v]
        assert cnt[v] == k
        np.testing.assert_array_equal(topo["ring"][ptr[v]:ptr[v + 1]], ring[v, :k])
    normals = _arr(L.refhost_normals(), NN * 3, np.float64).reshape(NN, 3)
    assert np.abs(topo["normals"] - normals).max() < 1e-12
    S0 = _arr(L.refhost_S0(), T, np.float64)
    assert np.abs(topo["S0"] - S0).max() <= 1e-14 * np.abs(S0).max()
    assert topo["S0_all"] == pytest.approx(L.refhost_S0_all(), rel=1e-13)
    assert topo["V0"] == pytest.approx(L.refhost_V0(), rel=1e-13)


def test_element_dumps_match_the_driver(gpu, driver, tmp_path):
    L, work, (C_, E, T, NN, R, P) = driver
    from platelet_fiber_gpu_gb300 import gpu as G
    lib = G.lib()
    dp = C.POINTER(C.c_double)
    lib.pfgpu_output_open_arrays.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double] + [dp] * 5 + \
        [C.POINTER(C.c_void_p)]
    lib.pfgpu_output_frame_arrays.argtypes = [C.c_void_p, C.c_longlong] + [dp] * 5
    lib.pfgpu_output_close.argtypes = [C.c_void_p, C.c_int]
    PE = P * E

    def pe(a):  # [E][maxCells] (cell fastest) -> [P][E]
        return np.ascontiguousarray(a.reshape(E, C_)[:, :P].T.reshape(PE))

    init = [pe(_arr(L.refhost_elem(k), E * C_, np.float64)) for k in range(10)]

    def frame(t):
        return [np.array([[L.refhost_pattern(i, j, t, k) for i in range(E)] for j in range(P)]).reshape(PE)
                for k in range(10)]

    def args(a):
        V = np.concatenate(a[4:7])
        F = np.concatenate(a[7:10])
        return [x.ctypes.data_as(dp) for x in (a[0], a[2], a[3], V, F)], (V, F)

    dt = float(np.float32(gpu.read_parameter_file(work / "Input" / "parameter.dat")["dt"]))
    h = C.c_void_p()
    a0, keep0 = args(init)
    assert lib.pfgpu_output_open_arrays(str(tmp_path).encode(), 0, P, E, dt, *a0, C.byref(h)) == 0
    steps = list(range(OUT_FREQ, STEPS + 1, OUT_FREQ))
    if steps[-1] != STEPS:
        steps.append(STEPS)
    for t in steps:
        fa = frame(t)
        a, keep = args(fa)
        assert lib.pfgpu_output_frame_arrays(h, t, *a) == 0
    assert lib.pfgpu_output_close(h, SEED) == 0
    names = ["cellsPos.data", "cellsVel.data", "cellsForce.data", "cellsPosASCII.dat", "cellsVelASCII.dat",
             "cellsForceASCII.dat", "cellsPauseTime.dat"]
    for name in names:
        ours, theirs = (tmp_path / name).read_bytes(), (work / "Output" / name).read_bytes()
        assert ours == theirs, name


def test_write_vtk_matches_the_driver(gpu, driver, tmp_path):
    L = driver[0]
    rng = np.random.default_rng(4)
    nx, ny, nz = 7, 5, 4
    rho, ux, uy, uz = (np.ascontiguousarray(rng.standard_normal((nz, ny, nx)).astype(np.float32)) for _ in range(4))
    (tmp_path / "ref").mkdir()
    L.refhost_write_vtk(12, nx, ny, nz, rho.ctypes.data, ux.ctypes.data, uy.ctypes.data, uz.ctypes.data,
                        str(tmp_path / "ref").encode(), b"LBMflow")
    gpu.write_vti(12, rho, np.stack([ux, uy, uz]), tmp_path / "ours", "LBMflow")
    name = "LBMflow_0000012.vti"
    assert (tmp_path / "ours" / name).read_bytes() == (tmp_path / "ref" / name).read_bytes()


def test_worm_like_chain_law():
    ob.build_refemu()
    F = C.CDLL(str(ob.HERE / "_ref" / "librefhost_fiber.so"))
    F.refhost_wlc.restype = C.c_double
    F.refhost_wlc.argtypes = [C.c_double] * 4
    rng = np.random.default_rng(9)
    for _ in range(200):
        l0 = float(rng.uniform(0.05, 2.0))
        l = l0 * float(rng.uniform(0.5, 1.8))
        mass = float(rng.uniform(0.1, 3.0))
        assert ob.wlc_force(l0, l, mass) == F.refhost_wlc(l0, l, float(rng.uniform(0, 5)), mass)
