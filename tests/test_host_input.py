"""Host input without a GPU: the parameter-file reader (ParReader,
gpuSEM_LB.c:148-343), the NEU mesh reader (NEUReader, :345-404) and the
topology build (:846-1055) of libpfgpu agree with the Python restatement the
scenes are built with (platelet_fiber_gpu_gb300.mesh) and with files written
here; out-of-order keywords and bad records are refused with a reason."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


KEYS = [("PDB_PATH", "Input/cells.pdb"), ("PSF_PATH", "Input/cells.psf"), ("NEU_PATH", "Input/platelet.neu"),
        ("DELTA_X", "0.2"), ("DELTA_T", "1e-7"), ("SIM_TIME", "200"), ("OUT_FREQ", "500"), ("MAX_CELL", "2"),
        ("MAX_ELEM", "600"), ("SURF_ELEM", "796"), ("RECEPTOR", "200"), ("RANDOM_SEED", "1101"),
        ("K_SPRING", "0.05"), ("Kr0", "3.21"), ("SHEAR_RATE", "1000"), ("INIT_RHO", "1.0239")]


def test_parameter_file(gpu, tmp_path):
    f = tmp_path / "parameter.dat"
    f.write_text("".join(f"{k}   {v}\n" for k, v in KEYS))
    p = gpu.read_parameter_file(f)
    assert p["pdb_path"] == "Input/cells.pdb" and p["neu_path"] == "Input/platelet.neu"
    assert p["dx"] == np.float32(0.2) and p["dt"] == np.float32(1e-7) and p["sim_time"] == 200.0
    assert (p["out_freq"], p["max_cell"], p["max_elem"], p["surf_elem"]) == (500, 2, 600, 796)
    hp = np.float32([200, 1101, 0.05, 0, 3.21, 1000, 1.0239])
    np.testing.assert_array_equal(np.float32(p["host_param"]), hp)
    swapped = KEYS[:]
    swapped[3], swapped[4] = swapped[4], swapped[3]
    f.write_text("".join(f"{k} {v}\n" for k, v in swapped))
    with pytest.raises(gpu.PfgpuError, match="DELTA_X"):
        gpu.read_parameter_file(f)
    with pytest.raises(gpu.PfgpuError, match="cannot open"):
        gpu.read_parameter_file(tmp_path / "missing.dat")


def write_neu(path, v, t, rng):
    """NEU text: counts, node records (1-based, shuffled), triangle records."""
    order = rng.permutation(len(v))
    lines = [f"{len(v)} {len(t)}"]
    lines += [f"{i + 1} {float(v[i, 0])!r} {float(v[i, 1])!r} {float(v[i, 2])!r}" for i in order]
    lines += [f"{k + 1} 3 3 {a + 1} {b + 1} {c + 1}" for k, (a, b, c) in enumerate(t)]
    path.write_text("\n".join(lines) + "\n")


@pytest.mark.parametrize("level", [0, 1, 2])
def test_neu_reader_and_topology(gpu, tmp_path, level):
    from platelet_fiber_gpu_gb300 import mesh as M
    v, t = M.ellipsoid_icosphere(level, (1.0, 1.0, 0.5))
    f = tmp_path / "platelet.neu"
    write_neu(f, v, t, np.random.default_rng(level))
    m = gpu.read_neu(f)
    np.testing.assert_array_equal(np.stack([m["X"], m["Y"], m["Z"]], 1), v)
    np.testing.assert_array_equal(m["tri"], t[:, :3])
    ptr, nbr, ln = M.edge_rest_lengths(v, t, len(v))
    np.testing.assert_array_equal(m["bond_ptr"], ptr)
    np.testing.assert_array_equal(m["bond_nbr"], nbr)
    np.testing.assert_array_equal(m["bond_len"], ln)

    topo = gpu.build_topology(m["tri"], m["X"], m["Y"], m["Z"])
    ref = M.build_topology(t, len(v), v)
    assert topo["n_nodes"] == ref.newnode
    np.testing.assert_array_equal(topo["tri6"], ref.tri6)
    np.testing.assert_array_equal(np.diff(topo["node_ptr"]), ref.node_ntri)
    for i in range(ref.newnode):
        a, b = topo["node_ptr"][i], topo["node_ptr"][i + 1]
        np.testing.assert_array_equal(topo["node_tri"][a:b], ref.node_share[i, :b - a])
        if i < len(v):
            np.testing.assert_array_equal(topo["ring"][a:b], ref.ring[i, :b - a])
    np.testing.assert_allclose(topo["normals"], ref.N, rtol=0, atol=1e-15)
    S0, S0_all, V0 = M.rest_area_volume(t, v)
    np.testing.assert_array_equal(topo["S0"], S0)
    assert topo["S0_all"] == S0_all and topo["V0"] == V0


def test_neu_reader_refuses_bad_records(gpu, tmp_path):
    f = tmp_path / "bad.neu"
    f.write_text("3 1\n1 0 0 0\n2 1 0 0\n4 0 1 0\n1 3 3 1 2 3\n")
    with pytest.raises(gpu.PfgpuError, match="node index out of range"):
        gpu.read_neu(f)
    f.write_text("3 1\n1 0 0 0\n2 1 0 0\n3 0 1 0\n1 3 3 1 2 9\n")
    with pytest.raises(gpu.PfgpuError, match="triangle node out of range"):
        gpu.read_neu(f)


def test_single_triangle_topology(gpu):
    """One triangle: the reference's special case numbers its edge nodes 3, 4, 5."""
    topo = gpu.build_topology(np.array([[0, 1, 2]]), np.array([0.0, 1, 0]), np.array([0.0, 0, 1]), np.zeros(3))
    np.testing.assert_array_equal(topo["tri6"], [[0, 1, 2, 3, 4, 5]])
    assert topo["n_nodes"] == 6
    np.testing.assert_array_equal(topo["ring"], [1, 2, 0])
    assert topo["S0_all"] == 0.5


def test_template_from_neu(gpu, tmp_path):
    """A platelet template built from a NEU file equals the one built from
    the same mesh in memory."""
    from platelet_fiber_gpu_gb300 import mesh as M
    from platelet_fiber_gpu_gb300.workloads import PlateletTemplate
    v, t = M.ellipsoid_icosphere(1, (0.6, 0.6, 0.3))
    f = tmp_path / "p.neu"
    write_neu(f, v, t, np.random.default_rng(0))
    a = PlateletTemplate.from_neu(f, 12, 3, (0.6, 0.6, 0.3))
    b = PlateletTemplate(v, t, 12, 3, (0.6, 0.6, 0.3))
    np.testing.assert_array_equal(a.local, b.local)
    np.testing.assert_array_equal(a.tris[:, :3], b.tris[:, :3])
    np.testing.assert_array_equal(a.sp_L0, b.sp_L0)
    assert a.mean_bond == b.mean_bond


def test_scene_from_reference_inputs(gpu, tmp_path):
    """A scene built from a parameter file and the NEU mesh it names carries
    the file's dx, dt, shear, density, spring constant, Kr0, receptor total
    and seed, MAX_CELL platelets of MAX_ELEM elements (mesh vertices first,
    then cytoplasm), and passes the library's scene checks."""
    from platelet_fiber_gpu_gb300 import mesh as M, workloads as W
    from platelet_fiber_gpu_gb300.scene import P_KR0, P_KSPRING, P_NUMRECEPTORS, P_RHO0, P_SEED, P_SHEAR
    v, t = M.ellipsoid_icosphere(2, (1.0, 1.0, 0.5))
    (tmp_path / "Input").mkdir()
    write_neu(tmp_path / "Input" / "platelet.neu", v, t, np.random.default_rng(1))
    keys = dict(KEYS)
    keys.update(MAX_CELL="3", MAX_ELEM=str(len(v) + 40), SURF_ELEM=str(len(t)), RECEPTOR="120")
    par = tmp_path / "Input" / "parameter.dat"
    par.write_text("".join(f"{k} {keys[k]}\n" for k, _ in KEYS))
    sc = W.from_reference_inputs(par, 64, 48, 32)
    assert (sc.n_platelets, sc.n_elem, sc.n_membrane) == (3, len(v) + 40, len(v))
    assert sc.dx == np.float32(0.2) or abs(sc.dx - 0.2) < 1e-7
    p = sc.params
    assert p[P_SHEAR] == 1000 and p[P_RHO0] == np.float32(1.0239) and p[P_KSPRING] == np.float32(0.05)
    assert p[P_KR0] == np.float32(3.21) and p[P_SEED] == 1101
    assert p[P_NUMRECEPTORS] == 120 and sc.n_rec == 40
    # membrane vertices of the first platelet are the mesh, shifted to its centre
    X = np.asarray(sc.X).reshape(3, -1)
    np.testing.assert_allclose(X[0, :len(v)] - X[0, :len(v)].mean(), v[:, 0] - v[:, 0].mean(), atol=1e-12)
    assert gpu.scene_device_bytes(sc, 1) > 0
    # the library's scene validation runs on the host before any CUDA call:
    # without a GPU a valid scene fails only there (PFGPU_ERR_CUDA)
    import ctypes as C
    L = gpu.lib()
    c = sc.to_c()
    h = C.c_void_p()
    rc = L.pfgpu_job_create(C.byref(c), 1, 0.0, C.byref(h))
    assert rc in (0, 2), L.pfgpu_last_error()
    if rc == 0:
        L.pfgpu_job_destroy(h)


def test_single_cell_gets_the_drivers_offset(gpu, tmp_path):
    """One cell: the mesh shifted by the reference driver's (8.0, 1.5, 0.32)
    um (gpuSEM_LB.c:811-820), RY equal to Y."""
    from platelet_fiber_gpu_gb300 import mesh as M, workloads as W
    v, t = M.ellipsoid_icosphere(1, (1.0, 1.0, 0.5))
    (tmp_path / "Input").mkdir()
    write_neu(tmp_path / "Input" / "platelet.neu", v, t, np.random.default_rng(2))
    keys = dict(KEYS)
    keys.update(MAX_CELL="1", MAX_ELEM=str(len(v)), RECEPTOR="30")
    par = tmp_path / "Input" / "parameter.dat"
    par.write_text("".join(f"{k} {keys[k]}\n" for k, _ in KEYS))
    sc = W.from_reference_inputs(par, 96, 48, 32)
    X, Y, Z = (np.asarray(a).reshape(-1) for a in (sc.X, sc.Y, sc.Z))
    np.testing.assert_allclose(X, v[:, 0] + 8.0, atol=1e-12)
    np.testing.assert_allclose(Y, v[:, 1] + 1.5, atol=1e-12)
    np.testing.assert_allclose(Z, v[:, 2] + 0.32, atol=1e-12)
    np.testing.assert_array_equal(np.asarray(sc.RY).reshape(-1), Y)
