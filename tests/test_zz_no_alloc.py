"""pfgpu_membrane_forces_noalloc (membrane pass on caller-owned device arrays,
scratch in a static device array) against the membrane forces the job path
computes for the same positions: the job's element force after one step is
the membrane force at the initial positions when Morse pairs, bonds and
fibrin are off.  Same kernel, same inputs: FP64, FP32 and FP16-shifted (whose
membrane pass is the FP32 one) agree bit for bit (tolerance 0); two calls in
a row must give the same result.  Inconsistent topology is rejected on the
device and reported by pfgpu_membrane_noalloc_status."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class MembraneArgs(C.Structure):
    _fields_ = [
        ("n_platelets", C.c_int), ("n_elem", C.c_int), ("n_membrane", C.c_int), ("n_tri", C.c_int),
        ("n_node", C.c_int), ("precision", C.c_int), ("membrane_forces", C.c_int),
        ("kspring", C.c_float), ("ks", C.c_float), ("kv", C.c_float), ("kbend", C.c_float), ("f0", C.c_float),
        ("X", C.c_void_p), ("Y", C.c_void_p), ("RY", C.c_void_p), ("Z", C.c_void_p),
        ("tri", C.c_void_p), ("node_ntri", C.c_void_p), ("ring", C.c_void_p),
        ("spring_ptr", C.c_void_p), ("spring_nbr", C.c_void_p), ("spring_L0", C.c_void_p),
        ("S0", C.c_void_p), ("S0_all", C.c_void_p), ("V0", C.c_void_p),
        ("F_out", C.c_void_p), ("S_V_out", C.c_void_p), ("km_out", C.c_void_p),
    ]


@pytest.fixture(scope="module")
def lib():
    from platelet_fiber_gpu_gb300 import build, gpu
    build.build()
    L = gpu.lib()
    L.pfgpu_membrane_forces_noalloc.argtypes = [C.POINTER(MembraneArgs), C.c_void_p]
    L.pfgpu_membrane_forces_noalloc.restype = C.c_int
    L.pfgpu_membrane_noalloc_scratch_bytes.restype = C.c_size_t
    L.pfgpu_membrane_noalloc_status.argtypes = [C.c_void_p]
    L.pfgpu_membrane_noalloc_status.restype = C.c_int
    return L


def _scene():
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(n_fib=0, n_links=0, n_rec=0)
    sc.morse = 0
    return sc


def _job_reference(sc, prec):
    from platelet_fiber_gpu_gb300 import gpu
    j = gpu.Job(sc, prec)
    j.step(1, graph=False)
    F = j.elements()["F"]
    M = j.membrane()
    j.close()
    return F, M


def _call(lib, sc, prec, torch, node_ntri=None, expect_rc=0, fill=0.0):
    from platelet_fiber_gpu_gb300.scene import P_KBEND, P_KS, P_KSPRING, P_KV, P_F0
    dev = torch.device("cuda", 0)
    keep = []

    def d(a, dt):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)
        keep.append(t)
        return C.c_void_p(t.data_ptr())

    PE = sc.n_platelets * sc.n_elem
    real = torch.float64 if prec == 0 else torch.float32
    F = torch.full((3 * PE,), fill, dtype=real, device=dev)
    SV = torch.zeros(2 * sc.n_platelets, dtype=torch.float64, device=dev)
    km = torch.zeros(sc.n_platelets * sc.n_membrane, dtype=real, device=dev)
    p = np.asarray(sc.params, dtype=np.float32)
    a = MembraneArgs(
        sc.n_platelets, sc.n_elem, sc.n_membrane, sc.n_tri, sc.n_node, prec, int(sc.membrane_forces),
        float(p[P_KSPRING]), float(p[P_KS]), float(p[P_KV]), float(p[P_KBEND]), float(p[P_F0]),
        d(sc.X, np.float64), d(sc.Y, np.float64), d(sc.RY, np.float64), d(sc.Z, np.float64),
        d(sc.tri, np.int32), d(sc.node_ntri if node_ntri is None else node_ntri, np.int32), d(sc.ring, np.int32),
        d(sc.spring_ptr, np.int32), d(sc.spring_nbr, np.int32), d(sc.spring_L0, np.float64),
        d(sc.S0, np.float64), d(sc.S0_all, np.float64), d(sc.V0, np.float64),
        C.c_void_p(F.data_ptr()), C.c_void_p(SV.data_ptr()), C.c_void_p(km.data_ptr()))
    rc = lib.pfgpu_membrane_forces_noalloc(C.byref(a), None)
    assert rc == 0, lib.pfgpu_last_error().decode()
    st = lib.pfgpu_membrane_noalloc_status(None)
    assert st == expect_rc, lib.pfgpu_last_error().decode()
    torch.cuda.synchronize()
    return (F.double().cpu().numpy().reshape(3, PE), SV.cpu().numpy().reshape(sc.n_platelets, 2),
            km.double().cpu().numpy().reshape(sc.n_platelets, sc.n_membrane))


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "fp32", "fp16"])
def test_noalloc_membrane_matches_job_path_twice(lib, prec):
    torch = pytest.importorskip("torch")
    sc = _scene()
    F_job, M_job = _job_reference(sc, prec)
    for _ in range(2):
        F, SV, km = _call(lib, sc, prec, torch)
        np.testing.assert_array_equal(F, F_job)
        np.testing.assert_array_equal(SV, M_job["S_V"])
        np.testing.assert_array_equal(km, M_job["km"])


def test_noalloc_rejects_oversize_scratch(lib):
    """A call whose scratch exceeds the static array fails with a clear
    error before touching the device."""
    big = MembraneArgs()
    big.n_platelets, big.n_elem, big.n_membrane, big.n_tri, big.n_node = 100000, 600, 400, 796, 1594
    big.precision = 1
    for f in ("X", "Y", "RY", "Z", "tri", "node_ntri", "ring", "spring_ptr", "S0", "S0_all", "V0", "F_out"):
        setattr(big, f, C.c_void_p(16))  # never dereferenced: the size check comes first
    rc = lib.pfgpu_membrane_forces_noalloc(C.byref(big), None)
    assert rc == 1
    msg = lib.pfgpu_last_error().decode()
    assert "scratch" in msg and str(lib.pfgpu_membrane_noalloc_scratch_bytes()) in msg


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
def test_noalloc_rejects_inconsistent_node_ntri(lib, prec):
    """node_ntri one above a node's real triangle count (still within 0..10,
    so every read stays inside the caller's arrays): the pass writes nothing
    and the status call reports the inconsistency; the next consistent call
    works again."""
    torch = pytest.importorskip("torch")
    sc = _scene()
    bad = np.array(sc.node_ntri, dtype=np.int32)
    q = int(np.argmax(bad < 10))
    bad[q] += 1
    F, _, _ = _call(lib, sc, prec, torch, node_ntri=bad, expect_rc=1, fill=7.0)
    assert "inconsistent" in lib.pfgpu_last_error().decode()
    assert np.all(F == 7.0)  # F_out untouched
    F_job, _ = _job_reference(sc, prec)
    F2, _, _ = _call(lib, sc, prec, torch)
    np.testing.assert_array_equal(F2, F_job)
