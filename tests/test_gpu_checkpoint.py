"""Job state snapshots (pfgpu_job_save / pfgpu_job_restore): a job restored
from a snapshot reads back exactly the saved state (lattice, elements, bonds,
fibrin, step counter) and continues as the saved job does -- bit for bit where
the step has no atomics (a marker-free lattice in FP32 and FP16), and to the
run-to-run rounding of the atomics otherwise (spreading, FP64 included),
with receptor bond states bit for bit.  A snapshot of another job layout is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def _state(j, sc):
    L = j.lattice()
    out = dict(steps=j.steps, fIN=L["fIN"], rho=L["rho"], u=L["u"])
    if sc.n_platelets:
        E, B = j.elements(), j.bonds()
        out.update(X=E["X"], Y=E["Y"], Z=E["Z"], RY=E["RY"], rec=B["rec_state"], vwf=B["vwf"])
    if sc.n_fib:
        F = j.fibrin()
        out["fX"] = F["X"]
        out["fV"] = F["V"]
    return out


def _scene(kind):
    from platelet_fiber_gpu_gb300 import workloads as W
    from platelet_fiber_gpu_gb300.scene import FIBCPL_PENALTY
    if kind == "full":
        return W.mixed_small()
    if kind == "penalty":
        # fibrin nodes with their own velocity: the node velocities and the
        # pending penalty reaction are part of the state
        sc = W.mixed_small()
        sc.fib_coupling = FIBCPL_PENALTY
        sc.fib_gamma = 0.05
        return sc
    sc = W.mixed_small(n_fib=300 if kind == "fibrin" else 0, n_links=600 if kind == "fibrin" else 0)
    sc.n_platelets = 0
    sc.n_rec = 0
    if kind == "lattice":
        sc.n_fib = 0
    return sc


@pytest.mark.parametrize("kind,prec,exact", [("fibrin", 0, False), ("lattice", 1, True), ("lattice", 2, True),
                                             ("full", 0, False), ("full", 1, False), ("full", 2, False),
                                             ("penalty", 1, False)],
                         ids=["fibrin-fp64", "lattice-fp32", "lattice-fp16", "full-fp64", "full-fp32", "full-fp16",
                              "penalty-fp32"])
def test_restore_resumes_the_saved_job(gpu, kind, prec, exact):
    sc = _scene(kind)
    a = gpu.Job(sc, prec)
    a.step(6)
    snap = a.save()
    at6 = _state(a, sc)
    a.step(5)
    at11 = _state(a, sc)
    a.close()
    b = gpu.Job(sc, prec)
    b.step(2)  # the restore replaces whatever the job had done
    b.restore(snap)
    got6 = _state(b, sc)
    for k, v in at6.items():
        np.testing.assert_array_equal(got6[k], v, err_msg=k)
    b.step(5)
    got11 = _state(b, sc)
    b.close()
    assert got11["steps"] == 11
    tol = 0 if exact else {0: 1e-13, 1: 1e-5, 2: 1e-3}[prec]
    for k, v in at11.items():
        if k in ("rec", "vwf", "steps") or exact:
            np.testing.assert_array_equal(got11[k], v, err_msg=k)
        else:
            assert np.abs(got11[k] - v).max() <= tol * max(np.abs(v).max(), 1.0), k


def test_snapshot_of_another_layout_is_refused(gpu):
    from platelet_fiber_gpu_gb300 import workloads as W
    a = gpu.Job(W.mixed_small(), 1)
    snap = a.save()
    a.close()
    other = gpu.Job(W.mixed_small(nx=48), 1)
    with pytest.raises(gpu.PfgpuError):
        other.restore(snap)
    fp64 = gpu.Job(W.mixed_small(), 0)
    with pytest.raises(gpu.PfgpuError):
        fp64.restore(snap)
    with pytest.raises(gpu.PfgpuError):
        fp64.restore(snap[:100])
    other.close()
    fp64.close()
