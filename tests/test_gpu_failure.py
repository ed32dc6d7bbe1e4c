"""Failure detection on the device without a GPU fault: every spin-wait of
the library's kernels is bounded.  The row-staged lattice kernel waits on
mbarriers for its bulk copies; with the wait limit set to zero
(PFGPU_WAIT_LIMIT_NS=0, the first unfinished wait gives up) the kernel takes
its give-up path: it sets ERR_WAIT_TIMEOUT in the job's control block, waits
(with the normal limit) for the copies it issued, and returns.  The host
reads the bit after the step and the job reports it; the context stays
usable and the same scene then runs normally."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_WAIT_TIMEOUT = 0x10
PFGPU_ERR_DEVICE = 5


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def _lattice_only():
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(nx=64, ny=16, nz=12, n_fib=0, n_links=0)
    sc.n_platelets = 0
    sc.n_rec = 0
    sc.n_fib = 0
    return sc


def test_bounded_wait_gives_up_and_the_job_reports_it(gpu, monkeypatch):
    sc = _lattice_only()
    monkeypatch.setenv("PFGPU_LBM_KERNEL", "rows")
    monkeypatch.setenv("PFGPU_WAIT_LIMIT_NS", "0")
    j = gpu.Job(sc, 1)
    assert j.lbm_kernel == "lbm_rows_k"
    with pytest.raises(gpu.PfgpuError) as e:
        j.step(2, graph=False)
    assert e.value.code == PFGPU_ERR_DEVICE
    assert f"0x{ERR_WAIT_TIMEOUT:x}" in str(e.value)
    j.close()
    # normal limit: the same kernel runs the scene and agrees with the
    # direct-gather kernel (the context survived the give-up path)
    monkeypatch.delenv("PFGPU_WAIT_LIMIT_NS")
    a = gpu.Job(sc, 1)
    assert a.lbm_kernel == "lbm_rows_k"
    assert a.step(4, graph=False) == 0
    monkeypatch.delenv("PFGPU_LBM_KERNEL")
    b = gpu.Job(sc, 1)
    assert b.step(4, graph=False) == 0
    fa, fb = a.lattice()["fIN"], b.lattice()["fIN"]
    assert np.abs(fa - fb).max() <= 1e-6 * np.abs(fb).max()
    a.close()
    b.close()
