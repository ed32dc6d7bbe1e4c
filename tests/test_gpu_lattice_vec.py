"""The vector lattice step (several x-nodes per thread, each population plane
moved as one 8- or 16-byte vector, x-neighbours by warp shuffle or a direct
load at warp, row and idle-lane edges) does per node the arithmetic of the
one-node-per-thread kernel in the same order: on lattices without markers
(no float atomics anywhere in the step) the two give the same bits, for
every vector width, row widths that are and are not whole warps, and the
first step after an upload as well as later ones.  With markers the step
still follows the oracle (the parity tests run this kernel by default)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def _lattice_only(nx, ny, nz, seed=3):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(seed=seed, nx=nx, ny=ny, nz=nz, n_fib=0, n_links=0)
    sc.n_platelets = 0
    sc.n_rec = 0
    sc.n_fib = 0
    return sc


def _run(gpu, sc, prec, width, steps):
    old = os.environ.get("PFGPU_LBM_VEC")
    os.environ["PFGPU_LBM_VEC"] = str(width)
    try:
        j = gpu.Job(sc, prec)
        j.step(steps, graph=True)
        L = j.lattice()
        j.close()
        return L
    finally:
        if old is None:
            os.environ.pop("PFGPU_LBM_VEC", None)
        else:
            os.environ["PFGPU_LBM_VEC"] = old


@pytest.mark.parametrize("dims", [(40, 32, 20), (256, 8, 12), (48, 10, 9)], ids=["40", "256", "48"])
@pytest.mark.parametrize("prec,width", [(1, 2), (1, 4), (2, 2), (2, 4), (2, 8)],
                         ids=["f32v2", "f32v4", "f16v2", "f16v4", "f16v8"])
def test_vector_step_bit_identical_without_markers(gpu, prec, width, dims):
    sc = _lattice_only(*dims)
    ref = _run(gpu, sc, prec, 0, 7)
    got = _run(gpu, sc, prec, width, 7)
    for k in ("fIN", "rho", "u"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


@pytest.mark.parametrize("prec,width,tol", [(1, 2, 1e-6), (2, 4, 1e-3)], ids=["f32v2", "f16v4"])
def test_vector_step_with_markers_matches_scalar(gpu, prec, width, tol):
    """With markers the spreading's float atomics differ run to run, so the
    two kernels agree to that rounding."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    ref = _run(gpu, sc, prec, 0, 10)
    got = _run(gpu, sc, prec, width, 10)
    assert np.abs(got["fIN"] - ref["fIN"]).max() <= tol * np.abs(ref["fIN"]).max()
