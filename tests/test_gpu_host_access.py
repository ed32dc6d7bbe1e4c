"""Job creation and the lattice download read and write the caller's host
arrays where they lie when the device can reach them (pinned memory, or any
host memory where the GPU walks the host page tables), and stage them
through device copies otherwise (PFGPU_HOST_DIRECT=0).  The three routes
must give the same bits for the initial lattice they build and download;
after a few steps they agree to the run-to-run rounding of the atomics in
the step (float spreading, FP64 area/volume sums); and the FP64 route still
follows the oracle (the one-pass initial-state kernel replaces the former
upload, moments and equilibrium kernels)."""
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


def _scene_with_populations(gpu, bounce):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.plain_small(nx=32, ny=16, nz=16) if bounce else W.mixed_small()
    j = gpu.Job(sc, 0)
    j.step(3, graph=False)
    f = j.lattice()["fIN"]
    j.close()
    sc.f_init = np.ascontiguousarray(f)
    return sc


def _run(gpu, sc, prec, route, steps=4):
    old = os.environ.get("PFGPU_HOST_DIRECT")
    try:
        if route == "staged":
            os.environ["PFGPU_HOST_DIRECT"] = "0"
        else:
            os.environ.pop("PFGPU_HOST_DIRECT", None)
        if route == "pinned":
            f = gpu.pinned(sc.f_init.shape)
            f[:] = sc.f_init
            keep, sc.f_init = sc.f_init, f
        j = gpu.Job(sc, prec)
        if route == "pinned":
            sc.f_init = keep
        N = sc.n_nodes
        if route == "pinned":
            out = {"fIN": gpu.pinned((19, N)), "rho": gpu.pinned(N), "u": gpu.pinned((3, N)), "F": gpu.pinned((3, N))}
        else:
            out = None
        L0 = {k: (None if v is None else np.array(v)) for k, v in j.lattice(out=out).items()}
        j.step(steps, graph=True)
        L1 = {k: (None if v is None else np.array(v)) for k, v in j.lattice(out=out).items()}
        E = j.elements()
        j.close()
        return L0, L1, E
    finally:
        if old is None:
            os.environ.pop("PFGPU_HOST_DIRECT", None)
        else:
            os.environ["PFGPU_HOST_DIRECT"] = old


@pytest.mark.parametrize("bounce", [False, True], ids=["zouhe", "bounceback"])
@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "fp32", "fp16"])
def test_routes_give_the_same_bits(gpu, prec, bounce):
    sc = _scene_with_populations(gpu, bounce)
    ref = _run(gpu, sc, prec, "staged")
    for route in ("direct", "pinned"):
        got = _run(gpu, sc, prec, route)
        for k in ("fIN", "rho", "u", "F"):
            np.testing.assert_array_equal(got[0][k], ref[0][k], err_msg=f"{route} {k}")
        tol = {0: 1e-13, 1: 1e-5, 2: 1e-3}[prec]
        for k in ("fIN", "rho", "u"):
            a, b = got[1][k], ref[1][k]
            assert np.abs(a - b).max() <= tol * np.abs(b).max(), (route, k)
        for k in ("X", "Y", "Z"):
            assert np.abs(got[2][k] - ref[2][k]).max() < 1e-7, (route, k)


def test_uploaded_populations_follow_the_oracle(gpu):
    """Given populations (no rho/u): the first step's moments come from them;
    FP64 after a few steps equals the oracle started from the same arrays."""
    from oracle import binding as ob
    sc = _scene_with_populations(gpu, False)
    o = ob.Oracle(sc)
    o.step(4)
    _, L1, E = _run(gpu, sc, 0, "direct")
    Lo, Eo = o.lattice(), o.elements()
    o.close()
    assert np.abs(L1["fIN"] - Lo["fIN"]).max() / np.abs(Lo["fIN"]).max() < 1e-12
    assert np.abs(E["X"] - Eo["X"]).max() < 1e-10
