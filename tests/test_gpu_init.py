"""The initial lattice of a scene without populations is the equilibrium of
its initial flow (rest, or the Zou/He channel's linear shear profile),
computed on the device in FP64 with the operation order of the reference
driver's host loop (gpuSEM_LB.c:1206-1258): the populations a job reports
before its first step match a numpy restatement of that loop to rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0], dtype=np.float64)
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1], dtype=np.float64)
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1], dtype=np.float64)
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def equilibrium(sc):
    from platelet_fiber_gpu_gb300.scene import P_SHEAR, P_UMAX
    p = sc.params
    shear = float(p[P_SHEAR])
    umax = shear * (sc.nz - 1) * float(np.float32(sc.dx)) if shear > 0 else float(p[P_UMAX])
    C0 = float(np.float32(np.float32(sc.dx) / np.float32(sc.dt))) / umax
    z = np.arange(sc.nz, dtype=np.float64)[:, None, None] * np.ones((sc.nz, sc.ny, sc.nx))
    u1 = shear * z * float(np.float32(sc.dx)) / umax
    uu = u1 * u1
    f = np.empty((19,) + z.shape)
    for d in range(19):
        cu = 3.0 * (CY[d] * u1)
        f[d] = 1.0 * W[d] * (1.0 + cu / C0 + 0.5 * cu * cu / (C0 * C0) - 1.5 * uu / (C0 * C0))
    return f.reshape(19, -1)


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


@pytest.mark.parametrize("prec,tol", [(0, 1e-15), (1, 1e-7), (2, 2e-3)], ids=["fp64", "fp32", "fp16"])
def test_initial_lattice_is_the_equilibrium(gpu, prec, tol):
    from platelet_fiber_gpu_gb300 import workloads as W_
    sc = W_.mixed_small()
    j = gpu.Job(sc, prec)
    got = j.lattice()["fIN"]
    ref = equilibrium(sc)
    # populations are stored shifted by their weights (and in FP32 / FP16)
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
    j.close()
