"""The kernel count a job reports for one step (pfgpu_job_launches_per_step,
the bench line's `gpu_launches` per step).  After a graph step it is the
number of kernel nodes of the captured step graph divided by its steps; after
a direct step it is the count the step's schedule keeps as it launches.  The
two must agree for every kind of scene."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def _scene(kind):
    from platelet_fiber_gpu_gb300 import workloads as W
    from platelet_fiber_gpu_gb300.scene import FIBCPL_PENALTY
    sc = W.mixed_small()
    if kind == "lattice":
        sc.n_platelets = 0
        sc.n_rec = 0
        sc.n_fib = 0
    elif kind == "penalty":
        sc.fib_coupling = FIBCPL_PENALTY
        sc.fib_gamma = 0.05
        sc.fib_node_mass = 2.0
    elif kind == "no_fibrin":
        sc.n_fib = 0
    return sc


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "fp32", "fp16"])
@pytest.mark.parametrize("kind", ["lattice", "mixed", "penalty", "no_fibrin"])
def test_step_kernel_count_matches_the_captured_graph(gpu, kind, prec):
    sc = _scene(kind)
    j = gpu.Job(sc, prec)
    try:
        j.step(1, graph=False)
        direct = j.launches_per_step
        j.step(4, graph=True)
        graphed = j.launches_per_step
        assert j.steps == 5
    finally:
        j.close()
    assert graphed > 0
    assert direct == graphed
