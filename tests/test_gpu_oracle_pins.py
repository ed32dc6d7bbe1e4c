"""Batched, served and long or full-size runs against the FP64 CPU oracle of
the same scenes (the reference's kernel logic, pinned to its golden
vectors), not only against the standalone CUDA job:

- every job of a fused batch (FP32, FP16-shifted; default and forced block
  shapes) after a few steps;
- every job the served loop (continuous batching, Poisson arrivals) finishes,
  against the same scene stepped alone on the GPU and against the oracle;
- the FP32 method over 1000 steps on a scene whose receptors bind and
  unbind (some to two vWF sites), bond states bit for bit;
- the 256x128x128 benchmark channel (50 platelets, 20k fibrin nodes, 10k
  receptors) against the oracle for 100 steps, and two FP32 runs of it
  against each other.

Tolerances (relative L2 against FP64): velocity 2e-5 FP32, 1e-3 FP16;
element and fibrin positions 1e-7 FP32 (1e-6 over 1000 steps), 1e-6
FP16-shifted; receptor bond states and vWF slot tables bit-exact.  Float
atomics in the spreading make two FP32 runs differ in the last bits of the
lattice; bond states may not differ.
"""
import numpy as np
import pytest

from conftest import assert_matches_oracle, oracle_state

pytestmark = pytest.mark.gpu

POS_TOL = {1: 1e-7, 2: 1e-6}  # element / fibrin positions, relative L2 against FP64


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def _rl2(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


_SCENES = {}


def _fused_scenes():
    from platelet_fiber_gpu_gb300 import workloads as W
    if not _SCENES:
        _SCENES.update({
            "ms3": W.mixed_small(seed=3),
            "ms5": W.mixed_small(seed=5, nx=48, n_fib=0, n_links=0),
            "bj0": W.batch_job(3, 0),
            "bj5": W.batch_job(3, 5),
        })
    return _SCENES


@pytest.mark.parametrize("prec", [1, 2], ids=["fp32", "fp16"])
def test_fused_batch_jobs_match_the_oracle(gpu, prec):
    scenes = _fused_scenes()
    b = gpu.Batch(16 << 30)
    slots = {k: b.admit(sc, prec) for k, sc in scenes.items()}
    b.step(4)
    b.step(3)
    for k, sc in scenes.items():
        assert_matches_oracle(b.job(slots[k]), oracle_state(sc, 7, key=k), prec, pos_tol=POS_TOL[prec])
    b.close()


@pytest.mark.parametrize("shape", [(1, 2, 64), (16, 16, 256), (2, 4, 96)], ids=["r1l2t64", "r16l16t256", "r2l4t96"])
def test_forced_shapes_match_the_oracle(gpu, shape):
    scenes = _fused_scenes()
    b = gpu.Batch(16 << 30)
    slots = {k: b.admit(sc, 1) for k, sc in scenes.items()}
    b.set_shape(*shape)
    b.step(5)
    for k, sc in scenes.items():
        assert_matches_oracle(b.job(slots[k]), oracle_state(sc, 5, key=k), 1)
    b.close()


@pytest.mark.parametrize("prec", [1, 2], ids=["fp32", "fp16"])
def test_served_jobs_same_alone_in_the_mix_and_vs_oracle(gpu, prec):
    """Jobs arrive while others run (Poisson, 60/s), join the fused batch as
    memory and slots free up, and leave at their own step counts.  Each
    finished job's state equals the same scene stepped alone (to float-atomic
    rounding, bonds exactly) and follows the oracle."""
    from platelet_fiber_gpu_gb300 import serve
    from platelet_fiber_gpu_gb300 import workloads as W
    pool = [W.mixed_small(seed=3), W.mixed_small(seed=6, nx=32, n_fib=100, n_links=200), W.batch_job(3, 0)]
    finished = []

    def keep(idx, req, job):
        finished.append(dict(idx=idx, req=req, steps=job.steps, fIN=job.lattice()["fIN"], u=job.lattice()["u"],
                             E=job.elements(), B=job.bonds(), Fb=job.fibrin()))

    r = serve.run_served(prec, rate=60.0, duration=0.4, seed=11, budget=4e9, chunk=10, steps_range=(10, 40),
                         scenes=pool, on_finish=keep)
    assert len(finished) == r["jobs"] >= 5
    assert r["mean_live_jobs"] > 1  # the jobs overlapped on the device
    tol = {1: 1e-5, 2: 1e-3}[prec]
    alone = {}
    for f in finished:
        sc = pool[f["idx"]]
        assert f["steps"] == f["req"]
        key = (f["idx"], f["req"])
        if key not in alone:
            j = gpu.Job(sc, prec)
            j.step(f["req"])
            alone[key] = dict(fIN=j.lattice()["fIN"], E=j.elements(), B=j.bonds())
            j.close()
        a = alone[key]
        assert np.abs(f["fIN"] - a["fIN"]).max() / np.abs(a["fIN"]).max() < tol
        for k in ("X", "Y", "Z"):  # um; FP16 stores amplify the atomics' rounding
            assert np.abs(f["E"][k] - a["E"][k]).max() < {1: 1e-6, 2: 1e-5}[prec]
        np.testing.assert_array_equal(f["B"]["rec_state"], a["B"]["rec_state"])
        ref = oracle_state(sc, f["req"], key=("served", f["idx"]))
        assert _rl2(f["u"], ref["u"]) < {1: 2e-5, 2: 1e-3}[prec]
        pos = np.stack([f["E"]["X"], f["E"]["Y"], f["E"]["Z"]])
        assert _rl2(pos, np.stack([ref["E"]["X"], ref["E"]["Y"], ref["E"]["Z"]])) < POS_TOL[prec]
        np.testing.assert_array_equal(f["B"]["rec_state"], ref["B"]["rec_state"])
        np.testing.assert_array_equal(f["B"]["vwf"], ref["B"]["vwf"])
        assert _rl2(f["Fb"]["X"], ref["Fb"]["X"]) < POS_TOL[prec]


def test_fp32_1000_steps_with_binding_receptors(gpu):
    """FP32 coupled step, 1000 steps, two platelets 0.02 um above the wall
    with 100 receptors each (p_on 0.2, p_off 0.05 per step): bonds form,
    break and double up; every receptor state and vWF slot equals the
    oracle's, velocity and positions within the FP32 tolerances."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(wall_gap=0.02, n_rec=100)
    ref = oracle_state(sc, 1000, key="binding1000")
    st = ref["B"]["rec_state"]
    assert (st[..., 2] > 0).sum() >= 5 and (st[..., 2] > 1).sum() >= 1  # the scene exercises binding
    j = gpu.Job(sc, 1)
    j.step(1000)
    assert_matches_oracle(j, ref, 1, pos_tol=1e-6)
    j.close()


@pytest.fixture(scope="module")
def large_scene():
    from platelet_fiber_gpu_gb300 import workloads as W
    return W.single_large()


def test_single_large_fp32_vs_oracle_100_steps(gpu, large_scene):
    """The benchmark channel at full size, 100 steps, against the CPU oracle
    (stencil-local IBM, FP64, all host threads)."""
    sc = large_scene
    ref = oracle_state(sc, 100, key="single_large100")
    j = gpu.Job(sc, 1)
    j.step(100)
    L, E, B = j.lattice(), j.elements(), j.bonds()
    j.close()
    assert _rl2(L["u"], ref["u"]) < 2e-5
    assert _rl2(L["rho"] - 1, ref["rho"] - 1) < 1e-4
    pos = np.stack([E["X"], E["Y"], E["Z"]])
    assert _rl2(pos, np.stack([ref["E"]["X"], ref["E"]["Y"], ref["E"]["Z"]])) < 1e-7
    differ = int((B["rec_state"] != ref["B"]["rec_state"]).any(axis=-1).sum())
    print(f"single_large 100 steps: receptor states differing from the oracle: {differ} of "
          f"{B['rec_state'].shape[0] * B['rec_state'].shape[1]}; bound {(B['rec_state'][..., 2] > 0).sum()}")
    assert differ == 0
    np.testing.assert_array_equal(B["vwf"], ref["B"]["vwf"])


def test_single_large_fp32_runs_repeat_bond_states(gpu, large_scene):
    """Two FP32 runs of the full-size channel (float atomics in the spreading
    sum in different orders, so positions differ in their last FP32-scale
    bits) reach the same receptor and vWF states."""
    runs = []
    for _ in range(2):
        j = gpu.Job(large_scene, 1)
        j.step(200)
        runs.append((j.bonds(), j.elements()["Z"]))
        j.close()
    np.testing.assert_array_equal(runs[0][0]["rec_state"], runs[1][0]["rec_state"])
    np.testing.assert_array_equal(runs[0][0]["vwf"], runs[1][0]["vwf"])
    assert np.abs(runs[0][1] - runs[1][1]).max() < 1e-6
