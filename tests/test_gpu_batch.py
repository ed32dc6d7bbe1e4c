"""Batch API (continuous batching of independent jobs): jobs stepped together
give the results they give alone; admission respects the device-memory
budget; retiring returns the memory."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def test_batched_jobs_match_standalone(gpu):
    from platelet_fiber_gpu_gb300 import workloads as W
    scenes = [W.mixed_small(seed=3), W.mixed_small(seed=5, nx=48)]
    b = gpu.Batch(8 << 30)
    slots = [b.admit(sc, 0) for sc in scenes]
    assert None not in slots and b.num_jobs == 2
    b.step(4)
    b.step(6)
    for sc, s in zip(scenes, slots):
        ref = gpu.Job(sc, 0)
        ref.step(10)
        got = b.job(s)
        assert got.steps == 10
        a, r = got.lattice()["fIN"], ref.lattice()["fIN"]
        assert np.abs(a - r).max() / np.abs(r).max() < 1e-13
        np.testing.assert_array_equal(got.bonds()["rec_state"], ref.bonds()["rec_state"])
        ref.close()
    b.close()


def test_batch_budget_and_retire(gpu):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    need = gpu.scene_device_bytes(sc, 1)
    b = gpu.Batch(int(need * 1.5))
    s0 = b.admit(sc, 1)
    assert s0 is not None
    used = b.bytes_in_use
    assert 0 < used <= need
    assert b.admit(sc, 1) is None  # a second copy does not fit
    b.retire(s0)
    assert b.bytes_in_use == 0 and b.num_jobs == 0
    s1 = b.admit(sc, 1)
    assert s1 == s0
    b.step(2)
    assert b.status(s1) == 0
    b.close()


def test_served_loop_small(gpu):
    """A short Poisson-arrival run of the serving loop completes every job and
    reports latencies."""
    from platelet_fiber_gpu_gb300 import serve
    r = serve.run_served(1, rate=8.0, duration=0.5, steps_range=(20, 60), pool=3, chunk=20)
    assert r["jobs"] >= 1 and r["mlups"] > 0
    assert 0 < r["latency_p50_s"] <= r["latency_p99_s"]


def _fused_scenes():
    from platelet_fiber_gpu_gb300 import workloads as W
    return [W.mixed_small(seed=3), W.mixed_small(seed=5, nx=48, n_fib=0, n_links=0), W.batch_job(3, 0),
            W.batch_job(3, 5)]


@pytest.mark.parametrize("prec,tol", [(1, 1e-5), (2, 1e-3)], ids=["fp32", "fp16"])
def test_fused_batch_matches_standalone(gpu, prec, tol, monkeypatch):
    """Reduced-precision batches step through the fused batch kernels (one
    launch per kernel over every job, per-job CTA offsets); each job's state
    matches the same job stepped alone and the per-job-graph batch
    (PFGPU_BATCH_FUSED=0).  Float atomics make the spreading order differ, so
    the lattice agrees to rounding; bond states exactly."""
    scenes = _fused_scenes()
    fused = gpu.Batch(16 << 30)
    fslots = [fused.admit(sc, prec) for sc in scenes]
    monkeypatch.setenv("PFGPU_BATCH_FUSED", "0")
    plain = gpu.Batch(16 << 30)
    pslots = [plain.admit(sc, prec) for sc in scenes]
    plain.step(4)
    plain.step(3)
    monkeypatch.delenv("PFGPU_BATCH_FUSED")
    fused.step(4)
    fused.step(3)
    for sc, fs, ps in zip(scenes, fslots, pslots):
        ref = gpu.Job(sc, prec)
        ref.step(7)
        for other in (fused.job(fs), plain.job(ps)):
            assert other.steps == 7
            a, r = other.lattice()["fIN"], ref.lattice()["fIN"]
            assert np.abs(a - r).max() / np.abs(r).max() < tol
            if sc.n_platelets:
                ea, er = other.elements(), ref.elements()
                for k in ("X", "Y", "Z"):
                    assert np.abs(ea[k] - er[k]).max() < 1e-6
                np.testing.assert_array_equal(other.bonds()["rec_state"], ref.bonds()["rec_state"])
            if sc.n_fib:
                assert np.abs(other.fibrin()["X"] - ref.fibrin()["X"]).max() < 1e-6
        ref.close()
    fused.close()
    plain.close()


@pytest.mark.parametrize("shape", [(1, 2, 64), (16, 16, 256), (2, 4, 96)], ids=["r1l2t64", "r16l16t256", "r2l4t96"])
def test_forced_shapes_match_standalone(gpu, shape):
    """Every block/tile shape of the fused step computes the same updates:
    a batch forced to a shape matches the jobs stepped alone."""
    scenes = _fused_scenes()
    b = gpu.Batch(16 << 30)
    slots = [b.admit(sc, 1) for sc in scenes]
    b.set_shape(*shape)
    assert b.shape() == (shape, 1)
    b.step(5)
    for sc, s in zip(scenes, slots):
        ref = gpu.Job(sc, 1)
        ref.step(5)
        got = b.job(s)
        a, r = got.lattice()["fIN"], ref.lattice()["fIN"]
        assert np.abs(a - r).max() / np.abs(r).max() < 1e-5
        if sc.n_platelets:
            np.testing.assert_array_equal(got.bonds()["rec_state"], ref.bonds()["rec_state"])
        ref.close()
    b.close()


def test_autotuner_fixes_a_shape_and_caches_it(gpu, tmp_path, monkeypatch):
    """The autotuner measures candidate shapes on the batch's own steps
    (coordinate descent over the three axes), then runs the fastest; the jobs
    advance by exactly the steps asked for and match the same jobs stepped
    alone; the class's result is reused by a new batch and written to
    PFGPU_TUNE_CACHE."""
    from platelet_fiber_gpu_gb300 import workloads as W
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("PFGPU_TUNE_CACHE", str(cache))
    scenes = [W.batch_job(7, 2), W.batch_job(9, 0)]
    b = gpu.Batch(16 << 30)
    slots = [b.admit(sc, 1) for sc in scenes]
    shape, state = b.shape()
    assert state == 0 and shape == (8, 8, 128)  # the default runs between trials
    taken = b.tune(max_steps=600, chunk=30)
    shape, state = b.shape()
    assert state == 1, taken
    assert shape[0] in (1, 2, 4, 8, 16, 32, 64) and shape[1] in (2, 4, 8, 16, 32, 64)
    assert shape[2] in (32, 64, 128, 256)
    b.step(4)
    for sc, s in zip(scenes, slots):
        ref = gpu.Job(sc, 1)
        ref.step(taken + 4)
        got = b.job(s)
        assert got.steps == taken + 4
        a, r = got.lattice()["fIN"], ref.lattice()["fIN"]
        assert np.abs(a - r).max() / np.abs(r).max() < 1e-4
        if sc.n_platelets:
            np.testing.assert_array_equal(got.bonds()["rec_state"], ref.bonds()["rec_state"])
        ref.close()
    b2 = gpu.Batch(16 << 30)
    for sc in scenes:
        b2.admit(sc, 1)
    assert b2.shape() == (shape, 1)
    b2.close()
    b.close()
    line = cache.read_text().split()
    assert [int(v) for v in line[1:4]] == list(shape)


def test_stop_steps(gpu):
    """A job given a stop step halts there by itself (later steps do nothing,
    the status reads done) and matches the same job stepped exactly that far;
    a later stop step lets it run on.  In a fused batch, jobs with different
    stop steps leave the batch step by themselves."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(seed=3)
    j = gpu.Job(sc, 1)
    j.set_stop(5)
    assert j.step(9) == gpu.PFGPU_DONE
    assert j.steps == 5
    ref = gpu.Job(sc, 1)
    ref.step(5)
    # float atomics in the spreading: equal to rounding, not bit for bit
    a, r = j.lattice()["fIN"], ref.lattice()["fIN"]
    assert np.abs(a - r).max() / np.abs(r).max() < 1e-6
    assert np.abs(j.elements()["X"] - ref.elements()["X"]).max() < 1e-9
    j.set_stop(8)
    assert j.step(2) == 0 and j.steps == 7
    assert j.step(5) == gpu.PFGPU_DONE and j.steps == 8
    j.close()
    ref.close()

    scenes = _fused_scenes()
    b = gpu.Batch(16 << 30)
    slots = [b.admit(s, 1) for s in scenes]
    stops = [3, 6, 0, 4]
    for s, t in zip(slots, stops):
        b.set_stop(s, t)
    b.step(8)
    for sc, s, t in zip(scenes, slots, stops):
        got = b.job(s)
        assert got.steps == (t or 8)
        assert b.status(s) == (gpu.PFGPU_DONE if t else 0)
        r = gpu.Job(sc, 1)
        r.step(t or 8)
        a, e = got.lattice()["fIN"], r.lattice()["fIN"]
        assert np.abs(a - e).max() / np.abs(e).max() < 1e-5
        r.close()
    b.close()


def test_next_path_options_in_a_batch(gpu):
    """Jobs with the reference's "next" code paths (FEM bending chain, y
    inflow/outflow planes, fibrin penalty coupling) share a batch with a
    plain job: the batch steps the three through their own graphs and the
    plain ones fused, and every job ends where it ends alone."""
    from platelet_fiber_gpu_gb300 import workloads as W
    from platelet_fiber_gpu_gb300.scene import FIBCPL_PENALTY, MEM_ALL, MEM_FEMBEND
    fem = W.mixed_small(seed=3)
    fem.membrane_forces = MEM_ALL | MEM_FEMBEND
    inout = W.inflow_small(seed=4)
    pen = W.mixed_small(seed=5)
    pen.fib_coupling = FIBCPL_PENALTY
    pen.fib_gamma = 0.02
    plain = W.mixed_small(seed=6)
    scenes = [fem, inout, pen, plain]
    b = gpu.Batch(16 << 30)
    slots = [b.admit(sc, 1) for sc in scenes]
    assert None not in slots
    b.step(5)
    b.step(3)
    for sc, s in zip(scenes, slots):
        ref = gpu.Job(sc, 1)
        ref.step(8)
        got = b.job(s)
        assert got.steps == 8
        a, r = got.lattice()["fIN"], ref.lattice()["fIN"]
        assert np.abs(a - r).max() / np.abs(r).max() < 1e-5
        ea, er = got.elements(), ref.elements()
        for k in ("X", "Y", "Z"):
            assert np.abs(ea[k] - er[k]).max() < 1e-6
        assert np.abs(got.fibrin()["X"] - ref.fibrin()["X"]).max() < 1e-6
        np.testing.assert_array_equal(got.bonds()["rec_state"], ref.bonds()["rec_state"])
        ref.close()
    b.close()
