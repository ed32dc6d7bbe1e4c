"""CUDA path (libpfgpu.so, through its C ABI) against the reference's golden
vectors and the CPU oracle.

Tolerances: FP64 lattice/positions to ~1e-12 (same arithmetic, different
summation order and libm); FP32 coupled step within 1e-5 relative L2 of the
FP64 oracle for velocity, density deviation and element positions after 1000
steps of the body-force channel; FP16-shifted populations within 1e-3; bond
states, vWF slot tables and cell lists bit-exact in every precision.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden"


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def rel_max(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def rel_l2(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def golden(name):
    from platelet_fiber_gpu_gb300.scene import scene_from_dict
    d = np.load(GOLDEN / f"{name}.npz")
    return scene_from_dict(d), int(d["nsteps"]), d


@pytest.mark.parametrize("name", ["ref_wall", "ref_edges", "ref_mesh958", "ref_fembend", "ref_fembend958"])
def test_fp64_matches_reference_kernels(gpu, name):
    sc, n, d = golden(name)
    j = gpu.Job(sc, 0)
    hist = []
    for _ in range(n):
        j.step(1)
        hist.append(j.bonds()["total"])
    L, E, B = j.lattice(), j.elements(), j.bonds()
    assert rel_max(L["fIN"], d["out.fIN"]) < 1e-13
    assert rel_max(L["rho"], d["out.rho"]) < 1e-13
    u_ref = np.stack([d["out.ux"], d["out.uy"], d["out.uz"]])
    assert rel_l2(L["u"], u_ref) < 1e-10
    for k in ("X", "Y", "RY", "Z"):
        assert np.abs(E[k] - d[f"out.{k}"]).max() < 1e-13
    np.testing.assert_array_equal(B["rec_state"], d["out.rec_state"])
    np.testing.assert_array_equal(B["vwf"], d["out.vwf"])
    np.testing.assert_array_equal(hist, d["out.total_bond"])
    j.close()


@pytest.mark.parametrize("name", ["ref_wall", "ref_mesh958"])
@pytest.mark.parametrize("prec,tol", [(1, 1e-4), (2, 2e-3)])
def test_reduced_precision_vs_reference_kernels(gpu, prec, tol, name):
    sc, n, d = golden(name)
    j = gpu.Job(sc, prec, 0.0)
    j.step(n)
    L, E, B = j.lattice(), j.elements(), j.bonds()
    u_ref = np.stack([d["out.ux"], d["out.uy"], d["out.uz"]])
    assert rel_l2(L["u"], u_ref) < tol
    pos = np.stack([E["X"], E["Y"], E["Z"]])
    pos_ref = np.stack([d["out.X"], d["out.Y"], d["out.Z"]])
    assert rel_l2(pos, pos_ref) < 1e-7
    np.testing.assert_array_equal(B["rec_state"], d["out.rec_state"])
    np.testing.assert_array_equal(B["vwf"], d["out.vwf"])
    j.close()


@pytest.mark.parametrize("name", ["ref_fembend", "ref_fembend958"])
@pytest.mark.parametrize("prec", [1, 2])
def test_fem_bending_reduced_precision(gpu, prec, name):
    """The reference's disabled FEM bending chain (sem_kernel.cu:1129-1497,
    launched in the slot of semLB.cu:518-520) in the FP32 per-vertex
    membrane kernel, against the reference kernels run with it: the chain
    dominates the membrane force of this case, so its FP32 rounding shows in
    the positions (tolerance written here), while bond states stay exact."""
    sc, n, d = golden(name)
    j = gpu.Job(sc, prec, 0.0)
    j.step(n)
    E, B = j.elements(), j.bonds()
    pos = np.stack([E["X"], E["Y"], E["Z"]])
    pos_ref = np.stack([d["out.X"], d["out.Y"], d["out.Z"]])
    err = rel_l2(pos, pos_ref)
    print(f"fem {name} prec {prec}: position rel L2 {err:.3e}")
    assert err < (1e-7 if prec == 1 else 5e-6)
    np.testing.assert_array_equal(B["rec_state"], d["out.rec_state"])
    j.close()


def _run_both(gpu, sc, n, prec, graph=True):
    from oracle import binding as ob
    o = ob.Oracle(sc)
    o.step(n)
    j = gpu.Job(sc, prec, 0.0)
    j.step(n, graph=graph)
    out = dict(Lo=o.lattice(), Lg=j.lattice(), Eo=o.elements(), Eg=j.elements(), Bo=o.bonds(), Bg=j.bonds(),
               Fo=o.fibrin() if sc.n_fib else None, Fg=j.fibrin() if sc.n_fib else None,
               Mo=o.membrane(), Mg=j.membrane())
    j.close()
    o.close()
    return out


@pytest.mark.parametrize("bell", [False, True], ids=["constant", "bell"])
def test_fp64_all_features_vs_oracle(gpu, bell):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(bell=bell)
    r = _run_both(gpu, sc, 20, 0)
    assert rel_max(r["Lg"]["fIN"], r["Lo"]["fIN"]) < 1e-12
    assert rel_l2(r["Lg"]["u"], r["Lo"]["u"]) < 1e-10
    assert rel_l2(r["Lg"]["F"], r["Lo"]["F"]) < 1e-10
    for k in ("X", "Y", "RY", "Z"):
        assert np.abs(r["Eg"][k] - r["Eo"][k]).max() < 1e-12
    assert rel_l2(r["Eg"]["F"], r["Eo"]["F"]) < 1e-10
    assert rel_l2(r["Fg"]["X"], r["Fo"]["X"]) < 1e-14
    assert rel_l2(r["Fg"]["F"], r["Fo"]["F"]) < 1e-9
    np.testing.assert_allclose(r["Mg"]["S_V"], r["Mo"]["S_V"], rtol=1e-12)
    np.testing.assert_allclose(r["Mg"]["km"], r["Mo"]["km"], rtol=1e-9, atol=1e-9)
    np.testing.assert_array_equal(r["Bg"]["rec_state"], r["Bo"]["rec_state"])
    np.testing.assert_array_equal(r["Bg"]["vwf"], r["Bo"]["vwf"])
    assert r["Bg"]["total"] == r["Bo"]["total"]


@pytest.mark.parametrize("prec,tol", [(1, 2e-5), (2, 1e-3)], ids=["fp32", "fp16"])
def test_reduced_precision_all_features_vs_oracle(gpu, prec, tol):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    r = _run_both(gpu, sc, 20, prec)
    assert rel_l2(r["Lg"]["u"], r["Lo"]["u"]) < tol
    pos = np.stack([r["Eg"]["X"], r["Eg"]["Y"], r["Eg"]["Z"]])
    pos_o = np.stack([r["Eo"]["X"], r["Eo"]["Y"], r["Eo"]["Z"]])
    assert rel_l2(pos, pos_o) < 1e-7
    np.testing.assert_array_equal(r["Bg"]["rec_state"], r["Bo"]["rec_state"])
    np.testing.assert_array_equal(r["Bg"]["vwf"], r["Bo"]["vwf"])


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "fp32", "fp16"])
def test_inflow_outflow_planes_vs_oracle(gpu, prec):
    """Velocity inlet / outlet on y (the reference's in/out-flow planes,
    LB_kernel.cu:78-392) with every marker feature, against the oracle: the
    FP64 lattice to 1e-12, reduced precision at the usual tolerances; the
    planes hold the prescribed shear profile."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.inflow_small()
    r = _run_both(gpu, sc, 20, prec)
    if prec == 0:
        assert rel_max(r["Lg"]["fIN"], r["Lo"]["fIN"]) < 1e-12
        assert rel_l2(r["Lg"]["u"], r["Lo"]["u"]) < 1e-10
        for k in ("X", "Y", "RY", "Z"):
            assert np.abs(r["Eg"][k] - r["Eo"][k]).max() < 1e-12
    else:
        assert rel_l2(r["Lg"]["u"], r["Lo"]["u"]) < (2e-5 if prec == 1 else 1e-3)
        pos = np.stack([r["Eg"]["X"], r["Eg"]["Y"], r["Eg"]["Z"]])
        pos_o = np.stack([r["Eo"]["X"], r["Eo"]["Y"], r["Eo"]["Z"]])
        assert rel_l2(pos, pos_o) < 1e-7
    np.testing.assert_array_equal(r["Bg"]["rec_state"], r["Bo"]["rec_state"])
    nx, ny, nz = sc.nx, sc.ny, sc.nz
    uy = r["Lg"]["u"][1].reshape(nz, ny, nx)
    prof = uy[-1, ny // 2, nx // 2] * np.arange(nz) / (nz - 1)
    for j in (0, ny - 1):
        assert np.abs(uy[2:-2, j, 2:-2] - prof[2:-2, None]).max() < 1e-3 * prof[-1]


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "fp32", "fp16"])
def test_fibrin_penalty_coupling_vs_oracle(gpu, prec):
    """Fibrin nodes with their own velocity (the reference's fibrin FSI
    design: penalty force from the flow at the node, reaction into the
    lattice, damped kick-drift-kick, fiber.cpp:501-814 and
    network.cpp:445-513,839-881) against the oracle, with friction."""
    from platelet_fiber_gpu_gb300 import workloads as W
    from platelet_fiber_gpu_gb300.scene import FIBCPL_PENALTY
    sc = W.mixed_small()
    sc.fib_coupling = FIBCPL_PENALTY
    sc.fib_gamma = 0.05
    sc.fib_node_mass = 2.0
    r = _run_both(gpu, sc, 20, prec)
    if prec == 0:
        assert rel_max(r["Lg"]["fIN"], r["Lo"]["fIN"]) < 1e-12
        assert rel_l2(r["Fg"]["X"], r["Fo"]["X"]) < 1e-14
        assert rel_l2(r["Fg"]["V"], r["Fo"]["V"]) < 1e-10
        assert rel_l2(r["Fg"]["F"], r["Fo"]["F"]) < 1e-9
    else:
        assert rel_l2(r["Lg"]["u"], r["Lo"]["u"]) < (2e-5 if prec == 1 else 1e-3)
        assert rel_l2(r["Fg"]["X"], r["Fo"]["X"]) < 1e-7
        assert rel_l2(r["Fg"]["V"], r["Fo"]["V"]) < (1e-4 if prec == 1 else 2e-3)
    np.testing.assert_array_equal(r["Bg"]["rec_state"], r["Bo"]["rec_state"])


def test_fp32_plain_channel_1000_steps(gpu):
    """The plain FP32 method on the 64x32x32 body-force channel with one
    600-element platelet and a 200-node fibrin mesh: velocity, density and
    element positions within 1e-5 relative L2 of the FP64 oracle after 1000
    steps."""
    from oracle import binding as ob
    from platelet_fiber_gpu_gb300 import workloads as W
    import os
    ob.set_threads(os.cpu_count() or 1)
    sc = W.plain_small()
    r = _run_both(gpu, sc, 1000, 1)
    assert rel_l2(r["Lg"]["u"], r["Lo"]["u"]) < 1e-5
    assert rel_l2(r["Lg"]["rho"] - 1, r["Lo"]["rho"] - 1) < 1e-5
    pos = np.stack([r["Eg"]["X"], r["Eg"]["Y"], r["Eg"]["Z"]])
    pos_o = np.stack([r["Eo"]["X"], r["Eo"]["Y"], r["Eo"]["Z"]])
    assert rel_l2(pos, pos_o) < 1e-5
    assert rel_l2(r["Fg"]["X"], r["Fo"]["X"]) < 1e-5


def test_graph_and_direct_stepping_agree(gpu):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    a = gpu.Job(sc, 0)
    b = gpu.Job(sc, 0)
    a.step(7, graph=True)
    b.step(7, graph=False)
    assert rel_max(a.lattice()["fIN"], b.lattice()["fIN"]) < 1e-14
    np.testing.assert_array_equal(a.bonds()["rec_state"], b.bonds()["rec_state"])
    assert a.steps == b.steps == 7


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 1e-5), (2, 1e-3)], ids=["fp64", "fp32", "fp16"])
def test_quiet_pass_schedules_agree(gpu, prec, tol, monkeypatch):
    """The quiet lattice pass at the fork, run ahead with one-step graphs, run
    ahead with four- and eight-step graphs, and run ahead while stepping
    directly give the same job, over step counts that leave remainders and
    across calls (the prologue of each call), a snapshot restore and a
    profiled step in between."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    variants = [dict(PFGPU_QUIET_AHEAD="0"), dict(PFGPU_GRAPH_STEPS="1"), dict(PFGPU_GRAPH_STEPS="4"),
                dict(PFGPU_GRAPH_STEPS="8"), dict(direct=True)]
    out = []
    for v in variants:
        for key in ("PFGPU_QUIET_AHEAD", "PFGPU_GRAPH_STEPS"):
            monkeypatch.delenv(key, raising=False)
        for key, val in v.items():
            if key != "direct":
                monkeypatch.setenv(key, val)
        j = gpu.Job(sc, prec, 0.0)
        g = not v.get("direct", False)
        j.step(5, graph=g)
        snap = j.save()
        j.step(9, graph=g)
        j.restore(snap)  # back to step 5: the next call runs its own prologue
        j.step(3, graph=g)
        j.profile(1)
        j.step(8, graph=g)
        assert j.steps == 17
        out.append((j.lattice()["fIN"], j.elements()["Z"], j.bonds()["rec_state"]))
        j.close()
    ref = out[0]
    for f, z, rs in out[1:]:
        assert rel_max(f, ref[0]) < tol
        assert np.abs(z - ref[1]).max() < (1e-12 if prec == 0 else 1e-6)
        np.testing.assert_array_equal(rs, ref[2])


@pytest.mark.parametrize("prec,tol", [(0, 1e-14), (1, 1e-6)], ids=["fp64", "fp32"])
def test_pipelined_and_serial_schedules_agree(gpu, prec, tol, monkeypatch):
    """The pipelined schedule updates the far region of step t+1 (bricks
    more than one brick / two rows from step t's force bricks) while step t
    spreads, passes its force bricks and interpolates; every node update is
    the one the serial schedule makes.  Graph and direct stepping, and a
    profile run in between (which restarts the pipeline), on a channel
    whose markers cover a small part of the lattice."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(nx=256, ny=64, nz=32, n_platelets=2, n_fib=40, n_links=60)
    monkeypatch.setenv("PFGPU_PIPELINE", "0")
    a = gpu.Job(sc, prec)
    monkeypatch.setenv("PFGPU_PIPELINE", "1")
    b = gpu.Job(sc, prec)
    monkeypatch.delenv("PFGPU_PIPELINE")
    for j in (a, b):
        j.step(5)
        j.step(3, graph=False)
        j.profile(2)
        j.step(4)
        assert j.steps == 14
    assert rel_max(a.lattice()["fIN"], b.lattice()["fIN"]) < tol
    for k in ("X", "Y", "Z"):
        assert rel_max(a.elements()[k], b.elements()[k]) < tol
    assert rel_max(a.fibrin()["X"], b.fibrin()["X"]) < tol
    np.testing.assert_array_equal(a.bonds()["rec_state"], b.bonds()["rec_state"])
    a.close()
    b.close()


def _lbm_scene(name):
    from platelet_fiber_gpu_gb300 import workloads as W
    if name == "shear":
        return W.mixed_small(nx=64)
    sc = W.plain_small(n_fib=0, n_links=0)
    sc.bc = (1, 1, 1)
    sc.ibm_wrap = (0, 0, 0)
    return sc


@pytest.mark.parametrize("scene", ["shear", "walls"])
@pytest.mark.parametrize("prec,tol", [(0, 1e-14), (1, 1e-6), (2, 1e-4)], ids=["fp64", "fp32", "fp16"])
def test_row_staged_and_direct_lbm_kernels_agree(gpu, scene, prec, tol, monkeypatch):
    """The row-staged step kernel (bulk copies into shared memory) and the
    direct-gather kernel do the same arithmetic on the same operands; the
    compiler may contract a different set of multiply-adds in each, so they
    agree to a few units in the last place (FP16: one step of the store).
    Scenes: Zou/He shear walls with periodic x/y, and a box with bounce-back
    on every axis (the x faces are read from global memory)."""
    sc = _lbm_scene(scene)
    monkeypatch.setenv("PFGPU_LBM_KERNEL", "rows")
    a = gpu.Job(sc, prec)
    monkeypatch.delenv("PFGPU_LBM_KERNEL")
    b = gpu.Job(sc, prec)
    assert a.lbm_kernel == "lbm_rows_k" and b.lbm_kernel != "lbm_rows_k"
    a.step(12)
    b.step(12)
    assert rel_max(a.lattice()["fIN"], b.lattice()["fIN"]) < tol
    assert rel_max(a.elements()["X"], b.elements()["X"]) < tol
    np.testing.assert_array_equal(a.bonds()["rec_state"], b.bonds()["rec_state"])
    a.close()
    b.close()


@pytest.mark.parametrize("prec,tol", [(1, 1e-6), (2, 1e-4)], ids=["fp32", "fp16"])
def test_one_thread_spreading_matches_four_lanes(gpu, prec, tol, monkeypatch):
    """The reduced-precision spreading with one thread per marker
    (PFGPU_SPREAD_LANES=1) and with four lanes per marker (the default) add
    the same product to the same nodes; only the order of the float atomics
    differs, so the two agree to that rounding (platelets, bonds and fibrin,
    all three force parts)."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    monkeypatch.setenv("PFGPU_SPREAD_LANES", "1")
    a = gpu.Job(sc, prec)
    monkeypatch.delenv("PFGPU_SPREAD_LANES")
    b = gpu.Job(sc, prec)
    a.step(5)
    b.step(5)
    La, Lb = a.lattice(), b.lattice()
    assert rel_l2(La["u"], Lb["u"]) < tol
    assert rel_l2(La["F"], Lb["F"]) < 10 * tol
    Ea, Eb = a.elements(), b.elements()
    for k in ("X", "Y", "Z"):
        assert np.abs(Ea[k] - Eb[k]).max() < 1e-3 * tol
    Fa, Fb = a.fibrin(), b.fibrin()
    assert np.abs(Fa["X"] - Fb["X"]).max() < 1e-3 * tol
    np.testing.assert_array_equal(a.bonds()["rec_state"], b.bonds()["rec_state"])
    a.close()
    b.close()


@pytest.mark.parametrize("prec,tol", [(1, 1e-6), (2, 1e-4)], ids=["fp32", "fp16"])
def test_platelet_box_ibm_matches_per_marker(gpu, prec, tol, monkeypatch):
    """Reduced precision spreads and interpolates platelet elements through a
    shared-memory node box per platelet; the per-marker kernels use the same
    nodes and weights, so only the order of float sums differs (in FP16 a
    last-bit difference can move a population by one step of the store)."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    monkeypatch.setenv("PFGPU_IBM", "boxes")
    a = gpu.Job(sc, prec)
    monkeypatch.delenv("PFGPU_IBM")
    b = gpu.Job(sc, prec)
    # five steps: the scene's Morse and bond dynamics amplify last-bit
    # differences over longer runs
    a.step(5)
    b.step(5)
    La, Lb = a.lattice(), b.lattice()
    assert rel_l2(La["u"], Lb["u"]) < tol
    assert rel_l2(La["F"], Lb["F"]) < 10 * tol
    Ea, Eb = a.elements(), b.elements()
    for k in ("X", "Y", "Z"):
        assert np.abs(Ea[k] - Eb[k]).max() < 1e-3 * tol
    assert rel_l2(Ea["V"], Eb["V"]) < 10 * tol
    np.testing.assert_array_equal(a.bonds()["rec_state"], b.bonds()["rec_state"])
    a.close()
    b.close()


@pytest.mark.parametrize("prec,tol", [(0, 1e-14), (1, 1e-6), (2, 1e-4)], ids=["fp64", "fp32", "fp16"])
def test_fast_and_generic_gather_agree(gpu, prec, tol, monkeypatch):
    """Lattices without bounce-back faces pull through 32-bit offsets without
    face tests; the generic gather reads the same populations."""
    sc = _lbm_scene("shear")
    a = gpu.Job(sc, prec)
    monkeypatch.setenv("PFGPU_GENERIC_GATHER", "1")
    b = gpu.Job(sc, prec)
    a.step(12)
    b.step(12)
    monkeypatch.delenv("PFGPU_GENERIC_GATHER")
    assert rel_max(a.lattice()["fIN"], b.lattice()["fIN"]) < tol
    assert rel_max(a.elements()["X"], b.elements()["X"]) < tol
    np.testing.assert_array_equal(a.bonds()["rec_state"], b.bonds()["rec_state"])
    a.close()
    b.close()


def test_row_staged_fp64_vs_oracle(gpu, monkeypatch):
    """FP64 row-staged kernel against the oracle on the bounce-back box."""
    sc = _lbm_scene("walls")
    monkeypatch.setenv("PFGPU_LBM_KERNEL", "rows")
    r = _run_both(gpu, sc, 15, 0)
    assert rel_max(r["Lg"]["fIN"], r["Lo"]["fIN"]) < 1e-12
    assert rel_l2(r["Lg"]["u"], r["Lo"]["u"]) < 1e-10
    for k in ("X", "Y", "Z"):
        assert np.abs(r["Eg"][k] - r["Eo"][k]).max() < 1e-12


def _stretched_membrane_scene():
    """Platelets stretched about their centroids (3, 4, 5 % along x, y, z) so
    that springs, area, volume and bending all carry force; Morse pairs,
    bonds and fibrin off, so the element force after one step is the membrane
    force at the initial positions."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(n_fib=0, n_links=0, n_rec=0)
    sc.morse = 0
    for name, s in (("X", 1.03), ("RY", 1.04), ("Z", 1.05)):
        a = np.asarray(getattr(sc, name), float).reshape(sc.n_platelets, sc.n_elem)
        c = a.mean(axis=1, keepdims=True)
        setattr(sc, name, (c + (a - c) * s).ravel())
    sc.Y = sc.RY.copy()
    return sc


def test_fp32_membrane_kernels_vs_oracle(gpu, monkeypatch):
    """FP32 membrane pass: the item-parallel kernel (default) and the
    per-vertex kernel (PFGPU_MEMBRANE_PER_VERTEX=1) against the FP64 oracle
    on stretched platelets; FP32 element forces and mean curvature within
    1e-4 relative L2, FP64-summed area and volume within 1e-6."""
    from oracle import binding as ob
    sc = _stretched_membrane_scene()
    o = ob.Oracle(sc)
    o.step(1)
    Fo, Mo = o.elements()["F"], o.membrane()
    o.close()
    assert np.linalg.norm(Fo) > 0
    got = {}
    for kern in ("items", "per_vertex"):
        if kern == "per_vertex":
            monkeypatch.setenv("PFGPU_MEMBRANE_PER_VERTEX", "1")
        j = gpu.Job(sc, 1)
        j.step(1, graph=False)
        got[kern] = (j.elements()["F"], j.membrane())
        j.close()
    monkeypatch.delenv("PFGPU_MEMBRANE_PER_VERTEX")
    for kern, (F, M) in got.items():
        assert rel_l2(F, Fo) < 1e-4, kern
        np.testing.assert_allclose(M["S_V"], Mo["S_V"], rtol=1e-6, err_msg=kern)
        assert rel_l2(M["km"], Mo["km"]) < 1e-4, kern


def test_cell_lists_bit_exact(gpu):
    from oracle import binding as ob
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    o = ob.Oracle(sc)
    o.step(10)
    j = gpu.Job(sc, 0)
    j.step(10)
    cell_g, counts_g, members_g, nc_g = j.cells()
    # the oracle's lists are those of the last Morse pass, i.e. of the positions
    # before the last position update; compare both at the same positions
    o.step(1)
    j.step(1)
    cell_o, order_o, nc_o = o.cells()
    np.testing.assert_array_equal(nc_g, nc_o)
    np.testing.assert_array_equal(cell_g, cell_o)
    np.testing.assert_array_equal(members_g, order_o)


def test_periodic_box_conserves_mass(gpu):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.plain_small(seed=4, nx=40, ny=24, nz=16, n_membrane=42, n_cyto=0, n_fib=0, n_links=0, g_lattice=0)
    sc.n_platelets = 0
    sc.bc = (0, 0, 0)
    sc.ibm_wrap = (1, 1, 0)
    rng = np.random.default_rng(0)
    N = sc.n_nodes
    sc.u_init = rng.normal(scale=0.01, size=(3, N))
    for prec, tol in ((0, 1e-13), (1, 1e-6)):
        j = gpu.Job(sc, prec)
        c0 = j.conservation()
        j.step(50)
        c1 = j.conservation()
        assert abs(c1[0] - c0[0]) / c0[0] < tol
        np.testing.assert_allclose(c1[1:], c0[1:], atol=tol * N)
        j.close()


def test_detach_stops_the_job(gpu):
    """With no bond on the platelet and a detach rate of 1 the job detaches
    at the first step whose bond count before it is zero (semLB.cu:451-455)."""
    from oracle import binding as ob
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small(n_rec=0)
    sc.detach_rate = 1.0
    o = ob.Oracle(sc)
    rc_o = o.step(5)
    j = gpu.Job(sc, 0)
    rc = j.step(5)
    assert rc == 6 and rc_o == 1
    assert j.steps == o.steps == 1
    j.close()


def test_invalid_scene_rejected_on_host(gpu):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    sc.rec_tri = sc.rec_tri.copy()
    sc.rec_tri[0, 0] = 10 ** 6
    with pytest.raises(gpu.PfgpuError) as e:
        gpu.Job(sc, 1)
    assert e.value.code == 1


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
def test_worm_like_chain_fibrin_vs_oracle(gpu, prec):
    """Fibrin links under the worm-like-chain law (fiber.cpp:710-733, pinned
    to the reference's own function in test_host_pins.py): FP64 link forces
    and positions as the oracle's; FP32 positions within the FP32 bound (its
    forces lose digits where 0.25/tl^2 - 0.25 cancels near the rest length)."""
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    sc.fib_law = 1
    sc.fib_mass = 1e-6
    r = _run_both(gpu, sc, 20, prec)
    if prec == 0:
        assert rel_l2(r["Fg"]["F"], r["Fo"]["F"]) < 1e-9
        assert np.abs(r["Fg"]["X"] - r["Fo"]["X"]).max() < 1e-12
    else:
        pos = np.stack([r["Fg"]["X"], r["Fg"]["Y"], r["Fg"]["Z"]])
        pos_o = np.stack([r["Fo"]["X"], r["Fo"]["Y"], r["Fo"]["Z"]])
        assert rel_l2(pos, pos_o) < 1e-7
    assert np.abs(r["Fo"]["F"]).max() > 0
