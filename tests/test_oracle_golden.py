"""The CPU oracle against golden vectors produced by the reference's own
kernel sources (tests/golden/make_golden.py)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import binding as ob
from platelet_fiber_gpu_gb300.scene import scene_from_dict

GOLDEN = Path(__file__).parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("ref_*.npz"))


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("brute", [True, False], ids=["node-centric", "stencil"])
def test_oracle_matches_reference(name, brute):
    d = np.load(GOLDEN / f"{name}.npz")
    sc = scene_from_dict(d)
    o = ob.Oracle(sc, brute=brute)
    o.step(int(d["nsteps"]))
    L, E, B = o.lattice(), o.elements(), o.bonds()
    tol = 1e-13
    assert _rel(L["fIN"], d["out.fIN"]) < tol
    assert _rel(L["rho"], d["out.rho"]) < tol
    for k, a in enumerate("xyz"):
        assert _rel(L["u"][k], d[f"out.u{a}"]) < 1e-12
        assert _rel(L["F"][k], d[f"out.F{a}"]) < 1e-12
        assert _rel(E["V"][k], d[f"out.V{a.upper()}"]) < 1e-12
        assert _rel(E["F"][k], d[f"out.F{a.upper()}"]) < 1e-12
    for k in ("X", "Y", "RY", "Z"):
        assert _rel(E[k], d[f"out.{k}"]) < 1e-14
    # bond states and wall slots are integer state: bit-exact
    np.testing.assert_array_equal(B["rec_state"], d["out.rec_state"])
    np.testing.assert_array_equal(B["vwf"], d["out.vwf"])
    assert B["total"] == int(d["out.total_bond"][-1])
    M = o.membrane()
    np.testing.assert_allclose(M["S_V"][0], d["out.S_V"][-1], rtol=1e-14)


@pytest.mark.parametrize("name", CASES)
def test_bond_count_history(name):
    d = np.load(GOLDEN / f"{name}.npz")
    sc = scene_from_dict(d)
    o = ob.Oracle(sc)
    hist = []
    for _ in range(int(d["nsteps"])):
        o.step(1)
        hist.append(o.bonds()["total"])
    np.testing.assert_array_equal(hist, d["out.total_bond"])
    assert max(hist) > 0, "golden case must exercise binding"


@pytest.mark.parametrize("name", CASES)
def test_trajectory_every_step(name):
    d = np.load(GOLDEN / f"{name}.npz")
    sc = scene_from_dict(d)
    o = ob.Oracle(sc)
    traj = d["out.traj"]
    for t in range(traj.shape[0]):
        o.step(1)
        E = o.elements()
        np.testing.assert_allclose(E["X"], traj[t, 0], rtol=0, atol=1e-13)
        np.testing.assert_allclose(E["Y"], traj[t, 1], rtol=0, atol=1e-13)
        np.testing.assert_allclose(E["Z"], traj[t, 2], rtol=0, atol=1e-13)
