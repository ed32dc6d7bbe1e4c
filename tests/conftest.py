import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


_ORACLE_RUNS = {}


def oracle_state(scene, nsteps: int, key=None):
    """The CPU oracle's state of `scene` after `nsteps` coupled steps
    (lattice, elements, bonds, fibrin), cached per (key, nsteps) so several
    GPU runs of one scene are checked against one oracle run."""
    import os

    from oracle import binding as ob
    k = (key if key is not None else id(scene), nsteps)
    if k not in _ORACLE_RUNS:
        ob.set_threads(os.cpu_count() or 1)
        o = ob.Oracle(scene)
        o.step(nsteps)
        L = o.lattice()
        st = dict(u=L["u"], rho=L["rho"], E=o.elements() if scene.n_platelets else None,
                  B=o.bonds() if scene.n_platelets else None, Fb=o.fibrin() if scene.n_fib else None,
                  steps=nsteps)
        o.close()
        _ORACLE_RUNS[k] = st
    return _ORACLE_RUNS[k]


# velocity tolerance (relative L2 against the FP64 oracle) by precision
ORACLE_U_TOL = {0: 1e-10, 1: 2e-5, 2: 1e-3}


def assert_matches_oracle(job, ref, precision: int, pos_tol: float = 1e-7):
    """A GPU job's state against an oracle_state(): velocity within the
    precision's relative L2 tolerance, element and fibrin positions within
    `pos_tol` relative L2, receptor bond states and vWF slot tables bit for
    bit."""
    import numpy as np

    def rl2(a, b):
        return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))

    assert job.steps == ref["steps"]
    L = job.lattice()
    assert rl2(L["u"], ref["u"]) < ORACLE_U_TOL[precision], rl2(L["u"], ref["u"])
    if ref["E"] is not None:
        E = job.elements()
        pos = np.stack([E["X"], E["Y"], E["Z"]])
        pos_o = np.stack([ref["E"]["X"], ref["E"]["Y"], ref["E"]["Z"]])
        assert rl2(pos, pos_o) < pos_tol, rl2(pos, pos_o)
        B = job.bonds()
        np.testing.assert_array_equal(B["rec_state"], ref["B"]["rec_state"])
        np.testing.assert_array_equal(B["vwf"], ref["B"]["vwf"])
    if ref["Fb"] is not None:
        assert rl2(job.fibrin()["X"], ref["Fb"]["X"]) < pos_tol
