"""Mesh preprocessing (restating gpuSEM_LB.c:846-1055) and workload builders."""
import numpy as np

from platelet_fiber_gpu_gb300 import mesh as M
from platelet_fiber_gpu_gb300 import workloads as W


def test_icosphere_topology_invariants():
    v, t = M.ellipsoid_icosphere(1)
    topo = M.build_topology(t, len(v), v)
    T = len(t)
    n_edges = 3 * T // 2
    assert topo.newnode == len(v) + n_edges
    # every midpoint node is shared by exactly two triangles, every vertex by its valence
    assert np.all(topo.node_ntri[len(v):] == 2)
    assert topo.node_ntri[:len(v)].sum() == 3 * T
    # rings close: consecutive ring vertices are mesh neighbours
    edges = {(min(a, b), max(a, b)) for a, b, c in t for a, b in ((a, b), (b, c), (c, a))}
    for i in range(len(v)):
        r = topo.ring[i, :topo.node_ntri[i]]
        assert len(set(r.tolist())) == len(r)
        for a, b in zip(r, np.roll(r, -1)):
            assert (min(a, b), max(a, b)) in edges


def test_rest_area_volume_of_ellipsoid():
    v, t = M.ellipsoid_fibonacci(400, (1.0, 1.0, 0.5), seed=3)
    S0, S_all, V0 = M.rest_area_volume(t, v + np.array([8.0, 1.5, 0.32]))
    assert np.all(S0 > 0)
    # true ellipsoid: V = 4/3 pi abc, polyhedral approximation slightly smaller
    assert 0.97 * 4 / 3 * np.pi * 0.5 < V0 < 4 / 3 * np.pi * 0.5
    assert 8.0 < S_all < 8.7


def test_springs_csr_sorted_and_symmetric():
    v, t = M.ellipsoid_icosphere(1)
    ptr, nbr, L0 = M.edge_rest_lengths(v, t, len(v) + 5)
    dense = M.dense_bond_lengths(ptr, nbr, L0, len(v) + 5)
    np.testing.assert_array_equal(dense, dense.T)
    for e in range(len(v)):
        assert np.all(np.diff(nbr[ptr[e]:ptr[e + 1]]) > 0)
    assert ptr[-1] == ptr[len(v)]  # cytoplasm elements carry no springs


def test_workloads_build():
    sc = W.mixed_small()
    assert sc.n_platelets == 3 and sc.n_fib == 300 and sc.n_rec == 40
    assert sc.fib_ptr[-1] == 2 * 600
    sc = W.plain_small(n_fib=50, n_links=100)
    assert sc.n_elem == 600 and sc.n_membrane == 400 and sc.n_tri == 2 * 400 - 4
