"""CPU tests: the oracle against the golden vectors and against its own
independent union-find; the generators against their committed outputs."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import components_gb300 as cc
import oracle
from components_gb300.graph import StaticGraph

GOLD = np.load(Path(__file__).with_name("golden") / "golden.npz")
ALGOS = ["exp", "local", "shortcuts", "labels", "allreduce"]


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    return built


def _golden_graph(name):
    idb = int(GOLD[f"{name}_idb"][0])
    col = GOLD[f"{name}_col"].astype(np.uint32 if idb == 4 else np.uint64)
    return StaticGraph(GOLD[f"{name}_rp"].astype(np.uint64), col)


def test_simple_graph_known_answer():
    """example/simple.graph: components {1,2,3} and {4,5,6} -> [0,0,0,3,3,3]."""
    G = cc.from_edges(int(GOLD["simple_n"][0]), GOLD["simple_edges"])
    want = GOLD["simple_labels"]
    assert np.array_equal(oracle.uf_labels(G), want)
    for algo in ALGOS:
        for P in (1, 2, 3):
            assert np.array_equal(oracle.solve(G, algo, P=P, seq=0), want), (algo, P)


@pytest.mark.parametrize("name", ["gnm_small", "gnm_sparse", "grid_16", "grid_40x25"])
def test_generators_reproduce_golden(name):
    mk = {
        "gnm_small": lambda: cc.gen_gnm(300, 400, seed=3, id_bytes=8),
        "gnm_sparse": lambda: cc.gen_gnm(1000, 600, seed=5, id_bytes=4),
        "grid_16": lambda: cc.gen_grid(16, 16, 0.5, seed=1, id_bytes=4),
        "grid_40x25": lambda: cc.gen_grid(40, 25, 0.55, seed=9, id_bytes=4),
    }[name]
    G = mk()
    rp, col = G.numpy()
    assert np.array_equal(rp, GOLD[f"{name}_rp"])
    assert np.array_equal(col, GOLD[f"{name}_col"])


@pytest.mark.parametrize("name", ["gnm_small", "gnm_sparse", "grid_16", "grid_40x25"])
@pytest.mark.parametrize("algo", ALGOS)
def test_oracle_solvers_match_golden(name, algo):
    G = _golden_graph(name)
    want = GOLD[f"{name}_labels"]
    for P in (1, 4):
        got = oracle.solve(G, algo, P=P, seq=0, seed=1001)
        assert np.array_equal(got, want), (name, algo, P)


def test_variates_pinned():
    assert np.array_equal(oracle.geo_table(0.1), GOLD["geo_beta0.1"])
    for a, h in zip(GOLD["hash3_args"], GOLD["hash3"]):
        assert oracle.hash3(int(a[0]), int(a[1]), int(a[2])) == int(h)


def test_stage_vectors_pinned():
    G = StaticGraph(GOLD["ldd_graph_rp"], GOLD["ldd_graph_col"].astype(np.uint32))
    cl, _ = oracle.ldd(G, GOLD["ldd_vid"], seed=1001, level=1, beta=0.1)
    assert np.array_equal(cl, GOLD["ldd_cluster"])
    sw = oracle.local_sweeps(G, GOLD["ldd_vid"], seed=1001, level=2)
    assert np.array_equal(sw, GOLD["sweeps_cluster"])


def test_geo_table_is_floor_exp():
    """T[k-1] = floor(2^64 exp(-beta k)) within one double rounding."""
    for beta in (0.1, 0.5, 1.0, 0.02):
        t = oracle.geo_table(beta)
        k = np.arange(1, len(t) + 1, dtype=np.float64)
        ref = np.ldexp(np.exp(-beta * k), 64)
        err = np.abs(t.astype(np.float64) - ref)
        assert np.all(err <= np.maximum(1e-12 * ref, 1.0))  # floor() costs < 1
        assert np.all(np.diff(t.astype(np.float64)) <= 0)


def test_deviates_are_geometric():
    """P(dev >= k) = exp(-beta k): the sampler's empirical tail."""
    beta = 0.1
    t = oracle.geo_table(beta)
    u = np.array([oracle.hash3(1001, i, 1) for i in range(20000)], np.uint64)
    dev = (u[:, None] < t[None, :40]).sum(axis=1)
    for k in (1, 5, 10, 20):
        emp = (dev >= k).mean()
        assert abs(emp - np.exp(-beta * k)) < 0.02, (k, emp)


def test_schedule_independence_oracle():
    G = cc.gen_gnm(2000, 2600, seed=4, id_bytes=8)
    want = oracle.uf_labels(G)
    for seed in (1001, 1002, 1003, 77):
        for P in (2, 5):
            assert np.array_equal(oracle.solve(G, "exp", P=P, seq=0, seed=seed), want)
            assert np.array_equal(oracle.solve(G, "local", P=P, seq=1, seed=seed), want)


def test_oracle_random_graphs():
    rng = np.random.default_rng(0)
    for trial in range(40):
        n = int(rng.integers(1, 400))
        m = int(rng.integers(0, 3 * n))
        G = cc.gen_gnm(n, m, seed=trial, id_bytes=8)
        want = oracle.uf_labels(G)
        for P in (1, 3, 8):
            for algo in ALGOS:
                got = oracle.solve(G, algo, P=P, seq=int(rng.integers(0, 3)), seed=trial)
                assert np.array_equal(got, want), (trial, P, algo)


def test_oracle_edge_cases():
    cases = {
        "empty": cc.from_edges(0, []),
        "single": cc.from_edges(1, []),
        "isolated": cc.from_edges(5, []),
        "path": cc.from_edges(50, [(i, i + 1) for i in range(49)]),
        "star": cc.from_edges(300, [(7, i) for i in range(300) if i != 7]),
        "two_cliques_bridge": cc.from_edges(
            12, [(a, b) for a in range(6) for b in range(a + 1, 6)]
            + [(a, b) for a in range(6, 12) for b in range(a + 1, 12)] + [(5, 6)]),
    }
    for name, G in cases.items():
        want = np.arange(G.n, dtype=np.uint64) if G.m == 0 else oracle.uf_labels(G)
        for algo in ALGOS:
            for P in (1, 2, 4):
                got = oracle.solve(G, algo, P=P, seq=0)
                assert np.array_equal(got, want), (name, algo, P)


def test_local_components_restrict_to_ranks():
    G = cc.from_edges(6, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5)])
    # P=2: ranks {0,1,2} and {3,4,5}; the edge 2-3 is a cut edge
    assert list(oracle.local_components(G, 2)) == [0, 0, 0, 3, 3, 3]
    assert list(oracle.local_components(G, 3)) == [0, 0, 2, 2, 4, 4]
