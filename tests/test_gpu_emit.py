"""GPU parity of the component-graph emit with virtual ranks on 32-bit ids:
the rank-local row groups stream their entries with 16-byte loads, a vector
that would reach past the id array is read entry by entry, and rows above the
hub limit (4096 entries with ranks) go to warp pieces.  Labels of the
exp_contraction and local_contraction options (with the component graph) are
compared with the oracle's union-find, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import components_gb300 as cc
import oracle

from test_gpu_parity import gpu_labels

pytestmark = pytest.mark.gpu


def _with_tail(G, k):
    """G plus k extra undirected edges, so that the directed entry count
    changes by 2k: a symmetric CSR has an even count, and k = 0, 1 give both
    of its residues modulo 4 (with 2, the last 16-byte vector of the id array
    holds two entries and two slots past its end)."""
    rp, col = G.numpy()
    n = G.n
    edges = [(int(v), int(u)) for v in range(n) for u in col[rp[v]:rp[v + 1]] if u > v]
    for j in range(k):
        edges.append((j, n - 1 - j))
    return cc.from_edges(n, edges, id_bytes=4)


@pytest.mark.parametrize("P", [2, 3, 7, 16])
def test_emit_rank_streams_match_oracle(cuda, P):
    base = cc.gen_rhg(1 << 13, 12.0, 2.6, seed=40 + P, id_bytes=4)
    for k in range(2):
        G = _with_tail(base, k) if k else base
        assert G.m % 4 in (0, 2)
        want = oracle.uf_labels(G)
        for algo in ("exp", "local"):
            for seq in (0, 1):
                conf = cc.Config(seed=1001, sequential_limit=seq, use_contraction=True)
                got = gpu_labels(G, algo, P, "device", conf)
                assert np.array_equal(got, want), (P, k, G.m % 4, algo, seq)


def test_emit_hub_rows_above_the_rank_limit(cuda):
    # a hub of 5000 neighbours spread over every rank, plus a path through the
    # other vertices: rows above 4096 entries take the piece path
    n = 6000
    edges = [(0, v) for v in range(1, 5001)] + [(v, v + 1) for v in range(5001, n - 1)]
    edges += [(4999, 5001), (17, 5999)]
    G = cc.from_edges(n, edges, id_bytes=4)
    want = oracle.uf_labels(G)
    for P in (2, 5, 16):
        for algo in ("exp", "local"):
            got = gpu_labels(G, algo, P, "device", cc.Config(seed=7, use_contraction=True))
            assert np.array_equal(got, want), (P, algo)
