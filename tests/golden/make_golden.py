"""Regenerate tests/golden/golden.npz.

    python tests/golden/make_golden.py

Contents (all small):
  simple_*      the reference's only fixture, example/simple.graph (6 vertices,
                edges 1-3, 2-3, 4-5, 4-6 in its 1-based METIS numbering),
                restated as a 0-based edge list, and its canonical labels
                [0,0,0,3,3,3] derived by hand
  <case>_rp/_col/_labels  CSRs from the seeded generators with their canonical
                labels from the oracle's union-find; they pin the generators
                and the labels across hosts
  geo_beta0.1   the deviate threshold table for beta = 0.1
  hash3         SplitMix64-based hash values for fixed arguments
  ldd_*, sweeps_*  cluster maps of one exponential-shift decomposition and one
                pair of local-contraction sweeps on a fixed graph
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import components_gb300 as cc  # noqa: E402
import oracle  # noqa: E402

CASES = {
    "gnm_small": lambda: cc.gen_gnm(300, 400, seed=3, id_bytes=8),
    "gnm_sparse": lambda: cc.gen_gnm(1000, 600, seed=5, id_bytes=4),
    "grid_16": lambda: cc.gen_grid(16, 16, 0.5, seed=1, id_bytes=4),
    "grid_40x25": lambda: cc.gen_grid(40, 25, 0.55, seed=9, id_bytes=4),
}


def main() -> None:
    out: dict[str, np.ndarray] = {}
    simple_edges = np.array([[0, 2], [1, 2], [3, 4], [3, 5]], np.uint64)
    out["simple_n"] = np.array([6], np.uint64)
    out["simple_edges"] = simple_edges
    out["simple_labels"] = np.array([0, 0, 0, 3, 3, 3], np.uint64)
    for name, mk in CASES.items():
        G = mk()
        rp, col = G.numpy()
        out[f"{name}_rp"] = rp
        out[f"{name}_col"] = col
        out[f"{name}_idb"] = np.array([G.id_bytes], np.uint64)
        out[f"{name}_labels"] = oracle.uf_labels(G)
    out["geo_beta0.1"] = oracle.geo_table(0.1)
    args = [(1, 0, 0), (1001, 12345, 1), (7, 2**32 + 5, 3), (2**63, 99, 64)]
    out["hash3_args"] = np.array(args, np.uint64)
    out["hash3"] = np.array([oracle.hash3(*a) for a in args], np.uint64)
    # one decomposition stage on a fixed graph (vertex order = label order)
    G = cc.gen_gnm(500, 900, seed=11, id_bytes=4)
    vid = np.arange(G.n, dtype=np.uint64) * 3 + 1
    cl, _ = oracle.ldd(G, vid, seed=1001, level=1, beta=0.1)
    out["ldd_graph_rp"], out["ldd_graph_col"] = G.numpy()
    out["ldd_vid"] = vid
    out["ldd_cluster"] = cl
    out["sweeps_cluster"] = oracle.local_sweeps(G, vid, seed=1001, level=2)
    np.savez_compressed(Path(__file__).with_name("golden.npz"), **out)
    print("wrote", Path(__file__).with_name("golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
