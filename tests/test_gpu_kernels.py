"""Stage-level GPU parity through the test hooks of include/cc_gpu_debug.h:
each kernel against the oracle's restatement of the same stage, bit-exact."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import components_gb300 as cc
import oracle
from components_gb300 import _lib
from components_gb300.graph import StaticGraph

pytestmark = pytest.mark.gpu
GOLD = np.load(Path(__file__).with_name("golden") / "golden.npz")


def _dev(G: StaticGraph):
    import torch
    D = G.to_device("cuda:0")
    return D, D.to_c()


def _t(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(dtype)).to("cuda:0")


def gpu_ldd(G, vid, seed, level, beta, gated=False):
    import torch
    D, g = _dev(G)
    v = _t(vid.astype(np.uint32), np.int32)
    out = torch.empty(max(G.n, 1), dtype=torch.int32, device="cuda:0")
    rounds = C.c_uint32()
    _lib.check(_lib.gpu().cc_debug_ldd(C.byref(g), v.data_ptr(), seed, level, beta, int(gated),
                                       out.data_ptr(), C.byref(rounds)))
    return out[: G.n].cpu().numpy().view(np.uint32).astype(np.uint64), rounds.value


@pytest.mark.parametrize("gated", [False, True])
def test_ldd_matches_oracle(cuda, gated):
    for seed, (n, m) in enumerate([(500, 900), (3000, 2500), (20000, 60000), (100, 40)]):
        G = cc.gen_gnm(n, m, seed=seed + 1, id_bytes=4)
        vid = np.sort(np.random.default_rng(seed).choice(10 * n, n, replace=False)).astype(np.uint64)
        for level in (1, 2, 5):
            for beta in (0.1, 0.4):
                want, _ = oracle.ldd(G, vid, 1001 + seed, level, beta)
                got, _ = gpu_ldd(G, vid, 1001 + seed, level, beta, gated)
                assert np.array_equal(got, want), (n, m, level, beta, gated)


def test_ldd_golden_vector(cuda):
    G = StaticGraph(GOLD["ldd_graph_rp"], GOLD["ldd_graph_col"].astype(np.uint32))
    got, _ = gpu_ldd(G, GOLD["ldd_vid"], 1001, 1, 0.1)
    assert np.array_equal(got, GOLD["ldd_cluster"])


def test_ldd_on_grid_and_hub(cuda):
    G = cc.gen_grid(200, 150, 0.6, seed=2)
    vid = np.arange(G.n, dtype=np.uint64)
    for gated in (False, True):
        want, _ = oracle.ldd(G, vid, 7, 1, 0.1)
        got, _ = gpu_ldd(G, vid, 7, 1, 0.1, gated)
        assert np.array_equal(got, want)
    H = cc.from_edges(4000, [(3, i) for i in range(4000) if i != 3] + [(10, 11), (11, 12)])
    vid = np.arange(H.n, dtype=np.uint64)
    want, _ = oracle.ldd(H, vid, 9, 1, 0.1)
    got, _ = gpu_ldd(H, vid, 9, 1, 0.1)
    assert np.array_equal(got, want)


def test_local_sweeps_match_oracle(cuda):
    import torch
    hubs = cc.from_edges(9000, [(h, i) for h in (4, 700, 8000) for i in range(0, 9000, 1 + h % 3)
                                if i != h] + [(1, 2), (2, 3)])  # rows of 3000-9000 entries: pieces
    for seed, G in enumerate([cc.gen_gnm(500, 900, seed=3, id_bytes=4),
                              cc.gen_gnm(5000, 20000, seed=4, id_bytes=4), hubs]):
        n = G.n
        vid = np.arange(n, dtype=np.uint64) * 2 + 5
        D, g = _dev(G)
        v = _t(vid.astype(np.uint32), np.int32)
        out = torch.empty(n, dtype=torch.int32, device="cuda:0")
        _lib.check(_lib.gpu().cc_debug_local_sweeps(C.byref(g), v.data_ptr(), 77, 2, out.data_ptr()))
        got = out.cpu().numpy().view(np.uint32).astype(np.uint64)
        assert np.array_equal(got, oracle.local_sweeps(G, vid, 77, 2))
    G = StaticGraph(GOLD["ldd_graph_rp"], GOLD["ldd_graph_col"].astype(np.uint32))
    D, g = _dev(G)
    v = _t(GOLD["ldd_vid"].astype(np.uint32), np.int32)
    out = torch.empty(G.n, dtype=torch.int32, device="cuda:0")
    _lib.check(_lib.gpu().cc_debug_local_sweeps(C.byref(g), v.data_ptr(), 1001, 2, out.data_ptr()))
    assert np.array_equal(out.cpu().numpy().view(np.uint32), GOLD["sweeps_cluster"].astype(np.uint32))


def gpu_contract(G, cl, ncl, vid_of_cluster=None, cut_parts=0):
    import torch
    D, g = _dev(G)
    clt = _t(cl.astype(np.uint32), np.int32)
    vt = _t(vid_of_cluster.astype(np.uint32), np.int32) if vid_of_cluster is not None else None
    rp = torch.zeros(ncl + 1, dtype=torch.int64, device="cuda:0")
    col = torch.zeros(max(G.m, 1), dtype=torch.int32, device="cuda:0")
    vid = torch.zeros(max(ncl, 1), dtype=torch.int32, device="cuda:0")
    newid = torch.zeros(max(ncl, 1), dtype=torch.int32, device="cuda:0")
    nn, mm = C.c_uint64(), C.c_uint64()
    _lib.check(_lib.gpu().cc_debug_contract(C.byref(g), clt.data_ptr(), ncl,
                                            vt.data_ptr() if vt is not None else None, cut_parts,
                                            rp.data_ptr(), col.data_ptr(), vid.data_ptr(),
                                            newid.data_ptr(), C.byref(nn), C.byref(mm)))
    k, m = nn.value, mm.value
    return (rp[: k + 1].cpu().numpy().view(np.uint64), col[:m].cpu().numpy().view(np.uint32),
            vid[:k].cpu().numpy().view(np.uint32), newid[:ncl].cpu().numpy().view(np.uint32))


def test_contraction_matches_oracle(cuda):
    for seed, (n, m) in enumerate([(1000, 3000), (30000, 90000), (7, 0)]):
        G = cc.gen_gnm(n, m, seed=seed + 5, id_bytes=4) if m else cc.from_edges(n, [])
        cl = np.random.default_rng(seed).integers(0, max(n // 3, 1), n).astype(np.uint64)
        ncl = max(n // 3, 1)
        rp_w, col_w, vid_w, newid_w = oracle.contract(G, cl, ncl)
        rp_g, col_g, vid_g, newid_g = gpu_contract(G, cl, ncl)
        assert np.array_equal(rp_g, rp_w)
        assert np.array_equal(col_g.astype(np.uint64), col_w)
        assert np.array_equal(vid_g.astype(np.uint64), vid_w)
        nw = np.where(newid_w == np.uint64(2**64 - 1), np.uint64(0xFFFFFFFF), newid_w)
        assert np.array_equal(newid_g.astype(np.uint64), nw)


def test_contraction_with_repeated_keys_matches_oracle(cuda):
    """Few clusters: almost every cut key repeats, so the emit kernels' set of
    written keys drops most of them before the sort (a hub row of 6000
    entries takes the piece-per-warp kernel); the quotient graph is the
    oracle's."""
    rng = np.random.default_rng(11)
    n = 20000
    e = rng.integers(0, n, size=(200000, 2))
    hub = np.stack([np.zeros(6000, np.int64), np.arange(1, 6001)], axis=1)
    G = cc.from_edges(n, np.concatenate([e, hub]))
    for ncl in (2, 3, 40):
        cl = rng.integers(0, ncl, n).astype(np.uint64)
        rp_w, col_w, vid_w, newid_w = oracle.contract(G, cl, ncl)
        rp_g, col_g, vid_g, newid_g = gpu_contract(G, cl, ncl)
        assert np.array_equal(rp_g, rp_w), ncl
        assert np.array_equal(col_g.astype(np.uint64), col_w), ncl
        assert np.array_equal(vid_g.astype(np.uint64), vid_w), ncl


def test_cut_graph_matches_oracle(cuda):
    """Component graph of the cut edges: local components then cut edges."""
    import torch
    for P in (2, 9):
        for idb in (4, 8):
            G = cc.gen_gnm(8000, 9000, seed=P, id_bytes=idb, num_parts=P)
            D, g = _dev(G)
            lab = torch.empty(G.n, dtype=torch.int32, device="cuda:0")
            _lib.check(_lib.gpu().cc_debug_local_components(C.byref(g), lab.data_ptr()))
            got_lab = lab.cpu().numpy().view(np.uint32).astype(np.uint64)
            want_lab = oracle.local_components(G, P)
            assert np.array_equal(got_lab, want_lab)
            rp_w, col_w, vid_w, _ = oracle.contract(G, want_lab, G.n, cut_parts=P)
            rp_g, col_g, vid_g, _ = gpu_contract(G, want_lab, G.n, None, cut_parts=P)
            assert np.array_equal(rp_g, rp_w) and np.array_equal(col_g.astype(np.uint64), col_w)
            assert np.array_equal(vid_g.astype(np.uint64), vid_w)


def test_radix_sort(cuda):
    import torch
    rng = np.random.default_rng(3)
    for n, bits in [(1, 8), (4095, 20), (4096, 40), (100003, 64), (1 << 20, 44)]:
        keys = rng.integers(0, 2**63, n, dtype=np.uint64) & np.uint64((1 << bits) - 1 if bits < 64 else 2**64 - 1)
        t = torch.from_numpy(keys.view(np.int64)).to("cuda:0")
        _lib.check(_lib.gpu().cc_debug_radix_sort(t.data_ptr(), n, bits))
        assert np.array_equal(t.cpu().numpy().view(np.uint64), np.sort(keys))


def test_shortcut_rounds_match_oracle(cuda):
    """Same Jacobi rounds as the restatement: same labels, same round count."""
    import torch
    for hitters in (0, 3):
        for seed, (n, m) in enumerate([(2000, 2200), (10000, 30000)]):
            G = cc.gen_gnm(n, m, seed=seed + 9, id_bytes=4)
            init = np.random.default_rng(seed).permutation(n).astype(np.uint64)
            want, rounds_w = oracle.shortcut(G, init, hitters)
            D, g = _dev(G)
            lab = _t(init.astype(np.uint32), np.int32)
            r = C.c_uint32()
            _lib.check(_lib.gpu().cc_debug_shortcut(C.byref(g), lab.data_ptr(), hitters, C.byref(r)))
            assert np.array_equal(lab.cpu().numpy().view(np.uint32).astype(np.uint64), want)
            assert r.value == rounds_w


def test_device_generators_equal_host_generators(cuda):
    """cc_gen_grid_device / cc_gen_gnm_device build the very graphs of the host
    generators (same hash, same sorted rows), for both id widths."""
    for idb in (4, 8):
        for X, Y, p, seed in [(300, 200, 0.5, 1), (1, 50, 0.7, 2), (64, 1, 1.0, 3), (40, 30, 0.0, 4),
                              (513, 129, 0.35, 9)]:
            H = cc.gen_grid(X, Y, p, seed=seed, id_bytes=idb)
            D = cc.gen_grid_device(X, Y, p, seed=seed, id_bytes=idb)
            rp, col = D.numpy()
            assert np.array_equal(rp, np.asarray(H.row_ptr, np.uint64)), (X, Y, p, idb)
            assert np.array_equal(col, np.asarray(H.col).astype(np.uint64)), (X, Y, p, idb)
        for n, m, seed in [(1 << 12, 3 << 12, 5), (1000, 4000, 6), (1, 3, 7), (17, 400, 8), (5000, 0, 9)]:
            H = cc.gen_gnm(n, m, seed=seed, id_bytes=idb)
            D = cc.gen_gnm_device(n, m, seed=seed, id_bytes=idb)
            rp, col = D.numpy()
            assert np.array_equal(rp, np.asarray(H.row_ptr, np.uint64)), (n, m, idb)
            assert np.array_equal(col, np.asarray(H.col).astype(np.uint64)), (n, m, idb)
    G = cc.gen_grid_device(700, 500, 0.5, seed=6)
    lab = cc.find_components(G, "exp")
    assert np.array_equal(lab.cpu().numpy().view(np.uint32).astype(np.uint64), oracle.uf_labels(G))


@pytest.mark.parametrize("n,d,gamma,seed,idb", [(1 << 12, 16.0, 2.6, 1, 4), (3000, 4.0, 2.2, 2, 8),
                                               (1 << 16, 8.0, 3.0, 5, 4), (1 << 20, 16.0, 2.6, 1, 4),
                                               (100, 32.0, 2.4, 9, 4)])
def test_device_rhg_equals_host_rhg(cuda, n, d, gamma, seed, idb):
    """cc_gen_rhg_device builds the host generator's hyperbolic graph bit for
    bit: the model's values and edge test are correctly rounded operations on
    both sides."""
    H = cc.gen_rhg(n, d, gamma, seed=seed, id_bytes=idb)
    D = cc.gen_rhg_device(n, d, gamma, seed=seed, id_bytes=idb)
    rp, col = D.numpy()
    assert np.array_equal(rp, np.asarray(H.row_ptr, np.uint64))
    assert np.array_equal(col, np.asarray(H.col).astype(np.uint64))
