"""GPU parity: canonical labels from every solver option, through the C ABI,
equal the oracle's on the same seeded inputs (bit-exact; labels are integers).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import components_gb300 as cc
import oracle
from components_gb300 import _lib
from components_gb300.graph import StaticGraph

from conftest import csr_from_rows

pytestmark = pytest.mark.gpu
ALGOS = ["exp", "local", "shortcuts", "labels", "allreduce"]
GOLD = np.load(Path(__file__).with_name("golden") / "golden.npz")


def gpu_labels(G: StaticGraph, algo: str, P: int = 1, where: str = "device", conf=None,
               ctx=None):
    import torch
    conf = conf or cc.Config(seed=1001)
    G = G.with_parts(P)
    dt_t = torch.int32 if G.id_bytes == 4 else torch.int64
    dt_n = np.uint32 if G.id_bytes == 4 else np.uint64
    if where == "device":
        D = G.to_device("cuda:0")
        lab = torch.full((G.n,), -1, dtype=dt_t, device="cuda:0")
        cc.SOLVERS[algo](conf, 0, P, ctx).FindComponents(D, lab)
        return lab.cpu().numpy().view(dt_n).astype(np.uint64)
    lab = np.full(G.n, 0xFFFFFFFF, dt_n)
    cc.SOLVERS[algo](conf, 0, P, ctx).FindComponents(G, lab)
    return lab.astype(np.uint64)


def test_simple_graph_known_answer(cuda):
    G = cc.from_edges(int(GOLD["simple_n"][0]), GOLD["simple_edges"])
    for algo in ALGOS:
        for P in (1, 2, 3):
            for where in ("device", "host"):
                got = gpu_labels(G, algo, P, where, cc.Config(seed=1001, sequential_limit=0))
                assert np.array_equal(got, GOLD["simple_labels"]), (algo, P, where)


@pytest.mark.parametrize("name", ["gnm_small", "gnm_sparse", "grid_16", "grid_40x25"])
@pytest.mark.parametrize("algo", ALGOS)
def test_golden_graphs(cuda, name, algo):
    idb = int(GOLD[f"{name}_idb"][0])
    G = StaticGraph(GOLD[f"{name}_rp"], GOLD[f"{name}_col"].astype(np.uint32 if idb == 4 else np.uint64))
    for P in (1, 4, 16):
        for seq in (0, 1):
            got = gpu_labels(G, algo, P, "device", cc.Config(seed=1001, sequential_limit=seq))
            assert np.array_equal(got, GOLD[f"{name}_labels"]), (name, algo, P, seq)


@pytest.mark.parametrize("algo", ALGOS)
def test_random_graphs_all_options(cuda, algo):
    rng = np.random.default_rng(42)
    for trial in range(12):
        n = int(rng.integers(2, 3000))
        m = int(rng.integers(0, 3 * n))
        idb = 4 if trial % 2 else 8
        G = cc.gen_gnm(n, m, seed=100 + trial, id_bytes=idb)
        want = oracle.uf_labels(G)
        P = int(rng.choice([1, 2, 5, 32]))
        conf = cc.Config(seed=1001 + trial, sequential_limit=int(rng.integers(0, 3)),
                         use_contraction=bool(trial % 3 == 0), use_bfs=bool(trial % 4 == 1),
                         number_of_hitters=int(rng.choice([0, 0, 4])))
        got = gpu_labels(G, algo, P, "device" if trial % 2 else "host", conf)
        assert np.array_equal(got, want), (algo, trial, n, m, P)


def test_exp_options_and_beta(cuda):
    G = cc.gen_gnm(20000, 30000, seed=8, id_bytes=8)
    want = oracle.uf_labels(G)
    for kw in [dict(), dict(use_bfs=True), dict(single_level_contraction=True),
               dict(use_contraction=True), dict(direct_contraction=True),
               dict(replicate_high_degree=True), dict(beta=0.5), dict(beta=0.02),
               dict(fixed_limit=True, sequential_limit=100), dict(sequential_limit=0)]:
        conf = cc.Config(seed=1003, **kw)
        for P in (3, 64):
            assert np.array_equal(gpu_labels(G, "exp", P, "device", conf), want), (kw, P)


def test_ids_at_every_16_byte_offset(cuda):
    """Device ids that start 4, 8 or 12 bytes past a 16-byte boundary (a view
    into a larger tensor): the kernels that read ids 16 bytes at a time start
    at the first 16-byte boundary of the array.  Every start gives the
    oracle's labels, with virtual ranks (exp) and without (local)."""
    import torch
    G = cc.gen_rhg(1 << 15, 12.0, 2.6, seed=4)
    want = oracle.uf_labels(G)
    D = G.to_device("cuda:0")
    for shift in (0, 1, 2, 3):
        buf = torch.zeros(D.col.numel() + 4, dtype=torch.int32, device="cuda:0")
        col = buf[shift:shift + D.col.numel()]
        col.copy_(D.col)
        assert (col.data_ptr() % 16 == 0) == (shift == 0)
        for algo, P in (("exp", 4), ("exp", 16), ("local", 1)):
            lab = torch.full((G.n,), -1, dtype=torch.int32, device="cuda:0")
            cc.SOLVERS[algo](cc.Config(seed=1001, sequential_limit=0), 0, P).FindComponents(
                StaticGraph(D.row_ptr, col, P), lab)
            got = lab.cpu().numpy().view(np.uint32).astype(np.uint64)
            assert np.array_equal(got, want), (shift, algo, P)


def test_schedule_independence(cuda):
    """Randomness changes the contraction schedule, never the partition."""
    G = cc.gen_gnm(50000, 60000, seed=21, id_bytes=4)
    want = oracle.uf_labels(G)
    for seed in (1001, 1002, 1003, 5, 123456789):
        for algo in ("exp", "local"):
            got = gpu_labels(G, algo, 16, "device", cc.Config(seed=seed, sequential_limit=0))
            assert np.array_equal(got, want), (algo, seed)


def test_edge_cases(cuda):
    cases = {
        "single": csr_from_rows([[]]),
        "isolated": csr_from_rows([[], [], [], []]),
        "self_loops": csr_from_rows([[0, 1], [0, 1, 1], [2], [4], [3, 3]]),
        "multi_edges": csr_from_rows([[1, 1, 1], [0, 0, 0, 2], [1]]),
        "path": cc.from_edges(2000, [(i, i + 1) for i in range(1999)]),
        "star_hub": cc.from_edges(5000, [(17, i) for i in range(5000) if i != 17]),
        "two_hubs": cc.from_edges(3000, [(0, i) for i in range(1, 1500)]
                                  + [(2999, i) for i in range(1500, 2999)]),
        "cliques_bridge": cc.from_edges(
            60, [(a, b) for a in range(30) for b in range(a + 1, 30)]
            + [(a, b) for a in range(30, 60) for b in range(a + 1, 60)] + [(29, 30)]),
        "u64_ids": cc.from_edges(10, [(0, 9), (3, 4), (4, 8)], id_bytes=8),
    }
    for name, G in cases.items():
        want = oracle.uf_labels(G)
        for algo in ALGOS:
            for P in (1, 2, 7):
                got = gpu_labels(G, algo, P, "device", cc.Config(seed=1001, sequential_limit=0))
                assert np.array_equal(got, want), (name, algo, P)


def test_empty_graph(cuda):
    G = StaticGraph(np.zeros(1, np.uint64), np.zeros(0, np.uint32))
    for algo in ALGOS:
        lab = np.zeros(0, np.uint32)
        cc.SOLVERS[algo](cc.Config(), 0, 1).FindComponents(G, lab)


def test_invalid_ids_are_reported_not_faulted(cuda):
    """An id >= n is caught by the kernels' own bounds checks (no access is
    made) and returned as CC_ERR_INVALID; the context stays usable."""
    bad = csr_from_rows([[1], [0, 9], [3], [2]])  # 9 >= n = 4
    for algo in ALGOS:
        with pytest.raises(_lib.CCError) as ei:
            gpu_labels(bad, algo, 1, "device")
        assert ei.value.status == _lib.CC_ERR_INVALID
    good = cc.from_edges(4, [(0, 1), (2, 3)])
    assert np.array_equal(gpu_labels(good, "exp", 1), [0, 0, 2, 2])


@pytest.mark.parametrize("idb", [4, 8])
def test_id_check_at_every_offset_of_col(cuda, idb):
    """The propagation options check ids in 16-byte vectors from the first
    16-byte boundary of col on: labels are right and a bad id is reported
    wherever it sits (before that boundary, inside a vector, after the last
    whole vector), for col starting at every id offset from a boundary."""
    import torch
    G = cc.gen_gnm(300, 700, seed=5, id_bytes=idb)
    want = oracle.uf_labels(G)
    dt = torch.int32 if idb == 4 else torch.int64
    rp = torch.from_numpy(G.row_ptr.view(np.int64)).to("cuda:0")
    ids = torch.from_numpy(np.ascontiguousarray(G.col).view(np.int32 if idb == 4 else np.int64))
    for shift in range(16 // idb):
        buf = torch.zeros(G.m + 16, dtype=dt, device="cuda:0")
        col = buf[shift:shift + G.m]
        col.copy_(ids.to("cuda:0"))
        D = StaticGraph(rp, col)
        for algo in ("shortcuts", "labels", "local"):
            lab = torch.full((G.n,), -1, dtype=dt, device="cuda:0")
            cc.SOLVERS[algo](cc.Config(seed=1001), 0, 1).FindComponents(D, lab)
            got = lab.cpu().numpy().view(np.uint32 if idb == 4 else np.uint64).astype(np.uint64)
            assert np.array_equal(got, want), (shift, algo)
        for pos in (0, 1, 2, G.m // 2, G.m - 2, G.m - 1):
            old = int(col[pos].item())
            col[pos] = G.n + 7
            for algo in ("shortcuts", "labels", "local"):
                lab = torch.full((G.n,), -1, dtype=dt, device="cuda:0")
                with pytest.raises(_lib.CCError) as ei:
                    cc.SOLVERS[algo](cc.Config(seed=1001), 0, 1).FindComponents(D, lab)
                assert ei.value.status == _lib.CC_ERR_INVALID, (shift, pos, algo)
            col[pos] = old


def test_id_check_in_long_rows(cuda):
    """A bad id inside a row of more than 64 entries (walked in pieces by a
    warp each) is reported by every propagation option; the same graph with
    the id repaired gives the oracle's labels."""
    import torch
    rows = [list(range(1, 201))] + [[0] for _ in range(200)] + [[202], [201]]
    G = csr_from_rows(rows)
    want = oracle.uf_labels(G)
    D = G.to_device("cuda:0")
    for algo in ("shortcuts", "labels", "local"):
        lab = torch.full((G.n,), -1, dtype=torch.int32, device="cuda:0")
        cc.SOLVERS[algo](cc.Config(seed=1001), 0, 1).FindComponents(D, lab)
        assert np.array_equal(lab.cpu().numpy().astype(np.uint64), want), algo
    col = D.col.clone()
    col[150] = G.n + 3  # inside row 0 (200 entries)
    for algo in ("shortcuts", "labels", "local"):
        lab = torch.full((G.n,), -1, dtype=torch.int32, device="cuda:0")
        with pytest.raises(_lib.CCError) as ei:
            cc.SOLVERS[algo](cc.Config(seed=1001), 0, 1).FindComponents(StaticGraph(D.row_ptr, col), lab)
        assert ei.value.status == _lib.CC_ERR_INVALID, algo


@pytest.mark.parametrize("idb", [4, 8])
def test_component_sizes_match_numpy(cuda, idb):
    """OutputComponents on the device: (size, count) pairs in ascending size
    and the number of components with more than one vertex, for host and
    device labels; a label >= n is reported, not counted."""
    import torch
    graphs = [cc.gen_grid(300, 200, 0.5, seed=3, id_bytes=idb), cc.gen_gnm(20000, 9000, seed=4, id_bytes=idb),
              cc.from_edges(7, [], id_bytes=idb), cc.gen_rhg(1 << 14, 8.0, 2.6, seed=2, id_bytes=idb)]
    for G in graphs:
        lab = cc.find_components(G, "exp")
        sizes, counts = np.unique(np.unique(lab, return_counts=True)[1], return_counts=True)
        want = np.stack([sizes, counts], axis=1).astype(np.uint64)
        for labels in (lab, torch.from_numpy(lab.view(np.int32 if idb == 4 else np.int64)).to("cuda:0")):
            got, num = cc.component_sizes(labels)
            assert np.array_equal(got, want), G.n
            assert num == int(counts[sizes != 1].sum())
    bad = np.array([0, 1, 9], np.uint32 if idb == 4 else np.uint64)  # 9 >= n = 3
    with pytest.raises(_lib.CCError) as ei:
        cc.component_sizes(bad)
    assert ei.value.status == _lib.CC_ERR_INVALID
    assert cc.component_sizes(np.zeros(0, np.uint32))[0].shape == (0, 2)


def test_context_reuse_and_stats(cuda):
    ctx = cc.Context(0, profiling=True)
    G = cc.gen_grid(300, 200, 0.5, seed=3)
    want = oracle.uf_labels(G)
    for _ in range(3):
        assert np.array_equal(gpu_labels(G, "exp", 1, "device", ctx=ctx), want)
    st = ctx.stats()
    assert st["num_components"] == len(np.unique(want))
    assert st["kernel_launches"] > 0 and st["bytes_algorithmic"] > 0
    assert any(k.startswith("uf_") for k in st["kernels"])  # hook pass timed
    tot = ctx.profile_totals()  # the three solves above, summed
    assert tot["solves"] == 3 and tot["kernel_launches"] >= 3 * 2
    for k, v in st["kernels"].items():
        assert tot["kernels"][k]["launches"] >= v["launches"]
    arena = ctx.arena_bytes()
    gpu_labels(G, "exp", 1, "device", ctx=ctx)
    assert ctx.arena_bytes() == arena  # steady state: the pool is reused
    ctx.close()


def test_stream_interop(cuda):
    """A context on a caller's torch stream."""
    import torch
    s = torch.cuda.Stream()
    ctx = cc.Context(0, stream=s)
    G = cc.gen_gnm(5000, 5000, seed=2, id_bytes=4)
    assert np.array_equal(gpu_labels(G, "exp", 4, "device", ctx=ctx), oracle.uf_labels(G))
    ctx.close()


@pytest.mark.parametrize("mode", [_lib.CC_HOOK_GLOBAL, _lib.CC_HOOK_TILED, _lib.CC_HOOK_SAMPLED])
def test_hook_modes_agree(cuda, mode):
    """Global, tiled and sampled hook passes give the same labels, also with
    ranks, hub rows, tiles smaller than a rank and ranks smaller than a tile,
    and with link rounds run as a tiled pass (grids, the angularly ordered
    hyperbolic graph) or as global rounds (G(n, m), the star)."""
    graphs = [cc.gen_grid(700, 500, 0.5, seed=6), cc.gen_gnm(60000, 80000, seed=6, id_bytes=8),
              cc.from_edges(40000, [(5, i) for i in range(6, 40000, 3)] + [(i, i + 1) for i in range(0, 39999, 7)]),
              cc.gen_grid(64, 2000, 0.7, seed=2), cc.gen_rhg(1 << 17, 16.0, 2.6, seed=3)]
    for tile in (1024, 16384):
        ctx = cc.Context(0)
        ctx.set_tuning(hook_mode=mode, tile_vertices=tile, tile_threads=256, hub_degree=16)
        for G in graphs:
            want = oracle.uf_labels(G)
            for algo in ("allreduce", "exp"):
                for P in (1, 3, 100):
                    got = gpu_labels(G, algo, P, "device", cc.Config(seed=1001), ctx=ctx)
                    assert np.array_equal(got, want), (mode, tile, G.n, algo, P)
        ctx.close()


def test_streamed_host_input(cuda):
    """Host CSR copied in tile-aligned chunks under the tile pass (each chunk's
    cut edges united before the next chunk's tiles): same labels for pageable
    and pinned buffers (with every setting of the in-place reads, which the
    tiled pass does not take), both id widths, many chunks, with virtual
    ranks."""
    import torch
    for idb in (4, 8):
        G = cc.gen_grid(1100, 900, 0.55, seed=12, id_bytes=idb)
        want = oracle.uf_labels(G)
        for tile in (0, 1024):
            ctx = cc.Context(0)
            ctx.set_tuning(hook_mode=_lib.CC_HOOK_TILED, tile_vertices=tile, tile_threads=256)
            for algo in ("exp", "allreduce"):
                for P in (1, 3):
                    assert np.array_equal(gpu_labels(G, algo, P, "host", ctx=ctx), want), (idb, tile, algo, P)
            Pn = G.pinned()
            dt = torch.int32 if idb == 4 else torch.int64
            for mode in (1, 2, 0):  # read in place, ids in place, copied
                ctx.set_host_reads(mode)
                lab = torch.empty(G.n, dtype=dt).pin_memory()
                solver = cc.ExponentialContraction(cc.Config(seed=1001), 0, 1, ctx)
                solver.FindComponents(Pn, lab)
                got = lab.numpy().view(np.uint32 if idb == 4 else np.uint64).astype(np.uint64)
                assert np.array_equal(got, want), (idb, tile, "pinned", mode)
                h2d = solver.last_stats["h2d_bytes"]  # the tiled pass copies in every mode
                assert G.m * idb <= h2d <= 8 * (G.n + 1) + G.m * idb, (h2d, idb, tile, mode)
            ctx.close()


def test_sampled_host_input_read_in_place(cuda):
    """Host graphs solved by sampled linking from page-locked buffers are read
    in place (the offsets and each row's link entries counted as h2d bytes);
    the same labels with only the ids read in place (offsets copied in chunks),
    with in-place reads switched off (rows copied in chunks) and from pageable
    buffers, in one chunk and in two, for both id widths, with virtual ranks,
    and on a sparse graph whose largest component holds 42 % of the vertices
    (most rows read by the remaining pass)."""
    import torch
    graphs = [cc.gen_rhg(1 << 18, 16.0, 2.6, seed=4), cc.gen_rhg(1 << 18, 16.0, 2.6, seed=4, id_bytes=8),
              cc.gen_rhg(1 << 18, 2.0, 2.2, seed=5)]
    for G in graphs:
        want = oracle.uf_labels(G)
        n, idb = G.n, G.id_bytes
        dt_t, dt_n = (torch.int32, np.uint32) if idb == 4 else (torch.int64, np.uint64)
        in_place = 8 * (n + 1) + min(G.m, 2 * n) * idb  # offsets, at most two link entries a row
        for tile in (0, 1024):  # 1024: the rows cross in two chunks
            ctx = cc.Context(0)
            ctx.set_tuning(tile_vertices=tile)
            for algo, P in (("exp", 1), ("allreduce", 1), ("allreduce", 3)):
                Pn = G.with_parts(P).pinned()
                for mode in (1, 2, 0):  # in place, ids in place, copied
                    ctx.set_host_reads(mode)
                    lab = torch.full((n,), -1, dtype=dt_t).pin_memory()
                    solver = cc.SOLVERS[algo](cc.Config(seed=1001), 0, P, ctx)
                    solver.FindComponents(Pn, lab)
                    got = lab.numpy().view(dt_n).astype(np.uint64)
                    assert np.array_equal(got, want), (n, idb, tile, algo, P, mode)
                    h2d = solver.last_stats["h2d_bytes"]
                    if mode == 1:
                        assert h2d == in_place, (h2d, idb, tile, algo, P)
                    elif mode == 2:  # later chunks' offsets as degree bytes
                        assert h2d <= in_place and (tile == 0) == (h2d == in_place), (h2d, idb, tile, algo, P)
                    else:  # every id copied
                        assert h2d >= G.m * idb, (h2d, idb, tile, algo, P)
                ctx.set_host_reads(1)
                assert np.array_equal(gpu_labels(G, algo, P, "host", ctx=ctx), want), (n, idb, algo, P, "pageable")
            ctx.close()


def test_registered_host_input_read_in_place(cuda):
    """Existing host arrays registered with cudaHostRegister (what a caller
    does to its graph buffers once) are read in place like page-locked
    allocations; after unregistering, the same call copies them."""
    import torch
    cudart = torch.cuda.cudart()
    G = cc.gen_rhg(1 << 18, 16.0, 2.6, seed=7)
    want = oracle.uf_labels(G)
    rp = np.ascontiguousarray(G.row_ptr, dtype=np.uint64)
    col = np.ascontiguousarray(G.col, dtype=np.uint32)
    n = G.n
    for a in (rp, col):
        assert int(cudart.cudaHostRegister(a.ctypes.data, a.nbytes, 0)) == 0
    try:
        H = cc.StaticGraph(rp, col)
        ctx = cc.Context(0)
        lab = np.full(n, 0xFFFFFFFF, np.uint32)
        solver = cc.ExponentialContraction(cc.Config(seed=1001), 0, 1, ctx)
        solver.FindComponents(H, lab)
        assert np.array_equal(lab.astype(np.uint64), want)
        assert solver.last_stats["h2d_bytes"] == 8 * (n + 1) + min(G.m, 2 * n) * 4
    finally:
        for a in (rp, col):
            cudart.cudaHostUnregister(a.ctypes.data)
    lab = np.full(n, 0xFFFFFFFF, np.uint32)
    solver.FindComponents(H, lab)
    assert np.array_equal(lab.astype(np.uint64), want)
    assert solver.last_stats["h2d_bytes"] >= G.m * 4
    ctx.close()
