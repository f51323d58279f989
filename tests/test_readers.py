"""The input-file readers of libccgen (METIS text, sorted edge file, sorted
binary file; the reference's GraphIO formats) against from_edges on the same
edges, and their error reports.  Host code: no GPU."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import components_gb300 as cc
from components_gb300 import _lib

GOLD = np.load(Path(__file__).with_name("golden") / "golden.npz")


def same_csr(a, b):
    ra, ca = a.numpy()
    rb, cb = b.numpy()
    return np.array_equal(ra, rb) and np.array_equal(ca, cb)


def write_metis(path, n, edges, header_m=None, comment=True):
    adj = [[] for _ in range(n)]
    for u, w in edges:
        adj[u].append(w)
        adj[w].append(u)
    lines = (["% restated test input"] if comment else []) + [f"{n} {header_m if header_m is not None else len(edges)}"]
    lines += [" ".join(str(w + 1) for w in row) for row in adj]
    Path(path).write_text("\n".join(lines) + "\n")


def test_metis_fixture(tmp_path):
    n, edges = int(GOLD["simple_n"][0]), [tuple(map(int, e)) for e in GOLD["simple_edges"]]
    p = tmp_path / "simple.graph"
    write_metis(p, n, edges, header_m=len(edges) + 1)  # the fixture's header overstates m
    G = cc.read_metis(str(p))
    assert same_csr(G, cc.from_edges(n, edges))


@pytest.mark.parametrize("idb", [4, 8])
def test_readers_match_from_edges(tmp_path, idb):
    rng = np.random.default_rng(3)
    n = 700
    e = rng.integers(0, n, size=(2000, 2))
    edges = [(int(u), int(w)) for u, w in e]  # self-loops and repeats included: dropped by all
    want = cc.from_edges(n, edges, id_bytes=idb)
    pm = tmp_path / "g.metis"
    write_metis(pm, n, [(u, w) for u, w in edges if u != w])
    assert same_csr(cc.read_metis(str(pm), id_bytes=idb), want)
    pe = tmp_path / "g.edges"
    pe.write_text(f"% comment\np {n} {len(edges)}\n" + "".join(f"e {u + 1} {w + 1}\n" for u, w in edges)
                  + "c ignored record\n")
    assert same_csr(cc.read_edge_list(str(pe), id_bytes=idb), want)
    pb = tmp_path / "g.bin"
    pb.write_bytes(np.array([n, len(edges)], np.uint64).tobytes()
                   + (np.array(edges, np.uint64) + 1).tobytes())
    assert same_csr(cc.read_binary_edges(str(pb), id_bytes=idb), want)


def test_reader_errors(tmp_path):
    bad = [("m0", "3 1\n0\n\n\n", cc.read_metis), ("mbig", "3 1\n4\n\n\n", cc.read_metis),
           ("e0", "p 3 1\ne 0 1\n", cc.read_edge_list), ("nohdr", "% only\n", cc.read_edge_list)]
    for name, text, fn in bad:
        p = tmp_path / name
        p.write_text(text)
        with pytest.raises(_lib.CCError) as ei:
            fn(str(p))
        assert ei.value.status == _lib.CC_ERR_INVALID, name
    p = tmp_path / "short.bin"
    p.write_bytes(np.array([3, 5], np.uint64).tobytes() + np.array([1, 2], np.uint64).tobytes())
    with pytest.raises(_lib.CCError):
        cc.read_binary_edges(str(p))
    with pytest.raises(_lib.CCError):
        cc.read_metis(str(tmp_path / "missing.graph"))


def test_metis_line_endings_and_whitespace(tmp_path):
    """CRLF line ends, tabs, trailing spaces, comment lines between vertex
    lines and a missing last line (an isolated vertex) read as the same graph."""
    n, edges = 5, [(0, 1), (1, 2), (3, 4)]
    text = "% c\r\n5 3\r\n2 \r\n1\t3\r\n% between\r\n2\r\n5\r\n4\r\n"
    p = tmp_path / "crlf.graph"
    p.write_bytes(text.encode())
    assert same_csr(cc.read_metis(str(p)), cc.from_edges(n, edges))
    q = tmp_path / "short.graph"
    q.write_text("4 1\n2\n1\n")  # vertices 2 and 3 have no line: isolated
    assert same_csr(cc.read_metis(str(q)), cc.from_edges(4, [(0, 1)]))


def test_load_graph_dispatches_like_the_drivers(tmp_path):
    """-input file|edgefile|binary -in <path> and -gen gnm_undirected|grid_2d|rhg
    through the parsed Config, as IOUtility::LoadGraph dispatches."""
    n, edges = 6, [(0, 1), (1, 2), (3, 4), (4, 5)]
    want = cc.from_edges(n, edges)
    pm = tmp_path / "g.graph"
    write_metis(pm, n, edges)
    pe = tmp_path / "g.edges"
    pe.write_text(f"p {n} {len(edges)}\n" + "".join(f"e {u + 1} {w + 1}\n" for u, w in edges))
    pb = tmp_path / "g.bin"
    pb.write_bytes(np.array([n, len(edges)], np.uint64).tobytes() + (np.array(edges, np.uint64) + 1).tobytes())
    for kind, path in (("file", pm), ("edgefile", pe), ("binary", pb)):
        conf = cc.parse_parameters(["-input", kind, "-in", str(path)])
        assert same_csr(cc.load_graph(conf), want), kind
    conf = cc.parse_parameters(["-gen", "gnm_undirected", "-n", "10", "-m", "12", "-seed", "3"])
    assert same_csr(cc.load_graph(conf), cc.gen_gnm(1 << 10, 1 << 12, seed=3, id_bytes=4))
    conf = cc.parse_parameters(["-gen", "grid_2d", "-n", "40", "-m", "30", "-p", "0.5", "-seed", "2"])
    assert same_csr(cc.load_graph(conf), cc.gen_grid(40, 30, 0.5, seed=2))
    conf = cc.parse_parameters(["-gen", "rhg", "-n", "12", "-d", "8", "-gamma", "2.6", "-seed", "4"])
    assert same_csr(cc.load_graph(conf), cc.gen_rhg(1 << 12, 8.0, 2.6, seed=4))
    for bad in (["-input", "partition", "-in", str(pe)], ["-gen", "ba"], ["-gen", "grid_2d", "-periodic"], []):
        with pytest.raises(ValueError):
            cc.load_graph(cc.parse_parameters(bad))


def test_cpp_load_graph(tmp_path):
    """ccgpu::LoadGraph (include/components_gb300_io.hpp), compiled with g++
    and linked with libccgen: the same CSR as the Python readers and
    generators."""
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ missing")
    root = Path(__file__).resolve().parent.parent
    exe = tmp_path / "io_main"
    gen_lib, gpu_lib = _lib.BUILD / "libccgen.so", _lib.gpu_lib_path()
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(root / "include"), str(root / "tests" / "cpp" / "io_main.cpp"),
                    "-o", str(exe), str(gen_lib), str(gpu_lib), f"-Wl,-rpath,{gen_lib.parent}"], check=True)

    def run(*args):
        out = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stderr
        lines = out.stdout.splitlines()
        rp = np.array(lines[1].split(), np.uint64)
        col = np.array(lines[2].split(), np.uint64)
        return rp, col

    def same(rpcol, G):
        rp, col = G.numpy()
        return np.array_equal(rpcol[0], rp) and np.array_equal(rpcol[1], col)

    n, edges = 6, [(0, 1), (1, 2), (3, 4), (4, 5)]
    pm = tmp_path / "g.graph"
    write_metis(pm, n, edges)
    assert same(run("file", pm), cc.from_edges(n, edges))
    pb = tmp_path / "g.bin"
    pb.write_bytes(np.array([n, len(edges)], np.uint64).tobytes() + (np.array(edges, np.uint64) + 1).tobytes())
    assert same(run("binary", pb), cc.from_edges(n, edges))
    assert same(run("gen", "gnm_undirected", 500, 900, 1.0, 16.0, 2.2, 3), cc.gen_gnm(500, 900, seed=3))
    assert same(run("gen", "grid_2d", 30, 20, 0.5, 16.0, 2.2, 2), cc.gen_grid(30, 20, 0.5, seed=2))
    bad = subprocess.run([str(exe), "gen", "ba", "10", "10", "1", "1", "1", "1"], capture_output=True, text=True)
    assert bad.returncode == 1 and "not supported" in bad.stderr


def test_device_loader_size_query(tmp_path):
    """The device loaders' size query reads only the header on the host (no
    device call): the vertex count and an upper bound of the entries; bad
    files are refused there already."""
    import ctypes as C
    lib = _lib.gpu()
    n, edges = 6, [(0, 1), (1, 2), (3, 4), (4, 5)]
    pm = tmp_path / "g.graph"
    write_metis(pm, n, edges)
    pb = tmp_path / "g.bin"
    pb.write_bytes(np.array([n, len(edges)], np.uint64).tobytes() + (np.array(edges, np.uint64) + 1).tobytes())
    nn, mm = C.c_uint64(), C.c_uint64()
    assert lib.cc_read_metis_device(None, str(pm).encode(), 4, None, None, 0, C.byref(nn), C.byref(mm)) == 0
    assert nn.value == n and mm.value >= 2 * len(edges)
    assert lib.cc_read_binary_edges_device(None, str(pb).encode(), 4, None, None, 0, C.byref(nn),
                                           C.byref(mm)) == 0
    assert nn.value == n and mm.value == 2 * len(edges)
    (tmp_path / "nohdr.graph").write_text("% only a comment\n")
    (tmp_path / "short.bin").write_bytes(np.array([3, 5], np.uint64).tobytes())
    for fn, name in ((lib.cc_read_metis_device, "nohdr.graph"), (lib.cc_read_binary_edges_device, "short.bin"),
                     (lib.cc_read_metis_device, "missing.graph")):
        assert fn(None, str(tmp_path / name).encode(), 4, None, None, 0, C.byref(nn), C.byref(mm)) == \
            _lib.CC_ERR_INVALID, name
