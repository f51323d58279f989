"""The device loaders (cc_read_metis_device, cc_read_binary_edges_device):
the file's bytes parsed and the CSR built on the GPU, bit for bit the CSR of
the host readers (the reference's GraphIO formats), on every line-format case
the host reader tests cover, and the same errors."""
from __future__ import annotations

import numpy as np
import pytest

import components_gb300 as cc
from components_gb300 import _lib
from test_readers import write_metis

pytestmark = pytest.mark.gpu


def same(dev, host):
    rd, cd = dev.numpy()
    rh, ch = host.numpy()
    return np.array_equal(rd, rh) and np.array_equal(cd, ch)


@pytest.mark.parametrize("idb", [4, 8])
def test_device_loaders_equal_host_readers(cuda, tmp_path, idb):
    rng = np.random.default_rng(5)
    n = 3000
    e = rng.integers(0, n, size=(12000, 2))
    edges = [(int(u), int(w)) for u, w in e]  # self-loops and repeats: dropped by both
    pm = tmp_path / "g.metis"
    write_metis(pm, n, [(u, w) for u, w in edges if u != w])
    assert same(cc.read_metis_device(str(pm), id_bytes=idb), cc.read_metis(str(pm), id_bytes=idb))
    pb = tmp_path / "g.bin"
    pb.write_bytes(np.array([n, len(edges)], np.uint64).tobytes() + (np.array(edges, np.uint64) + 1).tobytes())
    assert same(cc.read_binary_edges_device(str(pb), id_bytes=idb), cc.read_binary_edges(str(pb), id_bytes=idb))


def test_device_metis_line_cases(cuda, tmp_path):
    """CRLF ends, tabs, trailing blanks, comments before the header and between
    vertex lines, missing trailing lines, a line cut short by a character
    that is not a digit or blank, extra lines beyond n, a file without a final
    newline, and a header with a format field."""
    cases = {
        "crlf": "% c\r\n5 3\r\n2 \r\n1\t3\r\n% between\r\n2\r\n5\r\n4\r\n",
        "short": "4 1\n2\n1\n",
        "cut": "5 4\n2 3 x 4\n1\n1 4\n3 # 5 1\n\n",
        "extra": "3 2\n2\n1 3\n2\n1 2 3\n",
        "nofinal": "3 2\n2\n1 3\n2",
        "fmt": "%% header with format\n4 3 0\n2 3 4\n1\n1\n1\n",
        "spaces_pct": "3 1\n  % 2\n3\n2\n",
    }
    for name, text in cases.items():
        p = tmp_path / f"{name}.graph"
        p.write_bytes(text.encode())
        assert same(cc.read_metis_device(str(p)), cc.read_metis(str(p))), name


def test_device_loader_errors_and_reuse(cuda, tmp_path):
    """Ids outside [1, n] give CC_ERR_INVALID (as the host readers) and the
    context stays usable; a bigger file after a smaller one regrows the
    staging."""
    for name, text in (("m0", "3 1\n0\n\n\n"), ("mbig", "3 1\n4\n\n\n")):
        p = tmp_path / name
        p.write_text(text)
        with pytest.raises(_lib.CCError) as ei:
            cc.read_metis_device(str(p))
        assert ei.value.status == _lib.CC_ERR_INVALID, name
    pb = tmp_path / "bad.bin"
    pb.write_bytes(np.array([3, 1], np.uint64).tobytes() + np.array([1, 4], np.uint64).tobytes())
    with pytest.raises(_lib.CCError):
        cc.read_binary_edges_device(str(pb))
    G = cc.gen_rhg(1 << 14, 8.0, 2.4, seed=3)
    rp, col = G.numpy()
    pm = tmp_path / "rhg.graph"
    rows = [" ".join(str(int(w) + 1) for w in col[rp[v]:rp[v + 1]]) for v in range(G.n)]
    pm.write_text(f"{G.n} {G.m // 2}\n" + "\n".join(rows) + "\n")
    D = cc.read_metis_device(str(pm))
    assert same(D, G)
    lab = cc.find_components(D, "exp")
    assert np.array_equal(lab.cpu().numpy().view(np.uint32), cc.find_components(G, "exp"))
