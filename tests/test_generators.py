"""The seeded generators on the CPU.  The random hyperbolic graph is checked
against the model's own edge test applied to every vertex pair (so the
band-and-cell neighbour search misses nothing and adds nothing), for several
sizes, seeds and exponents, and its average degree against the target."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import components_gb300 as cc
from components_gb300 import _lib


def _rhg_host(n, d, gamma, seed, idb=4):
    hg = _lib.cc_host_graph()
    _lib.check(_lib.gen().cc_gen_rhg(n, d, gamma, seed, idb, C.byref(hg)))
    return hg


@pytest.mark.parametrize("k,d,gamma,seed", [(10, 16.0, 2.6, 1), (12, 16.0, 2.6, 7), (12, 4.0, 2.2, 3),
                                            (13, 8.0, 3.0, 11), (11, 32.0, 2.4, 5)])
def test_rhg_equals_all_pairs_test(built, k, d, gamma, seed):
    n = 1 << k
    hg = _rhg_host(n, d, gamma, seed, 8 if k == 11 else 4)
    try:
        bad = _lib.gen().cc_gen_rhg_verify(n, d, gamma, seed, C.byref(hg))
    finally:
        _lib.gen().cc_host_graph_free(C.byref(hg))
    assert bad == 0


def test_rhg_shape(built):
    G = cc.gen_rhg(1 << 16, 16.0, 2.6, seed=1)
    rp, col = G.numpy()
    assert G.m / G.n == pytest.approx(16.0, rel=0.08)
    deg = np.diff(rp)
    assert deg.max() > 50 * deg.mean()  # hubs: the power-law tail
    for v in range(0, G.n, 997):  # rows sorted, no self-loops, symmetric
        row = col[rp[v]:rp[v + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0) and v not in row
        for w in row[:4]:
            assert v in col[rp[w]:rp[w + 1]]


def test_rhg_radius_and_bad_arguments(built):
    R = _lib.gen().cc_gen_rhg_radius(1 << 20, 16.0, 2.6)
    assert 20.0 < R < 40.0 and R * 2 ** 32 == int(R * 2 ** 32)  # a multiple of 2^-32
    hg = _lib.cc_host_graph()
    assert _lib.gen().cc_gen_rhg(1 << 10, 16.0, 2.0, 1, 4, C.byref(hg)) == _lib.CC_ERR_INVALID
    assert _lib.gen().cc_gen_rhg(1, 16.0, 2.6, 1, 4, C.byref(hg)) == _lib.CC_ERR_INVALID
