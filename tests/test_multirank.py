"""The N > 1 host logic of bench.py on the CPU: one process per rank over
gloo (world size 2), the slowest rank's time taken by every rank, the
whole-job rate, and the reference arm run by rank 0 alone.  The GPU work of
each rank (an independent replica: no collective in the data path) is not
part of these tests."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(10.0 + 5.0 * rank, world)  # rank 1 is the slow one
    out.put((rank, slowest, bench.whole_job_gedges(world, 1_000_000, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [15.0, 15.0]  # both ranks hold the max
    # two replicas of 1e6 entries each in 15 ms per step: 2e6 / 15e-3 / 1e9 Gedges/s
    assert got[0][2] == pytest.approx(2e6 / 15e-3 / 1e9)


def test_one_rank_needs_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.whole_job_gedges(1, 134_191_308, 1.59) == pytest.approx(84.4, rel=1e-3)


def _bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_rank0_only():
    """Under torchrun every rank runs bench.py --impl reference: ranks other
    than 0 exit 0 without work or output, rank 0 prints the one JSON line."""
    r1 = _bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--impl", "reference", "--gpus", "2")
    assert r1.returncode == 0 and r1.stdout.strip() == ""
    r0 = _bench({"RANK": "0", "WORLD_SIZE": "2", "LOCAL_RANK": "0"}, "--impl", "reference", "--gpus", "2",
                "--workload", "grid", "--grid", "256", "--steps", "1", "--warmup", "0")
    assert r0.returncode == 0, r0.stderr[-2000:]
    lines = [ln for ln in r0.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"


_NO_GPU_LIB = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
args = bench.parse_args(["--impl", "reference", "--rhg-log2n", "12", "--steps", "1", "--warmup", "0"])
line = bench.reference_arm(args, bench.Workload("rhg", args), 1)
maps = open("/proc/self/maps").read()
print(json.dumps({"line": line, "gpu_lib": "libccgpu" in maps, "gen_lib": "libccgen" in maps,
                  "imported": any(m.startswith("components_gb300") for m in sys.modules)}))
"""


def test_reference_arm_loads_no_library_of_ours():
    """The reference arm builds its graph through the oracle's own input path:
    components_gb300 is never imported, and neither libccgpu.so nor
    libccgen.so is mapped into the process."""
    r = subprocess.run([sys.executable, "-c", _NO_GPU_LIB, str(ROOT)], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert not d["gpu_lib"] and not d["gen_lib"] and not d["imported"]
    assert d["line"]["impl"] == "reference" and d["line"]["value"] > 0


def test_both_arms_build_the_same_graph_and_config():
    """Workload.ours_host() (libccgen) and Workload.oracle() (the oracle's
    linked copy of the generators) give the same CSR, so both arms print the
    same config dict (the GPU arm's device generators give that CSR too: a
    GPU test checks them against the host generators)."""
    import numpy as np
    sys.path.insert(0, str(ROOT))
    import bench
    for wl_name, extra in (("rhg", ["--rhg-log2n", "13"]), ("grid", ["--grid", "96"])):
        args = bench.parse_args(["--workload", wl_name, *extra])
        wl = bench.Workload(wl_name, args)
        a, b = wl.ours_host(), wl.oracle()
        ra, ca = a.numpy()
        rb, cb = b.numpy()
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb)
        assert wl.config(a.n, a.m, 2) == wl.config(b.n, b.m, 2)
