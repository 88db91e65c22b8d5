"""Host logic of the multi-rank bench path on CPU (gloo, world size 2): configuration sharding
by rank, the max-over-ranks timing reduction, and the reference arm's rank-0-only rule."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    res = {}
    for name, w in bench.WORKLOADS.items():
        base = bench.conf_base_of(rank, w)
        n = sum(g[1] for g in w["groups"])
        res[name] = [base, base + n]
    # each rank times a different interval; every rank must see the largest
    res["max_ms"] = bench.max_over_ranks(dist, 10.0 + 5.0 * rank, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_two_rank_sharding_and_max_reduction(tmp_path):
    import torch.multiprocessing as mp

    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), str(tmp_path)), nprocs=ws,
                       start_method="spawn", join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(ws)]
    for r in res:
        assert r["max_ms"] == 15.0
    for name in res[0]:
        if name == "max_ms":
            continue
        a, b = res[0][name], res[1][name]
        # disjoint, contiguous ranges of disorder seeds: rank 1 starts where rank 0 ends
        assert a[0] == 0 and a[1] == b[0] and b[1] - b[0] == a[1] - a[0]


def test_reference_arm_nonzero_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"], env=env, capture_output=True,
                       text=True, timeout=120)
    assert p.returncode == 0
    assert p.stdout.strip() == ""


@pytest.mark.parametrize("name", ["batched_fp32_L32_64x32", "mixed_L16_24_32_48",
                                  "large_L96_vac5_wolff_8x48", "local_fp64_L16_T9.5"])
def test_workload_table_matches_configurations(name):
    sys.path.insert(0, ROOT)
    import bench

    w = bench.WORKLOADS[name]
    sites = sum(L ** 3 * n * r for L, n, r in w["groups"])
    expect = {"batched_fp32_L32_64x32": 2048 * 32 ** 3,
              "mixed_L16_24_32_48": 128 * 16 * 16 ** 3 + 64 * 24 * 24 ** 3 + 32 * 32 * 32 ** 3
              + 8 * 48 * 48 ** 3,
              "large_L96_vac5_wolff_8x48": 384 * 96 ** 3,
              "local_fp64_L16_T9.5": 16 ** 3}[name]
    assert sites == expect
