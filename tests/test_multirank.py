"""Replica parallelism over bitstrings with two gloo ranks on the CPU: each rank computes its
contiguous shard (the oracle stands in for the per-rank GPU programme) and rank 0 gathers; the
result equals the single-process computation.  A rank that fails is seen by the other through
a short process-group timeout instead of a hang."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, result_q, fail_rank):
    import datetime
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import __graft_entry__ as entry
    q = entry.load()
    from oracle import oracle
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    try:
        prog, bits, info = q.workloads.build_workload("rqc_3x4_d8_s3", time=1)
        mine = q.replicas.shard(bits, rank, world)
        if rank == fail_rank:
            raise RuntimeError("injected failure on the host")
        local = oracle.run_programme(prog, mine, nthreads=1)
        full = q.replicas.gather_amplitudes(local, len(bits), rank, world)
        if rank == 0:
            ref = oracle.run_programme(prog, bits, nthreads=1)
            result_q.put(("ok", float(np.max(np.abs(full - ref)))))
    except Exception as e:                      # noqa: BLE001 - reported to the parent
        result_q.put(("error", f"rank {rank}: {type(e).__name__}: {e}"))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, fail_rank=-1):
    ctx = mp.get_context("spawn")
    port = _free_port()
    rq = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, world, port, rq, fail_rank)) for r in range(world)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
    for p in ps:
        if p.is_alive():
            p.kill()
    out = []
    while not rq.empty():
        out.append(rq.get())
    return out


def test_shard_bounds_cover_everything(q):
    for n in (0, 1, 5, 64, 65):
        for w in (1, 2, 3, 8):
            got = []
            for r in range(w):
                b, e = q.replicas.shard_bounds(n, r, w)
                got += list(range(b, e))
            assert got == list(range(n))


def test_two_gloo_ranks_gather_equals_single_process(q):
    res = _run(2)
    oks = [r for r in res if r[0] == "ok"]
    assert oks and oks[0][1] < 1e-15, res


def test_failed_rank_is_reported_not_hung(q):
    res = _run(2, fail_rank=1)
    errs = [r for r in res if r[0] == "error"]
    assert any("injected failure" in e[1] for e in errs), res
