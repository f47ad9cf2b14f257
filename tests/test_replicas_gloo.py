"""The multi-GPU path on CPU: two ranks over the gloo backend (127.0.0.1).

Each rank transports its own block of primaries with the oracle (the
engine's per-primary streams are the same), with no data-path collective;
the job figures come from one reduction.  The union of the ranks' showers
must equal one process transporting every block."""
import os
import socket

import pytest

from conftest import BUNDLED_NPZ

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402

N_PER_RANK = 2
STEPS = 2
SEED = 11


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _showers(first, n):
    from oracle.shower import OracleShower, OracleTables
    sh = OracleShower(OracleTables(BUNDLED_NPZ, "graphite"), 0.010, seed=SEED)
    out = []
    for j in range(n):
        rows = sh.generate_shower((1.0, 0.0, 0.0, (1.0 - 0.000511 ** 2) ** 0.5), pid=11, mass=0.000511,
                                  primary_index=first + j)
        out.append((first + j, len(rows), tuple(r.pid for r in rows)))
    return out


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from petite_gb300.replicas import first_primary, reduce_job
    done, rows = [], 0
    for s in range(STEPS):
        res = _showers(first_primary(s, rank, world, N_PER_RANK), N_PER_RANK)
        done += res
        rows += sum(r[1] for r in res)
    t_max, rows_all = reduce_job(0.5 + rank, rows, dist)
    q.put((rank, done, rows, t_max, rows_all))
    dist.destroy_process_group()


def test_two_ranks_cover_disjoint_blocks_and_reduce():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    indices = sorted(i for _, done, *_ in got for i, _, _ in done)
    assert indices == list(range(world * N_PER_RANK * STEPS))       # disjoint, complete
    single = {i: (n, pids) for i, n, pids in _showers(0, world * N_PER_RANK * STEPS)}
    for _, done, *_ in got:
        for i, n, pids in done:
            assert single[i] == (n, pids)                          # same showers as one process
    total = sum(r[2] for r in got)
    for _, _, _, t_max, rows_all in got:
        assert t_max == 1.5 and rows_all == total                  # max time, summed units
