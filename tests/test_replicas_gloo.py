"""Multi-process (world_size 2, gloo, CPU) checks of the replica path's host logic:
batch sharding, per-rank seeds, max-over-ranks timing and whole-job throughput.  Rows
of a batch are independent, so each rank simulating its own shard (here with the
oracle) must reproduce the single-process result row for row."""
import json
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from torchquantum_gb300 import replicas as R


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _circuit(n):
    return [("u3", [0], (0.3, -1.1, 0.7)), ("cnot", [0, 2], ()), ("ry", [1], (0.9,)), ("crx", [2, 1], (1.3,)),
            ("cz", [1, 0], ()), ("rz", [2], (-0.4,))]


def _rows(start, count, n):
    """Oracle states of batch rows [start, start + count): row r starts in basis state r % 2^n."""
    from oracle import statevec as O

    out = []
    for r in range(start, start + count):
        s = np.zeros((1, 1 << n), dtype=np.complex128)
        s[0, r % (1 << n)] = 1.0
        for name, wires, p in _circuit(n):
            s = O.apply(s, O.gate_matrix(name, np.array([p]) if p else None), wires, n)
        out.append(s[0])
    return np.array(out).reshape(count, 1 << n)


def _worker(rank, world, port, total, n, outdir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    assert R.init("gloo")
    r, w, local = R.rank_env()
    start, count = R.shard(total, r, w)
    states = _rows(start, count, n)
    t = R.max_over_ranks(1.0 + r)  # rank r "took" 1 + r seconds
    R.barrier()
    np.save(os.path.join(outdir, f"rows{r}.npy"), states)
    with open(os.path.join(outdir, f"rank{r}.json"), "w") as f:
        json.dump({"rank": r, "world": w, "local": local, "start": start, "count": count, "tmax": t,
                   "seed": R.rank_seed(1, r), "rate": R.job_throughput(count, w, t)}, f)
    R.finish()


def test_shard_covers_every_unit_once():
    for total in (0, 1, 7, 16, 257):
        for world in (1, 2, 3, 8):
            got = [R.shard(total, r, world) for r in range(world)]
            assert sum(c for _, c in got) == total
            assert all(got[i][0] + got[i][1] == got[i + 1][0] for i in range(world - 1))
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        R.shard(4, 2, 2)


def test_single_process_defaults(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert R.rank_env() == (0, 1, 0)
    assert R.init("gloo") is False
    assert R.max_over_ranks(3.5) == 3.5
    assert R.job_throughput(16, 1, 2.0) == 8.0


def test_two_ranks_gloo(tmp_path):
    total, n, world = 10, 3, 2
    mp.start_processes(_worker, args=(world, _free_port(), total, n, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    infos = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    assert [i["rank"] for i in infos] == [0, 1] and all(i["world"] == world for i in infos)
    assert [(i["start"], i["count"]) for i in infos] == [(0, 5), (5, 5)]
    assert all(i["tmax"] == 2.0 for i in infos)  # the slowest rank's time on every rank
    assert infos[0]["seed"] != infos[1]["seed"]
    assert infos[0]["rate"] == pytest.approx(5 * 2 / 2.0)
    sharded = np.concatenate([np.load(tmp_path / f"rows{r}.npy") for r in range(world)])
    np.testing.assert_allclose(sharded, _rows(0, total, n), atol=1e-12)


def _leaving_worker(rank, world, port, out_dir):
    import time

    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    R.init("gloo", timeout_s=20)
    R.barrier()  # both ranks arrive here
    if rank == 1:
        os._exit(0)  # leaves between steps, before the next barrier, with nothing in flight
    t0 = time.time()
    err = None
    try:
        R.max_over_ranks(1.0)
    except Exception as e:  # noqa: BLE001 - any error type from the backend is the signal
        err = type(e).__name__
    with open(os.path.join(out_dir, "rank0.json"), "w") as f:
        json.dump({"error": err, "seconds": time.time() - t0}, f)


def test_rank_leaving_surfaces_as_error(tmp_path):
    """Failure detection on the host: a rank that leaves between steps makes the other
    rank's next collective raise (within the process-group timeout) instead of hanging."""
    world = 2
    ctx = mp.start_processes(_leaving_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=False,
                             start_method="spawn")
    while not ctx.join(timeout=60):
        pass
    info = json.load(open(tmp_path / "rank0.json"))
    assert info["error"] is not None and info["seconds"] < 30
