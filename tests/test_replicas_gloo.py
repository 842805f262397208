"""bench.py's multi-GPU host logic -- independent replicas, no data-path
collective -- with two gloo ranks on CPU: the barrier, the max over ranks of
the timed seconds, the whole-job value (ranks x steps / slowest rank), and the
reference arm's rule that only rank 0 prints."""
import io
import contextlib
import json
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, ws, port):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)


def _replica(rank, ws, port, q):
    _env(rank, ws, port)
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    secs = 0.5 + rank  # rank 1 is the slowest replica
    slowest = d.max(secs)
    q.put((rank, d.ws, slowest, bench.replica_value(d.ws, 10, slowest)))
    d.barrier()
    d.close()


def _reference_rank(rank, ws, port, q):
    _env(rank, ws, port)
    import bench
    calls = []
    bench.cpu_slices_per_s = lambda *a, **k: (calls.append(a) or (3.0, "port", 2))
    sys.argv = ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1"]
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(bench.parse())
    q.put((rank, out.getvalue(), len(calls)))


def _spawn(target, ws=2):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=target, args=(r, ws, port, q)) for r in range(ws)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


def test_two_replicas_max_and_value():
    pytest.importorskip("torch.distributed")
    res = _spawn(_replica)
    assert [r[0] for r in res] == [0, 1]
    for _, ws, slowest, value in res:
        assert ws == 2
        assert slowest == pytest.approx(1.5)          # max over ranks
        assert value == pytest.approx(2 * 10 / 1.5)   # both ranks' units / slowest time


def test_reference_arm_rank0_only():
    pytest.importorskip("torch.distributed")
    res = _spawn(_reference_rank)
    (r0, out0, n0), (r1, out1, n1) = res
    assert out1 == "" and n1 == 0                       # rank 1: no work, no line
    line = json.loads(out0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    assert n0 >= 2
