"""The multi-process (N > 1) path of bench.py on CPU: two ranks with the gloo backend on 127.0.0.1
run the same collectives as the NCCL run (the timing barrier and the max over ranks), and the
reference arm runs on rank 0 alone, which prints the one JSON line while rank 1 exits quietly."""
import contextlib
import io
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world, backend="gloo")
    try:
        d.barrier()
        mx = d.max(float(10 * rank + 1))
        ns = type("A", (), dict(size=128, steps=1, warmup=1, seed=42, gpus=world))()
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            bench.reference_arm(ns, d)
        d.barrier()
        q.put((rank, mx, buf.getvalue()))
    finally:
        d.close()


def test_two_gloo_ranks_share_the_barrier_and_the_max_and_rank0_alone_reports():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        rank, mx, text = q.get(timeout=240)
        out[rank] = (mx, text)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 11.0  # max over ranks of 1.0 and 11.0
    assert out[1][1] == ""  # rank 1 prints nothing
    lines = [ln for ln in out[0][1].splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
