"""Continuous-batching server on a GB300: every result of a mixed stream (sizes from 8 to 4096,
the three accuracy classes) is bit-identical when the request runs alone and when it runs in the
mix with others in flight; results meet their classes' error bounds against the compensated
oracle; admission honours the memory budget (rejection of requests that can never fit, a peak
below the budget); latency statistics are reported."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu

CLASSES = ["native", "split", "bf16"]
BOUND = {"native": lambda k: k * 2.0 ** -53, "split": lambda k: k * 2.0 ** -53, "bf16": lambda k: 1e-2}


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    G.lib()
    G.device_info()
    return t


def make_requests(torch, sizes, seed):
    reqs = []
    for i, n in enumerate(sizes):
        A = O.uniform(n * n, seed + 3 * i)
        B = O.uniform(n * n, seed + 3 * i + 1)
        reqs.append(dict(n=n, cls=CLASSES[i % 3], A=A, B=B, dA=torch.from_numpy(A).cuda(), dB=torch.from_numpy(B).cuda()))
    return reqs


def run_alone(srv, torch, reqs):
    outs = []
    for r in reqs:
        n = r["n"]
        dC = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        t = srv.submit(101, 111, 111, n, n, n, 1.0, r["dA"], n, r["dB"], n, 0.0, dC, n, accuracy=r["cls"])
        res = srv.wait(t)
        assert res.status == 0
        outs.append(dC.cpu().numpy())
    return outs


def run_mix(srv, torch, reqs):
    dCs, tickets = [], []
    for r in reqs:
        n = r["n"]
        dC = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        dCs.append(dC)
        tickets.append(srv.submit(101, 111, 111, n, n, n, 1.0, r["dA"], n, r["dB"], n, 0.0, dC, n, accuracy=r["cls"]))
    results = [srv.wait(t) for t in tickets]
    assert all(res.status == 0 for res in results)
    return [d.cpu().numpy() for d in dCs], results


def test_results_are_identical_alone_and_in_the_mix(torch):
    sizes = [8, 16, 40, 100, 128, 512, 777, 1024, 2048, 64, 12, 256, 1500, 4096, 96, 33, 600, 2048, 10, 128, 130]
    reqs = make_requests(torch, sizes, seed=500)
    srv = G.Server(slots=6, reserve_sms=16, large_threshold=2048)
    try:
        alone = run_alone(srv, torch, reqs)
        mixed, results = run_mix(srv, torch, reqs)
        for r, a, b, res in zip(reqs, alone, mixed, results):
            assert np.array_equal(a, b), (r["n"], r["cls"])
        # accuracy of every result against the compensated oracle (sampled rows for the large ones)
        for r, c, res in zip(reqs, mixed, results):
            n = r["n"]
            rows = np.arange(0, n, max(1, n // 64))
            P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, n, n, n, r["A"], n, r["B"], n, rows=rows)
            err = float(np.linalg.norm(c.reshape(n, n)[rows] - P) * np.sqrt(n / len(rows)) /
                        (np.linalg.norm(r["A"]) * np.linalg.norm(r["B"])))
            assert err <= BOUND[r["cls"]](n), (n, r["cls"], err)
        st = srv.stats()
        assert st.completed == 2 * len(reqs) and st.failed == 0 and st.rejected == 0
        assert 0 < st.p50_ms <= st.p99_ms <= st.max_ms
        assert st.peak_bytes <= st.budget_bytes
    finally:
        srv.close()


def test_admission_by_memory_budget(torch):
    srv = G.Server(budget_bytes=96 << 20, slots=4)
    try:
        n = 4096
        dA = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        dC = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        with pytest.raises(G.Gb300Error) as ei:
            srv.submit(101, 111, 111, n, n, n, 1.0, dA, n, dA, n, 0.0, dC, n, accuracy="split")
        assert ei.value.status == G.ERR_ADMISSION
        # requests that fit still run, several at a time, within the budget
        reqs = make_requests(torch, [300, 500, 700, 300, 500, 700, 900], seed=900)
        outs, results = run_mix(srv, torch, reqs)
        st = srv.stats()
        assert st.completed == len(reqs) and st.rejected == 1
        assert st.peak_bytes <= st.budget_bytes
    finally:
        srv.close()


def test_invalid_requests_are_refused(torch):
    srv = G.Server(slots=2)
    try:
        d = torch.zeros(64, dtype=torch.float64, device="cuda")
        with pytest.raises(G.Gb300Error) as ei:
            srv.submit(101, 111, 111, 8, 8, 8, 1.0, d, 4, d, 8, 0.0, d, 8)  # lda too small
        assert ei.value.status == G.ERR_INVALID_ARG
    finally:
        srv.close()
