"""Continuous-batching server on a GB300: every result of a mixed stream (sizes from 8 to 4096,
the three accuracy classes) is bit-identical when the request runs alone and when it runs in the
mix with others in flight; small requests complete through grouped launches that coalesce many
of them; results meet their classes' error bounds against the compensated oracle; admission
honours the memory budget (rejection of requests that can never fit, a peak below the budget);
large requests never hold more than their share of the slots; latency statistics are reported
overall and per size class."""
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
        torch.cuda.synchronize()  # operands and C are ready when a request is submitted
        t = srv.submit(101, 111, 111, n, n, n, 1.0, r["dA"], n, r["dB"], n, 0.0, dC, n, accuracy=r["cls"])
        res = srv.wait(t)
        assert res.status == 0
        outs.append(dC.cpu().numpy())
    return outs


def run_mix(srv, torch, reqs):
    dCs = [torch.zeros(r["n"] * r["n"], dtype=torch.float64, device="cuda") for r in reqs]
    torch.cuda.synchronize()  # operands and C are ready when a request is submitted
    tickets = []
    for r, dC in zip(reqs, dCs):
        n = r["n"]
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
        # small requests (every dimension <= 256) ran in grouped launches: one per request when
        # alone, at most one per request in the mix (how many a launch coalesces there depends on
        # how fast the submissions follow each other; test_small_requests_coalesce_into_grouped_launches
        # checks the coalescing)
        small = sum(1 for r in reqs if r["n"] <= 256)
        assert st.class_completed[0] == 2 * small
        assert st.class_completed[1] + st.class_completed[2] == 2 * (len(reqs) - small)
        assert small < st.grouped_launches <= 2 * small
        for c in range(3):
            if st.class_completed[c]:
                assert 0 < st.class_p50_ms[c] <= st.class_p99_ms[c] <= st.max_ms
        for r, res in zip(reqs, results):
            if r["n"] <= 256:
                assert res.method_used == G.METHOD_NATIVE and res.error_bound == r["n"] * 2.0 ** -53
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


def test_small_requests_coalesce_into_grouped_launches(torch):
    """Many small requests submitted together go out in a few grouped launches, each result equal
    to the oracle's restatement of Blaze's kernel within Blaze's relaxed equality."""
    from helpers import blaze_equal
    srv = G.Server(slots=4, batch_max=512)
    try:
        rng = np.random.default_rng(3)
        reqs = []
        for i in range(600):
            m, n, k = (int(v) for v in rng.integers(4, 200, 3))
            A = O.uniform(m * k, 7000 + 2 * i)
            B = O.uniform(k * n, 7001 + 2 * i)
            reqs.append((m, n, k, A, B, torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(),
                         torch.zeros(m * n, dtype=torch.float64, device="cuda")))
        torch.cuda.synchronize()  # operands and C are ready when a request is submitted
        tickets = [srv.submit(101, 111, 111, m, n, k, 1.0, dA, k, dB, n, 0.0, dC, n, accuracy=CLASSES[i % 3])
                   for i, (m, n, k, A, B, dA, dB, dC) in enumerate(reqs)]
        for t in tickets:
            assert srv.wait(t).status == 0
        st = srv.stats()
        assert st.class_completed[0] == 600
        assert st.grouped_launches < 600 and st.grouped_mean_batch > 1.0
        for (m, n, k, A, B, dA, dB, dC) in reqs:
            R = np.zeros(m * n)
            O.gemm(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, m, n, k, 1.0, A, k, B, n, 0.0, R, n, kernel="default")
            assert blaze_equal(R, dC.cpu().numpy(), 1e-8).all(), (m, n, k)
    finally:
        srv.close()


def test_large_requests_leave_slots_for_the_others(torch):
    """With one large slot, several large products queued ahead of medium ones do not hold the
    other slots: the medium requests finish before the last large one."""
    srv = G.Server(slots=4, large_slots=1, large_threshold=2048)
    try:
        big, mid = 4096, 600
        dA = torch.rand(big * big, dtype=torch.float64, device="cuda")
        Cs = [torch.zeros(big * big, dtype=torch.float64, device="cuda") for _ in range(3)]
        cm = [torch.zeros(mid * mid, dtype=torch.float64, device="cuda") for _ in range(6)]
        torch.cuda.synchronize()
        tl = [srv.submit(101, 111, 111, big, big, big, 1.0, dA, big, dA, big, 0.0, C, big, accuracy="native")
              for C in Cs]
        tm = [srv.submit(101, 111, 111, mid, mid, mid, 1.0, dA, mid, dA, mid, 0.0, C, mid, accuracy="split")
              for C in cm]
        lm = [srv.wait(t).latency_ms for t in tm]
        rl = [srv.wait(t) for t in tl]
        ll = [r.latency_ms for r in rl]
        assert max(lm) < max(ll), (lm, ll)
        # a large native request runs as a chain of k-panels: still FP64-accurate
        assert rl[0].method_used == G.METHOD_NATIVE and rl[0].error_bound == big * 2.0 ** -53
        hA = dA.cpu().numpy()
        rows = np.arange(0, big, big // 8)
        P = O.product_rows_dot2(O.ROW_MAJOR, O.NO_TRANS, O.NO_TRANS, big, big, big, hA, big, hA, big, rows=rows)
        got = Cs[0].view(big, big)[torch.from_numpy(rows).cuda()].cpu().numpy()
        err = float(np.linalg.norm(got - P) * np.sqrt(big / len(rows)) / np.linalg.norm(hA) ** 2)
        assert err <= big * 2.0 ** -53, err
        st = srv.stats()
        assert st.class_completed[2] == 3 and st.class_completed[1] == 6
    finally:
        srv.close()
