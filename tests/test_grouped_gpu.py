"""Persistent grouped GEMM (many uneven small products in one launch, CUDA graph) on a GB300:
every product of a seeded log-uniform batch against the oracle's restatement of Blaze's default
kernel (Blaze's relaxed equality for double, a float rounding bound for float), mixed storage
orders / transpositions / alpha-beta, plan re-runs, the per-product loop as a second witness, and
results unchanged by autotuning."""
import numpy as np
import pytest

import blaze_gb300 as G
import oracle as O
from batched import build, reference
from helpers import blaze_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    G.lib()
    G.device_info()
    return t


def check_batch(specs, got, ref, dtype):
    for sp in specs:
        sl = slice(sp["offC"], sp["offC"] + sp["rc"] * sp["ldc"])
        if dtype == np.float64:
            assert blaze_equal(ref[sl], got[sl], 1e-8).all(), sp
        else:
            err = np.max(np.abs(got[sl].astype(np.float64) - ref[sl].astype(np.float64)), initial=0.0)
            assert err <= max(sp["k"], 1) * 2.0 ** -21 * 4, (sp, err)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_grouped_batch_matches_oracle(torch, dtype):
    specs, A, B, C0, dA, dB, dC = build(torch, 600, seed=3, dtype=dtype, layouts=True, alphabeta=True)
    probs = G.problems(specs)
    (G.dgemm_grouped if dtype == np.float64 else G.sgemm_grouped)(probs)
    torch.cuda.synchronize()
    check_batch(specs, dC.cpu().numpy(), reference(specs, A, B, C0), dtype)


def test_plan_reruns_and_matches_per_product_loop(torch):
    specs, A, B, C0, dA, dB, dC = build(torch, 300, seed=5)
    probs = G.problems(specs)
    plan = G.GroupedPlan(probs, 8)
    ntiles, useful, padded = plan.info()
    assert ntiles > 0 and padded >= useful > 0
    plan.run()
    G.synchronize()
    first = dC.cpu().numpy().copy()
    plan.run()
    plan.run()
    G.synchronize()
    assert np.array_equal(first, dC.cpu().numpy())  # beta = 0: identical on every run
    plan.close()
    # a loop of single-product calls on the same operands agrees within Blaze's tolerance
    dC2 = torch.zeros_like(dC)
    for sp in specs:
        G.dgemm_ex(sp["order"], sp["transA"], sp["transB"], sp["m"], sp["n"], sp["k"], sp["alpha"], sp["A"], sp["lda"],
                   sp["B"], sp["ldb"], sp["beta"], dC2.data_ptr() + sp["offC"] * 8, sp["ldc"],
                   G.opts(method="native", residency=G.PTR_DEVICE))
    torch.cuda.synchronize()
    assert blaze_equal(dC2.cpu().numpy(), first, 1e-8).all()


def test_autotuned_table_keeps_results(torch, tmp_path):
    specs, A, B, C0, dA, dB, dC = build(torch, 200, seed=9, dtype=np.float64)
    G.grouped_autotune(8, 1)
    path = tmp_path / "tune.txt"
    G.lib().gb300_grouped_tuning_save(str(path).encode())
    lines = path.read_text().splitlines()
    # an autotuned table keeps its measured costs and the shape-picking policy the autotuner chose
    assert lines[0] == "gb300-grouped-tune v2" and lines[1].startswith("mode ")
    assert len(lines[2].split()) == 5 + 6
    before = [G.grouped_shape_for(8, m, n, k) for (m, n, k) in ((5, 9, 30), (100, 20, 300), (250, 40, 7))]
    assert G.lib().gb300_grouped_tuning_load(str(path).encode()) == 0
    assert [G.grouped_shape_for(8, m, n, k) for (m, n, k) in ((5, 9, 30), (100, 20, 300), (250, 40, 7))] == before
    G.dgemm_grouped(G.problems(specs))
    torch.cuda.synchronize()
    check_batch(specs, dC.cpu().numpy(), reference(specs, A, B, C0), np.float64)


def test_empty_and_degenerate_problems(torch):
    specs, A, B, C0, dA, dB, dC = build(torch, 20, seed=11)
    specs[0]["k"] = 0          # C = beta*C
    specs[1]["alpha"] = 0.0    # A, B not referenced
    specs[2]["m"] = 0          # nothing to do
    G.dgemm_grouped(G.problems(specs))
    torch.cuda.synchronize()
    got = dC.cpu().numpy()
    sp = specs[0]
    sl = slice(sp["offC"], sp["offC"] + sp["rc"] * sp["ldc"])
    assert np.all(got[sl] == 0.0)  # beta = 0
    check_batch(specs[3:], got, reference(specs[3:], A, B, C0), np.float64)
