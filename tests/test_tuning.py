"""Runtime bin thresholds and the autotuner: every setting in range gives the
oracle's product; out-of-range settings are refused."""
import numpy as np
import pytest

import dbd_gb300 as dbd
from dbd_gb300 import generators as gen
from test_gpu_parity import check, mixed_rows

pytestmark = pytest.mark.gpu

EXTREMES = [
    dict(warp_span_words=1, warp_max_nnz=1, sym_warp_max_products=32, rank_words_max=1, rank_shared_max_nnz=1,
         sym_hash_span_words=0, dense_warp_span_words=0, mid_span_words=0, dense_method=1),
    dict(warp_span_words=64, warp_max_nnz=256, sym_warp_max_products=512, rank_words_max=8192,
         rank_shared_max_nnz=4096, sym_hash_span_words=1 << 26, dense_warp_span_words=16, mid_span_words=2048,
         dense_method=2),
    dict(warp_span_words=8, warp_max_nnz=64, sym_warp_max_products=128, rank_words_max=1024,
         rank_shared_max_nnz=512, sym_hash_span_words=512, dense_warp_span_words=4, mid_span_words=100,
         dense_method=0),
    dict(warp_span_words=32, warp_max_nnz=128, sym_warp_max_products=256, rank_words_max=2048,
         rank_shared_max_nnz=1024, sym_hash_span_words=2048, dense_warp_span_words=8, mid_span_words=0,
         dense_method=3),
]


@pytest.mark.parametrize("knobs", EXTREMES)
def test_any_tuning_gives_the_oracle_product(orc, knobs):
    rng = np.random.default_rng(2)
    cases = [mixed_rows(rng, 400, 3000, 20000), mixed_rows(rng, 400, 3000, 600000),
             (gen.banded(2000, 32, seed=1), gen.banded(2000, 32, seed=2)), (gen.rmat(12, 8, seed=3), None)]
    with dbd.Context(cpu_gib=16, gpu_gib=16) as c:
        c.set_tuning(**knobs)
        assert c.tuning == knobs
        for A, B in cases:
            res = c.spgemm(A, B, scope="kernel")
            check(res.C, A, A if B is None else B, orc)


def test_out_of_range_tuning_refused(ctx):
    before = ctx.tuning
    for k, v in [("warp_span_words", 65), ("warp_max_nnz", 0), ("sym_warp_max_products", 513),
                 ("rank_words_max", 8193), ("rank_shared_max_nnz", 4097), ("sym_hash_span_words", -1),
                 ("dense_warp_span_words", 17), ("mid_span_words", 2049), ("dense_method", 4)]:
        with pytest.raises(dbd.DBDError):
            ctx.set_tuning(**{k: v})
    assert ctx.tuning == before


def test_autotune_keeps_parity(orc):
    A = gen.rmat(13, 8, seed=5)
    with dbd.Context(cpu_gib=16, gpu_gib=16) as c:
        c.spgemm(A, scope="kernel", fetch=False)
        best, ms = c.autotune(repeats=1)
        assert ms > 0 and c.tuning == best
        res = c.spgemm(A, scope="kernel")
        check(res.C, A, A, orc)


def test_autotune_after_a_batch(orc):
    pairs = [(gen.poisson_rows(500, 12, s), gen.poisson_rows(500, 12, s + 1)) for s in range(4)]
    pairs += [(gen.banded(700, 32, s), gen.banded(700, 32, s + 1)) for s in range(4)]
    As, Bs = [a for a, _ in pairs], [b for _, b in pairs]
    with dbd.Context(cpu_gib=16, gpu_gib=16) as c:
        c.spgemm_batched(As, Bs, scope="kernel", fetch=False)
        c.autotune(repeats=1)
        res = c.spgemm_batched(As, Bs, scope="kernel")
        for q in range(len(As)):
            check(res.C[q], As[q], Bs[q], orc)
