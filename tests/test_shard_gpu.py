"""GPU test of the row-sharded product: shards of A's rows (cut by product
count) multiplied by the device entry point, one after another on one GPU
in place of one GPU per rank, and concatenated with the offsets the ranks
would exchange, equal the single product and the oracle."""
import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nshards", [2, 3, 8])
def test_row_shards_concatenate_to_the_single_product(spws_lib, nshards):
    import sparsews_gb300 as sp
    from sparsews_gb300 import shard
    A = gen.rmat(13, 16, seed=41)
    b = shard.shard_bounds(A, A, nshards)
    parts = [sp.spgemm(shard.sub_rows(A, int(b[r]), int(b[r + 1])), A) for r in range(nshards)]
    pos, crd, vals = shard.concat_shards(parts)
    single = sp.spgemm(A, A)
    assert np.array_equal(pos, single[0]) and np.array_equal(crd, single[1])
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2]
    assert_csr_close((pos, crd, vals), oracle.spgemm("hash", A, A), scale, f"{nshards} shards vs oracle")
    assert_csr_close((pos, crd, vals), single, scale, f"{nshards} shards vs single")
