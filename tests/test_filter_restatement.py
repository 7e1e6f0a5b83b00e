"""The numpy restatement of the general-weight filters in tests/test_gpu_filter_weighted.py (the
GPU test's expected values) agrees with the C oracle's table path, which
tests/test_oracle_vs_reference.py pins bit for bit to the reference's own HeavisideFilter and
DensityFilter routines called with a general weight functor. CPU only."""
import numpy as np
import pytest

from oracle import build as obuild
from tests import test_gpu_filter_weighted as G


@pytest.fixture(scope="module")
def oracle():
    from oracle.olib import Oracle
    obuild.build_oracle()
    return Oracle("oracle")


@pytest.mark.parametrize("nd,shape,R", [(2, (40, 30, 1), 3.0), (3, (14, 12, 10), 2.5)])
def test_restatement_matches_oracle(oracle, nd, shape, R):
    q = 9 if nd == 2 else 15
    L = oracle.lat(q, *shape)
    n = shape[0] * shape[1] * shape[2]
    tp = G.taps(nd, R)
    assert oracle.filter_ntaps(L, R) == len(tp)
    rng = np.random.default_rng(5)
    s, d = rng.random(n), rng.standard_normal(n)
    table = 0.1 + rng.random((n, len(tp)))
    wfun = lambda t, i, j, k, i2, j2, k2: table[i + shape[0] * (j + shape[1] * k), t]  # noqa: E731
    ref = G.filters(nd, shape, R, 8.0, s, d, wfun)
    for op in range(3):
        G.close(oracle.filter_table(L, op, R, s, table, b=d, beta=8.0), ref[op], 1e-14)
