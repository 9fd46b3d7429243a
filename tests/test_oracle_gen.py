"""CPU checks: the oracle's web-like generator and threaded transpose give the
same arrays as the product's host generator and transpose, so the CPU
reference arm of the benchmark can build the benchmark graph without loading
the product library."""
import numpy as np
import pytest

from oracle import pyoracle as O


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    pagerank_gb300.load()
    return pagerank_gb300


@pytest.mark.parametrize("n,dmin,seed", [(1, 5.9, 42), (1000, 5.9, 42), (50_000, 5.9, 7), (20_000, 40.0, 3)])
def test_weblike_equal_to_product_generator(pg, n, dmin, seed):
    want = pg.graphs.weblike(n, alpha=2.1, dmin=dmin, dmax=100000, local=0.7, window=4096, seed=seed)
    got = O.gen_weblike(n, alpha=2.1, dmin=dmin, dmax=100000, local=0.7, window=4096, seed=seed)
    for a, b in zip(got, want):
        assert np.array_equal(a, np.asarray(b))


def test_threaded_transpose_equal(pg):
    xoff, xedg = O.gen_weblike(30_000, seed=11)
    serial = O.transpose(xoff, xedg)
    threaded = O.transpose(xoff, xedg, threads=True)
    prod = pg.graphs.transpose(xoff, xedg)
    for a, b, c in zip(serial, threaded, prod):
        assert np.array_equal(a, b) and np.array_equal(a, np.asarray(c))


def test_weblike_rejects_bad_arguments():
    with pytest.raises(ValueError):
        O.gen_weblike(0)
    with pytest.raises(ValueError):
        O.gen_weblike(10, alpha=1.0)
