"""The product's host-side input builders reproduce the reference's factories
bit for bit (same generator, same draw order) -- checked against the oracle,
which restates factory/tt_factory.hpp and tt_matrix_factory.hpp."""
import numpy as np
import pytest

from oracle import pyoracle as O


def same(a, b):
    return len(a) == len(b) and all(x.shape == y.shape and np.array_equal(x, y)
                                    for x, y in zip(a, b))


@pytest.mark.parametrize("shape,rank,seed", [([4] * 10, 8, 42), ([2, 3, 4], 100, 0),
                                             ([8] * 5, 16, 46), ([3], 5, 7)])
def test_random_tt(ttg, shape, rank, seed):
    assert same(ttg.random(shape, rank, seed), O.random(shape, rank, seed))
    assert same(ttg.random(shape, rank, seed, fan_in_scale=True),
                O.random(shape, rank, seed, fan_in_scale=True))


def test_random_matrix(ttg):
    a = ttg.random_matrix([4] * 5, [4] * 5, 8, 44, fan_in_scale=True)
    b = O.random_matrix([4] * 5, [4] * 5, 8, 44, fan_in_scale=True)
    assert same(a, b) and a[0].ndim == 4


def test_random_uneven(ttg):
    for s in (1000, 1001, 5095):
        assert same(ttg.random_uneven(s), O.random_uneven(s))


def test_ones_add_sub(ttg):
    a, b = ttg.random([3, 4, 5], 4, 1), ttg.random([3, 4, 5], 4, 2)
    assert same(ttg.add(a, b), O.add(a, b))
    assert same(ttg.sub(a, b), O.sub(a, b))
    assert same(ttg.axpby(2.5, a, -0.7, b), O.axpby(2.5, a, -0.7, b))
    assert same(ttg.ones([2, 3]), O.ones([2, 3]))
    assert same(ttg.add(ttg.ones([4]), ttg.ones([4])), O.add(O.ones([4]), O.ones([4])))
