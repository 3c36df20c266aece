"""Error of the device reductions on cancellation-heavy data, against exact
arithmetic.

The FP32 build accumulates its dot products and sums in double-float: a
(hi, lo) pair of floats carried by error-free transformations (TwoProduct by
FMA, TwoSum), about 48 significant bits, widened to FP64 once per reduction.
The reference's CUDA backend reduces in its working precision
(algebra/cuda/src/cuda_lin_alg.cu, cuBLAS dot / nrm2).  On data whose terms
cancel to a tiny fraction of their magnitude, a plain FP32 sum loses every
significant digit; the double-float sum must stay within

    |result - exact| <= 2^-23 |exact| + 2^-40 sum|a_i b_i|

(the first term: the FP32 build returns the value as a float; the second:
about 2^-48 per addition, with room for the reduction tree's depth).  FP32
products are exact in FP64 and math.fsum adds them exactly, so the reference
value is the exact dot product rounded once."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cancelling_pair(n, seed):
    rg = np.random.default_rng(seed)
    a = (rg.standard_normal(n) * 10.0 ** rg.uniform(-3, 3, n)).astype(np.float32)
    b = (rg.standard_normal(n) * 10.0 ** rg.uniform(-3, 3, n)).astype(np.float32)
    d = (b * rg.uniform(-1e-6, 1e-6, n)).astype(np.float32)
    # a.b - a.(b + d): the large terms cancel exactly, the rest is -a.d
    a2 = np.concatenate([a, a])
    b2 = np.concatenate([b, -(b + d)]).astype(np.float32)
    p = rg.permutation(2 * n)
    return a2[p], b2[p]


def exact_dot(a, b):
    prods = a.astype(np.float64) * b.astype(np.float64)   # exact: 24 + 24 bits
    return math.fsum(prods.tolist()), float(np.sum(np.abs(prods)))


@pytest.mark.parametrize("n", [1 << 12, 1 << 18])
def test_f32_dot_double_float_bound(n):
    from osqp_gb300.algebra import AlgebraLib
    alg = AlgebraLib("f32")
    a, b = cancelling_pair(n, 11)
    ex, mag = exact_dot(a, b)
    got = float(alg.lib.OSQPVectorf_dot_prod(alg.vec(a), alg.vec(b)))
    bound = 2.0 ** -23 * abs(ex) + 2.0 ** -40 * mag
    assert abs(got - ex) <= bound, (got, ex, mag, abs(got - ex) / mag)
    # the data are hard: summing the FP32 products in FP32, in order, misses the bound
    naive = float(np.cumsum((a * b).astype(np.float32), dtype=np.float32)[-1])
    assert abs(naive - ex) > bound, (naive, ex)


def test_f32_norm_and_sum_double_float_bound():
    from osqp_gb300.algebra import AlgebraLib
    alg = AlgebraLib("f32")
    a, b = cancelling_pair(1 << 16, 12)
    # 2-norm: sum of squares without cancellation, relative bound
    sq = math.fsum((a.astype(np.float64) ** 2).tolist())
    got = float(alg.lib.OSQPVectorf_norm_2(alg.vec(a)))
    assert abs(got - math.sqrt(sq)) <= 2.0 ** -22 * math.sqrt(sq), (got, math.sqrt(sq))
    # signed dots (the support-function terms of the termination test)
    ex_pos = math.fsum((a.astype(np.float64) * np.maximum(b, 0).astype(np.float64)).tolist())
    mag = float(np.sum(np.abs(a.astype(np.float64) * b.astype(np.float64))))
    got = float(alg.lib.OSQPVectorf_dot_prod_signed(alg.vec(a), alg.vec(b), 1))
    assert abs(got - ex_pos) <= 2.0 ** -23 * abs(ex_pos) + 2.0 ** -40 * mag, (got, ex_pos)


def test_f64_dot_bound():
    from osqp_gb300.algebra import AlgebraLib
    alg = AlgebraLib("f64")
    a, b = cancelling_pair(1 << 18, 13)
    ex, mag = exact_dot(a, b)
    got = float(alg.lib.OSQPVectorf_dot_prod(alg.vec(a.astype(np.float64)), alg.vec(b.astype(np.float64))))
    assert abs(got - ex) <= 2.0 ** -52 * abs(ex) + 2.0 ** -40 * mag, (got, ex)
