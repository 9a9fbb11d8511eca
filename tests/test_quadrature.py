"""Quadrature rules of the curved-element path (host library) against the
oracle's stand-ins for Gmsh's Gauss(2p) rules: same point count, points in
the same order (the first face points define the reference's normal sign and
3-D tangent frame) and weights; and exactness on monomials up to the rule's
degree."""
import math

import numpy as np
import pytest

CASES = [(1, n) for n in (2, 3, 4, 5)] + [(2, d) for d in (2, 4, 6, 8)] + [(3, d) for d in (2, 4, 6, 8)]


@pytest.mark.parametrize("kind,degree", CASES)
def test_rule_matches_oracle(pkg, oracle, kind, degree):
    x, w = pkg.host.quadrature(kind, degree)
    xo, wo = oracle.rule(kind, degree)
    assert x.shape == xo.shape and w.shape == wo.shape
    np.testing.assert_allclose(x, xo, rtol=0, atol=2e-15)
    np.testing.assert_allclose(w, wo, rtol=0, atol=2e-15)


def _simplex_monomial(e):
    """Integral of prod x_d^e_d over the unit simplex: prod(e_d!) / (dim + sum e)!"""
    return math.prod(math.factorial(a) for a in e) / math.factorial(len(e) + sum(e))


@pytest.mark.parametrize("kind,degree", CASES)
def test_rule_is_exact(pkg, kind, degree):
    x, w = pkg.host.quadrature(kind, degree)
    if kind == 1:
        # n Gauss points integrate degree 2n - 1 exactly on [-1, 1]
        for k in range(2 * degree):
            exact = 0.0 if k % 2 else 2.0 / (k + 1)
            assert abs(np.dot(w, x[:, 0] ** k) - exact) < 1e-14, k
        return
    dim = kind
    for total in range(degree + 1):
        for e in np.ndindex(*([total + 1] * dim)):
            if sum(e) != total:
                continue
            val = np.dot(w, np.prod(x ** np.array(e), axis=1))
            assert abs(val - _simplex_monomial(e)) < 1e-13, (e, val)
