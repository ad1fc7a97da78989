"""The quadrature far-field form, restated in the oracle (oracle.pair_quad):
the checker of a planned GPU form, pinned to the analytic pair force.

A pair's nodal forces are line integrals of (σ̃ b) × l, with σ̃ the other
segment's non-singular stress (the reference's σ̃ formula).  Gauss rules
converge fast in L/R. Against the analytic formula (the reference's
arithmetic), at centre distances R = R/L × (L1 + L2)/2, per pair relative to
its largest force, the 3-point rule must stay within 1e-5 at R/L = 10
(measured max 2.5e-6) and 1e-7 at R/L = 30 (measured 3.3e-8).  At R/L = 30
the 2-point rule must stay within 1e-4 (measured 1.1e-5), and its median must
fall from R/L = 10 to 30 by more than 10 (measured 28).
Beyond R/L ~ 100 the analytic formula's own FP64 error (up to ~6e-4 against
long double) dominates any comparison.
"""
import numpy as np
import pytest

K5 = np.array([1.0, 1 / (4 * np.pi), 1 / (8 * np.pi), 1 / (4 * np.pi) / (1 - 0.28), 0.28 / (4 * np.pi) / (1 - 0.28)])


def _errors(oracle, rl, nq, seed, m=60):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(m):
        L1, L2 = rng.uniform(20, 200, 2)
        d1, d2, off, b1, b2 = (v / np.linalg.norm(v) for v in rng.normal(size=(5, 3)))
        n11 = rng.normal(size=3) * 10
        n12 = n11 + d1 * L1
        n21 = n11 + off * rl * 0.5 * (L1 + L2)
        n22 = n21 + d2 * L2
        F = oracle.pair(K5, b1, n11, n12, b2, n21, n22)
        Q = oracle.pair_quad(K5, b1, n11, n12, b2, n21, n22, nq)
        out.append(np.abs(Q - F).max() / np.abs(F).max())
    return np.array(out)


@pytest.mark.parametrize("rl,bound", [(10, 1e-5), (30, 1e-7)])
def test_three_point_rule(oracle, rl, bound):
    e = _errors(oracle, rl, 3, seed=rl)
    assert e.max() <= bound, (np.median(e), e.max())


def test_two_point_rule_order(oracle):
    e10 = _errors(oracle, 10, 2, seed=1)
    e30 = _errors(oracle, 30, 2, seed=1)
    assert e30.max() <= 1e-4, e30.max()
    assert np.median(e10) >= 10 * np.median(e30), (np.median(e10), np.median(e30))


def test_rule_bounds(oracle):
    z = np.zeros(3)
    x = np.array([100.0, 0.0, 0.0])
    assert not np.any(oracle.pair_quad(K5, x, z, x, x, z + 500, x + 500, 0))  # nq outside 1..4: zeros
