"""The reference's gsQuadratureRules_test restated for the oracle's Gauss-Legendre rules (the
rules the device tables are built from agree with them through every parity test): an n-point
rule, mapped to [0, 1.0123] per direction (gsQuadRule::mapTo), integrates the polynomial
sum_i x_i^(2 n_i - 1) exactly, in 1D and as tensor rules in 3D, for the node counts the
reference tests (1..22)."""
import itertools

import numpy as np
import pytest

U = 1.0123
CASES = [(3,), (5,), (1, 5, 9), (2, 6, 7), (3, 4, 8), (10, 17), (11, 16), (12, 15), (13, 14), (18,), (19,), (20,),
         (21,), (22,)]


@pytest.mark.parametrize("nodes", CASES, ids=["_".join(map(str, c)) for c in CASES])
def test_gauss_rule_exactness(nodes):
    from oracle import oracle as O
    d = len(nodes)
    rules = []
    for n in nodes:
        x, w = O.gauss(n)
        h = U / 2.0
        rules.append((h * (np.asarray(x) + 1.0), h * np.asarray(w)))
    deg = [max(2 * n - 1, 0) for n in nodes]
    total = 0.0
    for idx in itertools.product(*[range(len(r[0])) for r in rules]):
        wt = np.prod([rules[k][1][i] for k, i in enumerate(idx)])
        pt = [rules[k][0][i] for k, i in enumerate(idx)]
        total += wt * sum(pt[k] ** deg[k] for k in range(d))
    # anti-derivative of sum_i x_i^deg_i over [0, U]^d
    expected = sum(U ** (deg[k] + 1) / (deg[k] + 1) * U ** (d - 1) for k in range(d))
    assert abs(total - expected) <= 1e-12 * abs(expected), (total, expected)
