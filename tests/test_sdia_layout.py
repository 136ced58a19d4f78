"""Host model of the half-diagonal FP32 inner operator (gismo_gb300/csrc/sdia.cu).

The layout stores, for a symmetric matrix on a box of m0 x m1 x m2 unknowns numbered
lexicographically with the neighbour box [-p, p]^3, only the diagonals of the lexicographically
non-negative half offsets; the product reads every stored value twice (its own row and the mirrored
one). This test restates the builder's offset order and the kernel's index arithmetic (zero padding
around x and after every diagonal, unclamped indices) in numpy and checks the product against the
full sparse matrix, on boxes down to the smallest width the library accepts (2p + 1)."""
import itertools

import numpy as np
import pytest

scipy_sparse = pytest.importorskip("scipy.sparse")


def half_offsets(p):
    """Storage order of the builder: the centre line (0, 0, o0 >= 0), then the lines (o2, o1) with
    o2 > 0 or (o2 = 0, o1 > 0), o0 ascending."""
    out = [(o0, 0, 0) for o0 in range(0, p[0] + 1)]
    for o2 in range(0, p[2] + 1):
        for o1 in range(-p[1] if o2 else 1, p[1] + 1):
            for o0 in range(-p[0], p[0] + 1):
                out.append((o0, o1, o2))
    return out


def random_box_matrix(m, p, rng):
    n = int(np.prod(m))
    rows, cols, vals = [], [], []
    coords = np.array(list(itertools.product(range(m[2]), range(m[1]), range(m[0]))))[:, ::-1]  # (i0, i1, i2)
    lin = lambda c: c[:, 0] + m[0] * (c[:, 1] + m[1] * c[:, 2])
    for o in itertools.product(*[range(-pk, pk + 1) for pk in p]):
        c2 = coords + np.array(o)
        ok = np.all((c2 >= 0) & (c2 < np.array(m)), axis=1)
        rows.append(lin(coords[ok]))
        cols.append(lin(c2[ok]))
        vals.append(rng.standard_normal(ok.sum()))
    A = scipy_sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    return (A + A.T).tocsr()


def build_half(A, m, p):
    n = A.shape[0]
    H = half_offsets(p)
    d = np.zeros((len(H), n))
    Ad = A.toarray()
    for h, o in enumerate(H):
        for r in range(n):
            b = (r % m[0], (r // m[0]) % m[1], r // (m[0] * m[1]))
            c = tuple(b[k] + o[k] for k in range(3))
            if all(0 <= c[k] < m[k] for k in range(3)):
                d[h, r] = Ad[r, c[0] + m[0] * (c[1] + m[1] * c[2])]
    return d, H


def half_product(d, H, m, x, ns):
    """The kernel's arithmetic: diagonals of stride ns whose padding [n, ns) holds zeros, x with
    `reach` zeros before and after it, no clamping: the mirrored value of row r comes from flat index
    h ns + r - L even when r - L < 0 (diagonal h - 1, multiplied by a padding zero of x)."""
    n = len(x)
    r = np.arange(n)
    reach = max(abs(o[0] + m[0] * (o[1] + m[1] * o[2])) for o in H)
    xp = np.concatenate([np.zeros(reach), x, np.zeros(reach)])
    flat = np.zeros(len(H) * ns)
    for h in range(len(H)):
        flat[h * ns:h * ns + n] = d[h]
    y = np.zeros(n)
    for h, o in enumerate(H):
        L = o[0] + m[0] * (o[1] + m[1] * o[2])
        y += flat[h * ns + r] * xp[reach + r + L]
        if L != 0:
            idx = h * ns + r - L
            assert idx.min() >= 0 and idx.max() < len(flat)
            y += flat[idx] * xp[reach + r - L]
    return y


@pytest.mark.parametrize("m,p", [((7, 7, 7), (3, 3, 3)), ((5, 8, 6), (2, 3, 2)), ((9, 5, 1), (4, 2, 0)),
                                 ((3, 4, 5), (1, 1, 1)), ((12, 7, 1), (3, 3, 0))])
def test_half_diagonal_product_equals_full_product(m, p):
    rng = np.random.default_rng(sum(m) * 7 + sum(p))
    A = random_box_matrix(m, p, rng)
    d, H = build_half(A, m, p)
    assert len(H) == 1 + (np.prod([2 * pk + 1 for pk in p]) - 1) // 2
    # every non-zero of the half box is stored exactly once; the other half is its mirror
    assert np.count_nonzero(d) * 2 - np.count_nonzero(d[0]) == A.nnz
    ns = (A.shape[0] + 255) // 256 * 256
    for _ in range(3):
        x = rng.standard_normal(A.shape[0])
        assert np.allclose(half_product(d, H, m, x, ns), A @ x, rtol=1e-13, atol=1e-12)
    # all mirrored reads stay inside the stored array (the kernel's unclamped value index)
    n = A.shape[0]
    for h, o in enumerate(H):
        L = o[0] + m[0] * (o[1] + m[1] * o[2])
        if h >= 1:
            assert 0 < L < n
            assert h * n + 0 - L >= 0 and h * n + (n - 1) - L < len(H) * n
