"""The algebra behind entity block-Jacobi (no GPU): for a complex-symmetric
entity block A_aa = L D L^T (no pivoting), S = D^-1/2 L^-1 with the
principal square root gives S A S^T = I (COCG runs on S A S^T) and
S^T S = A_aa^-1 (GMRES's right preconditioner M^-1), and M^-1 keeps complex
symmetry."""
import numpy as np


def ldlt_nopivot(a):
    n = a.shape[0]
    w = a.astype(complex).copy()
    L = np.eye(n, dtype=complex)
    d = np.zeros(n, dtype=complex)
    for c in range(n):
        d[c] = w[c, c]
        for i in range(c + 1, n):
            L[i, c] = w[i, c] / d[c]
        for i in range(c + 1, n):
            for j in range(c + 1, n):
                w[i, j] -= L[i, c] * d[c] * L[j, c]
    return L, d


def test_block_factors():
    rng = np.random.default_rng(0)
    for na in (1, 2, 3, 6, 12):
        b = rng.normal(size=(na, na)) + 1j * rng.normal(size=(na, na))
        a = b + b.T + na * (3.0 - 1.0j) * np.eye(na)        # complex symmetric, well conditioned
        L, d = ldlt_nopivot(a)
        assert np.allclose(L @ np.diag(d) @ L.T, a, rtol=1e-12, atol=1e-12)
        S = np.diag(1.0 / np.sqrt(d)) @ np.linalg.inv(L)  # numpy's sqrt is the principal root
        assert np.allclose(S @ a @ S.T, np.eye(na), atol=1e-12)
        minv = S.T @ S
        assert np.allclose(minv, np.linalg.inv(a), rtol=1e-10, atol=1e-12)
        assert np.allclose(minv, minv.T, atol=1e-13)
