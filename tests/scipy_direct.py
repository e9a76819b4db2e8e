"""Independent direct solve for the acceptance tests (assembled CSR + spsolve).

A second oracle built a different way from the matrix-free path: the
finite-volume operator (harmonic faces, boundary face = own permeability, as
in the reference's python/darcy/reference.py:29-85) assembled as a sparse
matrix and factorised.
"""

from __future__ import annotations

import numpy as np


def assemble(a: np.ndarray):
    from scipy import sparse

    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    hm = lambda x, y: 2.0 * x * y / (x + y)  # noqa: E731
    east = np.empty_like(a)
    east[:, :-1] = hm(a[:, :-1], a[:, 1:])
    east[:, -1] = a[:, -1]
    west = np.empty_like(a)
    west[:, 1:] = hm(a[:, 1:], a[:, :-1])
    west[:, 0] = a[:, 0]
    north = np.empty_like(a)
    north[:-1] = hm(a[:-1], a[1:])
    north[-1] = a[-1]
    south = np.empty_like(a)
    south[1:] = hm(a[1:], a[:-1])
    south[0] = a[0]
    idx = np.arange(n * n).reshape(n, n)
    rows = [idx.ravel(), idx[:, :-1].ravel(), idx[:, 1:].ravel(), idx[:-1].ravel(), idx[1:].ravel()]
    cols = [idx.ravel(), idx[:, 1:].ravel(), idx[:, :-1].ravel(), idx[1:].ravel(), idx[:-1].ravel()]
    vals = [(east + west + north + south).ravel(), -east[:, :-1].ravel(), -west[:, 1:].ravel(),
            -north[:-1].ravel(), -south[1:].ravel()]
    return sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                             shape=(n * n, n * n))


def direct_solve(a: np.ndarray, f=1.0) -> np.ndarray:
    from scipy.sparse.linalg import spsolve

    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    h2 = (1.0 / (n + 1)) ** 2
    rhs = np.full(n * n, float(f)) if np.isscalar(f) else np.asarray(f, dtype=np.float64).ravel()
    return np.asarray(spsolve(assemble(a), rhs * h2)).reshape(n, n)
