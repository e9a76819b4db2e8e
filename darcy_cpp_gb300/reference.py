"""SciPy direct solve of the same discretisation (independent check).

Restates the reference's python/darcy/reference.py:29-85 construction: the
finite-volume operator (harmonic faces, the cell's own permeability on
boundary faces, level.hpp:79-97) assembled as an explicit CSR matrix and
factorised with spsolve, so agreement with the matrix-free multigrid path is
evidence from a different algorithm and representation. SciPy is optional.
"""

from __future__ import annotations

import numpy as np

__all__ = ["assemble_matrix", "solve_reference"]


def _harmonic(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    return 2.0 * x * y / (x + y)


def assemble_matrix(a: np.ndarray):
    """The (n*n, n*n) CSR operator for permeability ``a``."""
    from scipy import sparse

    a = np.asarray(a, dtype=np.float64)
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise ValueError("a must be a square 2-D array")
    n = a.shape[0]
    east = np.empty_like(a)
    east[:, :-1] = _harmonic(a[:, :-1], a[:, 1:])
    east[:, -1] = a[:, -1]
    west = np.empty_like(a)
    west[:, 1:] = _harmonic(a[:, 1:], a[:, :-1])
    west[:, 0] = a[:, 0]
    north = np.empty_like(a)
    north[:-1] = _harmonic(a[:-1], a[1:])
    north[-1] = a[-1]
    south = np.empty_like(a)
    south[1:] = _harmonic(a[1:], a[:-1])
    south[0] = a[0]
    idx = np.arange(n * n).reshape(n, n)
    rows = [idx.ravel(), idx[:, :-1].ravel(), idx[:, 1:].ravel(), idx[:-1].ravel(), idx[1:].ravel()]
    cols = [idx.ravel(), idx[:, 1:].ravel(), idx[:, :-1].ravel(), idx[1:].ravel(), idx[:-1].ravel()]
    vals = [(east + west + north + south).ravel(), -east[:, :-1].ravel(), -west[:, 1:].ravel(),
            -north[:-1].ravel(), -south[1:].ravel()]
    return sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                             shape=(n * n, n * n))


def solve_reference(a: np.ndarray, f=1.0) -> np.ndarray:
    """u with A u = f h^2, h = 1 / (n + 1), by a sparse direct factorisation."""
    from scipy.sparse.linalg import spsolve

    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    h2 = (1.0 / (n + 1)) ** 2
    rhs = np.full(n * n, float(f)) if np.isscalar(f) else np.asarray(f, dtype=np.float64).ravel()
    return np.asarray(spsolve(assemble_matrix(a), rhs * h2)).reshape(n, n)
