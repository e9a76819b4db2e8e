"""GB300-native engine for the darcy MG-PCG solve path.

Drop-in for the reference package's solve path (darcy-cpp v1.0.0,
python/darcy/__init__.py): the same functions, keyword arguments, defaults,
result dataclasses and ValueError behaviour, with the compute in hand-written
sm_103a CUDA kernels behind the C ABI of ``libdarcy_gpu.so``
(include/darcy_gpu.h). There is no CPU fallback: if the native extension is
missing, importing this package fails.

Additive extensions (the reference calls keep their meaning):
  * ``form="mixed"``: FP32 multigrid cycle inside FP64 CG;
  * ``x0=``: warm start for PCG (same stopping test);
  * :func:`solve_batch_uneven`: many problems of different sizes, one launch;
  * :func:`gpu_info`: device details (``build_info`` keeps its five keys).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Literal, Sequence

import numpy as np

try:
    from . import _core
except ImportError as exc:  # no fallback: the GPU engine is the product
    raise ImportError(
        "darcy_cpp_gb300: the native extension is not built (run `python darcy_cpp_gb300/build.py`); "
        f"original error: {exc}"
    ) from exc

from .fields import gaussian_random_field, two_phase_permeability

__all__ = [
    "BatchResult",
    "SolveResult",
    "UnevenBatchResult",
    "__version__",
    "apply_operator",
    "apply_preconditioner",
    "build_info",
    "gaussian_random_field",
    "gpu_info",
    "has_openmp",
    "num_threads",
    "set_num_threads",
    "solve",
    "solve_batch",
    "solve_batch_uneven",
    "two_phase_permeability",
]

__version__: str = _core.__version__

Preconditioner = Literal["multigrid", "jacobi", "none"]
Form = Literal["fp64", "mixed"]

_DEFAULT_TOL = 1e-10  # python/darcy/__init__.py:60


@dataclass(frozen=True)
class SolveResult:
    """Outcome of one solve (fields as python/darcy/__init__.py:63-95).

    ``true_residual`` (||b - A u|| / ||b|| recomputed on the GPU) and
    ``device_ms`` are additions; the first six fields are the reference's.
    """

    u: np.ndarray
    iterations: int
    residual: float
    converged: bool
    levels: int
    history: np.ndarray = field(default_factory=lambda: np.empty(0))
    true_residual: float = float("nan")
    device_ms: float = float("nan")

    def __repr__(self) -> str:
        return (
            f"SolveResult(shape={self.u.shape}, iterations={self.iterations}, "
            f"residual={self.residual:.3e}, converged={self.converged}, levels={self.levels})"
        )


@dataclass(frozen=True)
class BatchResult:
    """Outcome of a batched solve (python/darcy/__init__.py:98-116)."""

    u: np.ndarray
    iterations: np.ndarray
    residuals: np.ndarray
    converged: np.ndarray

    @property
    def all_converged(self) -> bool:
        return bool(self.converged.all())

    def __repr__(self) -> str:
        return (
            f"BatchResult(batch={self.u.shape[0]}, shape={self.u.shape[1:]}, "
            f"mean_iterations={self.iterations.mean():.1f}, all_converged={self.all_converged})"
        )


@dataclass(frozen=True)
class UnevenBatchResult:
    """Outcome of :func:`solve_batch_uneven`: per-problem arrays of their own size."""

    u: list
    iterations: np.ndarray
    residuals: np.ndarray
    converged: np.ndarray
    levels: np.ndarray

    @property
    def all_converged(self) -> bool:
        return bool(self.converged.all())

    def __repr__(self) -> str:
        sides = sorted({x.shape[0] for x in self.u})
        return (
            f"UnevenBatchResult(batch={len(self.u)}, sides={sides}, "
            f"mean_iterations={self.iterations.mean():.1f}, all_converged={self.all_converged})"
        )


def solve(
    a: Any,
    f: float | Any = 1.0,
    *,
    tol: float = _DEFAULT_TOL,
    max_iter: int = 10_000,
    preconditioner: Preconditioner = "multigrid",
    pre_sweeps: int = 1,
    post_sweeps: int = 1,
    cycle_index: int = 2,
    record_history: bool = False,
    form: Form = "fp64",
    x0: Any = None,
) -> SolveResult:
    """Solve ``-div(a grad u) = f`` with u = 0 on the boundary, on the GPU.

    Arguments and errors as the reference's ``darcy.solve``
    (python/darcy/__init__.py:119-183). ``form="mixed"`` runs the multigrid
    cycle in FP32 (CG, dots and the residual stay FP64); ``x0`` starts PCG
    from a given field instead of zero.
    """
    raw = _core.solve(
        a, f, tol=tol, max_iter=max_iter, preconditioner=preconditioner, pre_sweeps=pre_sweeps,
        post_sweeps=post_sweeps, cycle_index=cycle_index, record_history=record_history, form=form, x0=x0,
    )
    return SolveResult(
        u=raw.u, iterations=raw.iterations, residual=raw.residual, converged=raw.converged, levels=raw.levels,
        history=np.asarray(raw.history, dtype=np.float64), true_residual=raw.true_residual,
        device_ms=raw.device_ms,
    )


def solve_batch(
    a: Any,
    f: float | Any = 1.0,
    *,
    tol: float = _DEFAULT_TOL,
    max_iter: int = 10_000,
    preconditioner: Preconditioner = "multigrid",
    pre_sweeps: int = 1,
    post_sweeps: int = 1,
    cycle_index: int = 2,
    threads: int = 0,
    form: Form = "fp64",
    x0: Any = None,
) -> BatchResult:
    """Solve a (batch, n, n) stack of independent problems in one GPU launch.

    As python/darcy/__init__.py:186-223; ``threads`` is accepted and ignored
    (the GPU schedules the samples).
    """
    u, iters, residuals, converged = _core.solve_batch(
        a, f, tol=tol, max_iter=max_iter, preconditioner=preconditioner, pre_sweeps=pre_sweeps,
        post_sweeps=post_sweeps, cycle_index=cycle_index, threads=threads, form=form, x0=x0,
    )
    return BatchResult(
        u=u,
        iterations=np.asarray(iters, dtype=np.int64),
        residuals=np.asarray(residuals, dtype=np.float64),
        converged=np.asarray(converged, dtype=bool),
    )


def solve_batch_uneven(
    fields: Sequence[Any],
    f: float | Sequence[Any] = 1.0,
    *,
    tol: float = _DEFAULT_TOL,
    max_iter: int = 10_000,
    preconditioner: Preconditioner = "multigrid",
    pre_sweeps: int = 1,
    post_sweeps: int = 1,
    cycle_index: int = 2,
    form: Form = "fp64",
    x0: Sequence[Any] | None = None,
) -> UnevenBatchResult:
    """Solve problems of different grid sizes together (one GPU launch).

    ``f`` is a scalar for all problems or one scalar/array per problem. The
    solutions ``u`` are views into one array (disjoint, writeable, C-ordered),
    which stays alive while any of them does.
    """
    fl = list(fields)
    fa: Any = f
    if isinstance(f, (list, tuple)):
        fa = [float(v) * np.ones_like(np.asarray(fl[q], dtype=np.float64)) if np.isscalar(v) else v
              for q, v in enumerate(f)]
    us, iters, residuals, converged, levels = _core.solve_batch_uneven(
        fl, fa, tol=tol, max_iter=max_iter, preconditioner=preconditioner, pre_sweeps=pre_sweeps,
        post_sweeps=post_sweeps, cycle_index=cycle_index, form=form,
        x0=None if x0 is None else list(x0),
    )
    return UnevenBatchResult(
        u=list(us),
        iterations=np.asarray(iters, dtype=np.int64),
        residuals=np.asarray(residuals, dtype=np.float64),
        converged=np.asarray(converged, dtype=bool),
        levels=np.asarray(levels, dtype=np.int64),
    )


def apply_operator(a: Any, x: Any) -> np.ndarray:
    """y = A x with the finite-volume operator, on the GPU (reference test hook)."""
    return _core.apply_operator(a, x)


def apply_preconditioner(
    a: Any, r: Any, *, pre_sweeps: int = 1, post_sweeps: int = 1, cycle_index: int = 2, form: Form = "fp64"
) -> np.ndarray:
    """One multigrid cycle from zero, z = M r, on the GPU (reference test hook)."""
    return _core.apply_preconditioner(a, r, pre_sweeps=pre_sweeps, post_sweeps=post_sweeps,
                                      cycle_index=cycle_index, form=form)


def num_threads() -> int:
    """Host threads the solver uses (1: the work is on the GPU)."""
    return _core.num_threads()


def set_num_threads(threads: int) -> None:
    """Accepted for compatibility with the reference; has no effect."""
    _core.set_num_threads(threads)


def has_openmp() -> bool:
    """False: the engine does not use host OpenMP."""
    return _core.has_openmp()


def build_info() -> dict[str, Any]:
    """Version and build details; exactly the reference's five keys."""
    return {
        "version": __version__,
        "compiler": _core.__compiler__,
        "openmp": has_openmp(),
        "max_threads": num_threads(),
        "numpy": np.__version__,
    }


def gpu_info() -> str:
    """Device name, SM count, memory and the CG loop mode in use."""
    return _core.gpu_info()
