"""Learned warm start for the batched solve.

A 6-layer 3x3 convolutional network (2 -> 32 x 5 -> 1 channels, GELU, BF16
weights and activations with FP32 accumulation) predicts the initial iterate
u0 of PCG from (log a, f); f enters as f times the grid's constant-coefficient
solution (its global shape, which a 13 x 13 receptive field cannot see), and
training minimises the error in the energy norm that CG itself minimises. It is trained on the GPU by the library's own
kernels (tensor-core implicit-GEMM convolutions, CUDA-core weight gradients,
Adam; include/darcy_gpu.h ``dgpu_net_*``) on (a, u) pairs that the GPU solver
itself produced. The solve that follows always runs to the requested
tolerance: the network only changes where PCG starts, never what it accepts.

The reference has no learned component (it always starts from u0 = 0,
include/darcy/solver.hpp:96-102); its ``darcy dataset`` command
(python/darcy/cli.py:77-115) is the data source this module reproduces on the
GPU (``darcy_cpp_gb300.dataset``).
"""

from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

import numpy as np

from . import capi
from .fields import gaussian_random_field, two_phase_permeability

__all__ = ["WarmStartNet", "generate_pairs", "solve_batch_learned", "LearnedBatchResult", "PAPER_CONFIG"]

# Training recipe of the 64 x 64 warm-start workload: 20000 solver-generated
# pairs from seeds 10000..29999, Adam with lr 1e-3, batch 256.
PAPER_CONFIG = {"side": 64, "train_seeds": (10000, 30000), "eval_seeds": (30000, 32000), "batch": 256,
                "lr": 1e-3, "hi": 12.0, "lo": 3.0, "f": 1.0}

_CTX: capi.Context | None = None


def _context() -> capi.Context:
    global _CTX
    if _CTX is None:
        _CTX = capi.Context()
    return _CTX


def permeability_fields(seeds: Sequence[int], side: int, hi: float = 12.0, lo: float = 3.0, alpha: float = 2.0,
                        tau: float = 3.0) -> np.ndarray:
    """Two-phase fields, one per seed (python/darcy/fields.py:31-83 construction)."""
    out = np.empty((len(seeds), side, side))
    for q, s in enumerate(seeds):
        out[q] = two_phase_permeability(gaussian_random_field(side, alpha=alpha, tau=tau, seed=int(s)), hi, lo)
    return out


def generate_pairs(seeds: Sequence[int], side: int, hi: float = 12.0, lo: float = 3.0, f: float = 1.0,
                   tol: float = 1e-10, form: str = "fp64", chunk: int = 8192) -> tuple[np.ndarray, np.ndarray]:
    """(a, u) training pairs: fields from `seeds`, solved on the GPU to `tol`.

    Raises RuntimeError if any solve did not converge (the reference's dataset
    command fails the same way, cli.py:97-100).
    """
    a = permeability_fields(seeds, side, hi, lo)
    u = np.empty_like(a)
    ctx = _context()
    for at in range(0, len(seeds), chunk):
        r = ctx.solve_batch(a[at:at + chunk], f, tol=tol, form=form)
        if not r["converged"].all():
            bad = int((~r["converged"]).sum())
            raise RuntimeError(f"{bad}/{len(r['converged'])} training solves did not converge")
        u[at:at + chunk] = r["u"]
    return a, u


class WarmStartNet:
    """The warm-start network for one grid side."""

    def __init__(self, side: int, seed: int = 0) -> None:
        self._net = capi.Net(side, seed)
        self.side = int(side)

    # -- parameters -------------------------------------------------------
    @property
    def num_params(self) -> int:
        return self._net.num_params

    def params(self) -> np.ndarray:
        return self._net.get_params()

    def set_params(self, w: np.ndarray) -> None:
        self._net.set_params(w)

    def scaling(self) -> np.ndarray:
        """[mean of log a, std of log a, RMS of u at f = fref, fref]."""
        return self._net.get_scaling()

    def set_scaling(self, s) -> None:
        self._net.set_scaling(s)

    def set_loss(self, kind: str) -> None:
        """'energy' (default: e^T A e / u^T A u per sample) or 'mse'."""
        self._net.set_loss(kind)

    def set_engine(self, engine: str) -> None:
        """'tensor' (default) or 'simt' (the CUDA-core cross-check)."""
        self._net.set_engine(engine)

    @property
    def handle(self) -> capi.Net:
        return self._net

    # -- training ---------------------------------------------------------
    def fit(self, a, u, f=None, steps: int | None = None, epochs: float = 1.0, batch: int = 256, lr: float = 1e-3,
            seed: int = 0) -> np.ndarray:
        """Loads (a, u) onto the GPU and runs Adam; returns the per-step losses."""
        a = np.asarray(a)
        self._net.load_pairs(a, u, f)
        count = a.shape[0]
        if steps is None:
            steps = max(1, int(round(epochs * count / batch)))
        return self._net.train(steps, batch=min(batch, count), lr=lr, seed=seed)

    def train_more(self, steps: int, batch: int = 256, lr: float = 1e-3, seed: int = 1) -> np.ndarray:
        """More Adam steps on the pairs already loaded."""
        return self._net.train(steps, batch=batch, lr=lr, seed=seed)

    def gradients(self, a, u, f=None) -> tuple[np.ndarray, float]:
        """Loss and its gradient for one batch (no update)."""
        return self._net.gradients(a, u, f)

    # -- inference --------------------------------------------------------
    def features(self, a, f=None) -> np.ndarray:
        """The network input (count, side, side, 2) after BF16 rounding."""
        return self._net.features(a, f)

    def predict(self, a, f=None) -> np.ndarray:
        return self._net.predict(a, f)

    def save(self, path: str | Path) -> None:
        """Weights file: FP32 parameters, scaling and side (.npz)."""
        np.savez(path, params=self.params(), scaling=self.scaling(), side=np.int64(self.side),
                 format=np.bytes_(b"darcy-warmstart-v1"))

    @classmethod
    def load(cls, path: str | Path) -> "WarmStartNet":
        with np.load(path) as z:
            if bytes(z["format"]) != b"darcy-warmstart-v1":
                raise ValueError("not a warm-start weights file")
            net = cls(int(z["side"]))
            net.set_params(z["params"])
            net.set_scaling(z["scaling"])
        return net


@dataclass(frozen=True)
class LearnedBatchResult:
    u: np.ndarray
    iterations: np.ndarray
    residuals: np.ndarray
    converged: np.ndarray
    levels: np.ndarray

    @property
    def all_converged(self) -> bool:
        return bool(np.all(self.converged))


def solve_batch_learned(net: WarmStartNet, a, f: float = 1.0, *, tol: float = 1e-10, max_iter: int = 10000,
                        preconditioner: str = "multigrid", pre_sweeps: int = 1, post_sweeps: int = 1,
                        cycle_index: int = 2, form: str = "mixed") -> LearnedBatchResult:
    """solve_batch with the warm start predicted on the GPU (one call, the
    prediction never leaves the device); same tolerance as a zero start."""
    a = np.asarray(a, dtype=np.float64)
    if a.ndim != 3 or a.shape[1] != a.shape[2]:
        raise ValueError("a must have shape (batch, n, n)")
    r = _context().solve_batch_learned(net.handle, a, float(f), tol=tol, max_iter=max_iter,
                                       preconditioner=preconditioner, pre_sweeps=pre_sweeps,
                                       post_sweeps=post_sweeps, cycle_index=cycle_index, form=form)
    return LearnedBatchResult(r["u"], r["iterations"].astype(np.int64), r["residuals"], r["converged"],
                              r["levels"].astype(np.int64))
