"""``darcy dataset`` on the GPU: (a, u) training pairs for neural operators.

Restates the reference's dataset command (python/darcy/cli.py:77-115, defaults
:161-170): B two-phase fields drawn serially from ONE shared random stream
``default_rng(seed)`` (:79-84), all solved together through the batched solve
(:87-94, here the GPU batched engine), failure if any sample did not converge
(:97-100), and ``npz(a, u)`` written with ``savez_compressed`` in float32 by
default (:103-107). The same seed gives the same fields as the reference.

    python -m darcy_cpp_gb300.dataset --n-samples 1000 --grid 64 --output data/darcy_train.npz
"""

from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

from .fields import gaussian_random_field, two_phase_permeability

__all__ = ["draw_fields", "draw_fields_gpu", "generate", "main"]


def draw_fields(n_samples: int, grid: int, seed: int = 0, alpha: float = 2.0, tau: float = 3.0) -> np.ndarray:
    """The reference's field loop (cli.py:79-84): one generator for all samples."""
    rng = np.random.default_rng(seed)
    a = np.empty((n_samples, grid, grid), dtype=np.float64)
    for i in range(n_samples):
        a[i] = two_phase_permeability(gaussian_random_field(grid, alpha=alpha, tau=tau, seed=rng))
    return a


def draw_fields_gpu(n_samples: int, grid: int, seed: int = 0, alpha: float = 2.0, tau: float = 3.0,
                    hi: float = 12.0, lo: float = 3.0) -> np.ndarray:
    """The same construction generated on the GPU (grid <= 128): same
    distribution as draw_fields, a different random stream."""
    from .capi import random_fields

    return random_fields(grid, n_samples, seed, alpha, tau, hi, lo)


def generate(n_samples: int = 1000, grid: int = 64, seed: int = 0, alpha: float = 2.0, tau: float = 3.0,
             f: float = 1.0, tol: float = 1e-10, max_iter: int = 10000, preconditioner: str = "multigrid",
             form: str = "fp64", dtype: str = "float32", output: str | Path | None = None,
             gpu_fields: bool = False) -> dict:
    """Draws the fields, solves them on the GPU and (optionally) writes the npz.

    gpu_fields draws the fields on the GPU as well (not the reference's
    random stream). Returns a dict with a, u (float64), iterations and the
    solve time.
    """
    from . import solve_batch

    if gpu_fields:
        a = draw_fields_gpu(n_samples, grid, seed, alpha, tau)
    else:
        a = draw_fields(n_samples, grid, seed, alpha, tau)
    t0 = time.perf_counter()
    batch = solve_batch(a, f, tol=tol, max_iter=max_iter, preconditioner=preconditioner, form=form)
    elapsed = time.perf_counter() - t0
    if not batch.all_converged:
        failed = int((~batch.converged).sum())
        raise RuntimeError(f"{failed}/{n_samples} samples did not converge")
    if output is not None:
        out = Path(output)
        out.parent.mkdir(parents=True, exist_ok=True)
        np.savez_compressed(out, a=a.astype(dtype), u=batch.u.astype(dtype))
    return {"a": a, "u": batch.u, "iterations": batch.iterations, "seconds": elapsed}


def main(argv: list[str] | None = None) -> int:
    p = argparse.ArgumentParser(prog="python -m darcy_cpp_gb300.dataset",
                                description="generate a training dataset on the GPU")
    p.add_argument("--n-samples", type=int, default=1000)
    p.add_argument("--grid", type=int, default=64)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--alpha", type=float, default=2.0)
    p.add_argument("--tau", type=float, default=3.0)
    p.add_argument("--f", type=float, default=1.0)
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--max-iter", type=int, default=10_000)
    p.add_argument("--preconditioner", default="multigrid", choices=["none", "jacobi", "multigrid"])
    p.add_argument("--form", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--dtype", default="float32", choices=["float32", "float64"])
    p.add_argument("--output", type=Path, default=Path("data/darcy_train.npz"))
    p.add_argument("--gpu-fields", action="store_true",
                   help="draw the fields on the GPU too (same distribution, not the reference's random stream)")
    args = p.parse_args(argv)
    try:
        r = generate(args.n_samples, args.grid, args.seed, args.alpha, args.tau, args.f, args.tol, args.max_iter,
                     args.preconditioner, args.form, args.dtype, args.output, gpu_fields=args.gpu_fields)
    except RuntimeError as e:
        print(f"error: {e}", file=sys.stderr)
        return 1
    per = r["seconds"] / args.n_samples
    print(f"wrote {args.output}: {args.n_samples} samples at {args.grid}x{args.grid}")
    print(f"  {r['seconds']:.2f} s total, {per * 1e3:.3f} ms/sample, "
          f"{np.mean(r['iterations']):.1f} mean CG iterations")
    return 0


if __name__ == "__main__":
    sys.exit(main())
