"""Benchmark harness with GPU rows (the reference's ``darcy bench``).

Restates python/darcy/benchmark.py:54-144: per grid and preconditioner, the
minimum over repeats of a single solve (the run least polluted by scheduler
noise), CG iterations, levels, and the speed-up and relative error against a
sparse direct factorisation (SciPy, optional), rendered as the same Markdown
table, with the arithmetic form (FP64 / mixed) as an extra column; plus a
batched 64 x 64 row in solves/s. Fields: the reference's generator, seed 0.

    python -m darcy_cpp_gb300.benchmark --grids 64 128 256 512 --repeats 3 [--no-scipy] [--json out.json]
"""

from __future__ import annotations

import argparse
import json
import sys
import time
from collections.abc import Callable, Sequence
from dataclasses import asdict, dataclass
from pathlib import Path
from typing import Any

import numpy as np

__all__ = ["BenchmarkRow", "BatchRow", "format_table", "run_benchmark", "run_batch", "to_json", "main"]


@dataclass
class BenchmarkRow:
    grid: int
    preconditioner: str
    form: str
    seconds: float
    device_ms: float
    iterations: int
    levels: int
    residual: float
    scipy_seconds: float | None = None
    relative_error: float | None = None

    @property
    def speedup(self) -> float | None:
        if self.scipy_seconds is None or self.seconds <= 0:
            return None
        return self.scipy_seconds / self.seconds


@dataclass
class BatchRow:
    grid: int
    count: int
    form: str
    seconds: float
    mean_iterations: float

    @property
    def solves_per_s(self) -> float:
        return self.count / self.seconds


def _time(fn: Callable[[], Any], repeats: int) -> tuple[float, Any]:
    best, result = float("inf"), None
    for _ in range(repeats):
        start = time.perf_counter()
        result = fn()
        best = min(best, time.perf_counter() - start)
    return best, result


def run_benchmark(grids: Sequence[int] = (64, 128, 256, 512),
                  preconditioners: Sequence[str] = ("multigrid", "jacobi"),
                  forms: Sequence[str] = ("fp64", "mixed"), repeats: int = 3, compare_scipy: bool = True,
                  tol: float = 1e-10, seed: int = 0, verbose: bool = True) -> list[BenchmarkRow]:
    """Time single solves across grid sizes, preconditioners and forms."""
    import darcy_cpp_gb300 as darcy

    rows: list[BenchmarkRow] = []
    if verbose:
        print(darcy.gpu_info())
        print()
    for n in grids:
        a = darcy.two_phase_permeability(darcy.gaussian_random_field(n, seed=seed))
        u_ref, scipy_seconds = None, None
        if compare_scipy:
            try:
                from .reference import solve_reference

                scipy_seconds, u_ref = _time(lambda a=a: solve_reference(a), 1)
            except ImportError:
                compare_scipy = False
        for name in preconditioners:
            # the Jacobi baseline needs O(n) iterations on large grids; cap it
            # as the reference does rather than let it dominate the run
            max_iter = 100_000 if name != "multigrid" else 1_000
            for form in forms:
                if name != "multigrid" and form != "fp64":
                    continue  # the mixed form changes only the multigrid cycle
                darcy.solve(a, tol=tol, preconditioner=name, max_iter=max_iter, form=form)  # plan, graph
                seconds, result = _time(lambda a=a, name=name, form=form, max_iter=max_iter: darcy.solve(
                    a, tol=tol, preconditioner=name, max_iter=max_iter, form=form), repeats)
                rel = None
                if u_ref is not None:
                    rel = float(np.linalg.norm(result.u - u_ref) / np.linalg.norm(u_ref))
                row = BenchmarkRow(n, name, form, seconds, float(result.device_ms), result.iterations,
                                   result.levels, result.residual, scipy_seconds, rel)
                rows.append(row)
                if verbose:
                    print(_format_row(row))
    if verbose:
        print()
        print(format_table(rows))
    return rows


def run_batch(grid: int = 64, count: int = 4096, forms: Sequence[str] = ("fp64", "mixed"), repeats: int = 3,
              tol: float = 1e-10, verbose: bool = True) -> list[BatchRow]:
    """Batched solves/s: `count` fields of seeds 0..count-1, one call each."""
    import darcy_cpp_gb300 as darcy

    batch = np.stack([darcy.two_phase_permeability(darcy.gaussian_random_field(grid, seed=s))
                      for s in range(count)])
    rows = []
    for form in forms:
        darcy.solve_batch(batch, tol=tol, form=form)  # tune the launch shape
        seconds, r = _time(lambda form=form: darcy.solve_batch(batch, tol=tol, form=form), repeats)
        rows.append(BatchRow(grid, count, form, seconds, float(r.iterations.mean())))
        if verbose:
            print(f"  batch {count} x {grid}^2 {form:>5}: {count / seconds:10.0f} solves/s, "
                  f"{r.iterations.mean():.1f} mean iterations")
    return rows


def _format_row(row: BenchmarkRow) -> str:
    speedup = f"{row.speedup:.2f}x" if row.speedup is not None else "-"
    err = f"{row.relative_error:.1e}" if row.relative_error is not None else "-"
    return (f"  {row.grid:>5} {row.preconditioner:>10} {row.form:>5}  {row.seconds * 1e3:>9.2f} ms  "
            f"{row.iterations:>6} iters  speedup {speedup:>8}  rel.err {err}")


def format_table(rows: Sequence[BenchmarkRow], batch: Sequence[BatchRow] = ()) -> str:
    """Markdown, the reference's columns plus the form and the device time."""
    header = ("| grid | preconditioner | form | CG iters | levels | time (ms) | device (ms) | "
              "SciPy direct (ms) | speed-up | rel. err |")
    lines = [header, "|" + "|".join(["---"] * 10) + "|"]
    for r in rows:
        scipy_ms = f"{r.scipy_seconds * 1e3:.1f}" if r.scipy_seconds is not None else "-"
        speedup = f"{r.speedup:.2f}x" if r.speedup is not None else "-"
        err = f"{r.relative_error:.1e}" if r.relative_error is not None else "-"
        lines.append(f"| {r.grid} | {r.preconditioner} | {r.form} | {r.iterations} | {r.levels} | "
                     f"{r.seconds * 1e3:.2f} | {r.device_ms:.2f} | {scipy_ms} | {speedup} | {err} |")
    if batch:
        lines += ["", "| batch | form | solves/s | mean CG iters |", "|---|---|---|---|"]
        for b in batch:
            lines.append(f"| {b.count} x {b.grid}² | {b.form} | {b.solves_per_s:.0f} | {b.mean_iterations:.1f} |")
    return "\n".join(lines)


def to_json(rows: Sequence[BenchmarkRow], batch: Sequence[BatchRow] = ()) -> dict[str, Any]:
    return {"single": [asdict(r) | {"speedup": r.speedup} for r in rows],
            "batch": [asdict(b) | {"solves_per_s": b.solves_per_s} for b in batch]}


def main(argv: list[str] | None = None) -> int:
    p = argparse.ArgumentParser(prog="python -m darcy_cpp_gb300.benchmark")
    p.add_argument("--grids", type=int, nargs="+", default=[64, 128, 256, 512])
    p.add_argument("--repeats", type=int, default=3)
    p.add_argument("--no-scipy", action="store_true", help="skip the SciPy direct-solver baseline")
    p.add_argument("--preconditioners", nargs="+", default=["multigrid", "jacobi"],
                   choices=["multigrid", "jacobi", "none"])
    p.add_argument("--batch", type=int, default=4096, help="batched 64 x 64 row size (0 skips it)")
    p.add_argument("--json", type=Path, help="also write the results as JSON")
    args = p.parse_args(argv)
    rows = run_benchmark(args.grids, args.preconditioners, repeats=args.repeats, compare_scipy=not args.no_scipy)
    batch = run_batch(64, args.batch, repeats=args.repeats) if args.batch > 0 else []
    if batch:
        print()
        print(format_table([], batch).strip())
    if args.json:
        args.json.write_text(json.dumps(to_json(rows, batch), indent=2))
    return 0


if __name__ == "__main__":
    sys.exit(main())
