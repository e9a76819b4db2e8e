"""Run one benchmark workload a few times, for a profiler to watch.

    python -m darcy_cpp_gb300.profile_run solve --n 1024 --form mixed --reps 2
    python -m darcy_cpp_gb300.profile_run batch --n 64 --count 304 --form mixed
    python -m darcy_cpp_gb300.profile_run net --side 64 --count 256
    python -m darcy_cpp_gb300.profile_run kernels --n 1024 --form mixed --reps 3

`solve` is the 1024 x 1024 headline workload (two-phase field of seed 1,
a in {1e3, 1e-3}; other sizes use seed 0 and {12, 3}); `batch` is the 64 x 64
batched solve; `net` runs the warm-start network (a few training steps on
solver-generated pairs, then one prediction); `kernels` times each finest-
level kernel and the tail product back to back (dgpu_profile_kernels), each
launched directly on the stream (DARCY_GPU_PROFILE_DIRECT=1) so that a kernel
profiler sees the kernels that can end the CG loop too. The CUDA-graph while loop of the
single solve cannot be replayed by a kernel profiler, so `solve` runs with the
host-driven loop (DARCY_GPU_LOOP=host) unless --device-loop is given.
"""

from __future__ import annotations

import argparse
import os
import sys
import time


def main(argv: list[str] | None = None) -> int:
    p = argparse.ArgumentParser(prog="python -m darcy_cpp_gb300.profile_run")
    p.add_argument("workload", choices=["solve", "batch", "net", "kernels"])
    p.add_argument("--n", type=int, default=1024)
    p.add_argument("--form", default="mixed", choices=["fp64", "mixed"])
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--count", type=int, default=304)
    p.add_argument("--side", type=int, default=64)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--device-loop", action="store_true")
    args = p.parse_args(argv)
    if args.workload in ("solve", "kernels") and not args.device_loop:
        os.environ.setdefault("DARCY_GPU_LOOP", "host")
    if args.workload == "kernels":
        os.environ.setdefault("DARCY_GPU_PROFILE_DIRECT", "1")

    import numpy as np

    import darcy_cpp_gb300 as darcy

    if args.workload == "solve":
        big = args.n >= 1024
        a = darcy.two_phase_permeability(darcy.gaussian_random_field(args.n, seed=1 if big else 0),
                                         *((1e3, 1e-3) if big else (12.0, 3.0)))
        for _ in range(args.reps):
            r = darcy.solve(a, form=args.form)
        print(f"solve n={args.n} form={args.form}: {r.iterations} iterations, converged {r.converged}")
    elif args.workload == "kernels":
        from .capi import Context

        big = args.n >= 1024
        a = darcy.two_phase_permeability(darcy.gaussian_random_field(args.n, seed=1 if big else 0),
                                         *((1e3, 1e-3) if big else (12.0, 3.0)))
        rows = Context().profile_kernels(a, reps=args.reps, form=args.form)
        for row in rows:
            print(f"{row['name']:24s} {row['avg_ms'] * 1e3:9.2f} us  {row['bytes'] / 1e6:9.2f} MB  "
                  f"x{row['launches_per_iteration']:g} per iteration")
    elif args.workload == "batch":
        b = np.stack([darcy.two_phase_permeability(darcy.gaussian_random_field(args.n, seed=s))
                      for s in range(args.count)])
        for _ in range(args.reps):
            t0 = time.perf_counter()
            r = darcy.solve_batch(b, form=args.form)
            dt = time.perf_counter() - t0
        print(f"batch {args.count} x {args.n}^2 form={args.form}: {args.count / dt:.0f} solves/s, "
              f"mean {r.iterations.mean():.1f} iterations")
    else:
        from . import learn

        a, u = learn.generate_pairs(range(args.count), args.side)
        net = learn.WarmStartNet(args.side)
        losses = net.fit(a, u, steps=args.steps, batch=min(256, args.count))
        u0 = net.predict(a)
        print(f"net side={args.side}: {args.steps} steps, loss {losses[-1]:.4g}, predicted {u0.shape}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
