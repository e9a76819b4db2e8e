"""Generate the golden vectors that pin the CPU oracle (run where the reference exists).

Everything here comes from the reference itself:
  * fields from the reference's own generator (python/darcy/fields.py), loaded
    by file path from the checkout;
  * solver outputs from the reference's own C++ headers, compiled by
    oracle/build_ref.py into oracle/_ref/libdarcy_ref.so and run with ONE
    OpenMP thread so reductions have a fixed order.

Output: tests/golden/golden.npz (arrays) and tests/golden/golden.json (scalars).
Usage:  python tests/golden/make_golden.py [--ref PATH]   (default: $DARCY_REFERENCE, else
        the checkout location oracle/build_ref.py names)
"""

from __future__ import annotations

import argparse
import hashlib
import importlib.util
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402


def load_ref_fields(ref: Path):
    spec = importlib.util.spec_from_file_location("ref_fields", ref / "python" / "darcy" / "fields.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def main() -> None:
    ap = argparse.ArgumentParser()
    import os

    from oracle.build_ref import DEFAULT_REF

    ap.add_argument("--ref", type=Path, default=Path(os.environ.get("DARCY_REFERENCE", DEFAULT_REF)))
    args = ap.parse_args()
    if not oracle.have_ref():
        subprocess_rc = __import__("subprocess").run(
            [sys.executable, str(ROOT / "oracle" / "build_ref.py"), "--ref", str(args.ref)]).returncode
        if subprocess_rc or not oracle.have_ref():
            raise SystemExit("oracle/_ref/libdarcy_ref.so could not be built")
    oracle.ref_set_threads(1)
    F = load_ref_fields(args.ref)

    def field(n, seed, hi=12.0, lo=3.0):
        return F.two_phase_permeability(F.gaussian_random_field(n, seed=seed), hi=hi, lo=lo)

    arrays: dict[str, np.ndarray] = {}
    meta: dict = {"fields": {}, "solves": {}, "generator": "reference fields.py + reference headers, 1 thread"}

    # --- field hashes (the generator is numpy+scipy arithmetic, so pin it) ---
    for n, seed, hi, lo in [(64, 0, 12.0, 3.0), (1024, 1, 1e3, 1e-3), (2048, 1, 1e3, 1e-3),
                            (128, 0, 12.0, 3.0), (32, 5, 12.0, 3.0), (128, 3, 1e2, 1e-2),
                            (512, 7, 1e2, 1e-2), (64, 13, 1e6, 1.0)]:
        grf = F.gaussian_random_field(n, seed=seed)
        a = F.two_phase_permeability(grf, hi=hi, lo=lo)
        key = f"n{n}_s{seed}_{hi:g}_{lo:g}"
        meta["fields"][key] = {"n": n, "seed": seed, "hi": hi, "lo": lo, "sha256": sha(a),
                               "grf_sha256": sha(grf), "hi_fraction": float((a == hi).mean())}
        if n <= 128:
            arrays[f"grf_{key}"] = grf
    meta["fields"]["grf_alpha1.5_n16_s3"] = {"sha256": sha(F.gaussian_random_field(16, alpha=1.5, tau=2.0, seed=3))}

    def record(name, a, f=1.0, store_u=False, **kw):
        out = oracle.ref_solve(a, f, **kw)
        u = out["u"]
        meta["solves"][name] = {
            "n": int(a.shape[0]), "kwargs": kw, "iterations": out["iterations"],
            "residual": out["residual"], "converged": out["converged"], "levels": out["levels"],
            "u_sum": float(u.sum()), "u_norm": float(np.linalg.norm(u)), "u_max": float(u.max()),
            "u_mid": float(u[u.shape[0] // 2, u.shape[1] // 2]) if u.size else 0.0,
            "history": [float(h) for h in out["history"]],
        }
        if store_u:
            arrays[f"u_{name}"] = u
        return out

    # cfg1: 64^2 seed 0 {12,3}, f=1, tol 1e-10, default W-cycle
    a64 = field(64, 0)
    arrays["a_cfg1"] = a64
    record("cfg1", a64, store_u=True, tol=1e-10, record_history=True)

    # tiny and odd grids, every preconditioner (reference tests/test_correctness.py:20-33, :153-159)
    for n in (1, 2, 3, 4, 5):
        record(f"tiny{n}", np.full((n, n), 2.0), store_u=True, tol=1e-13)
    for n in (16, 17, 31, 32, 33, 48):
        a = field(n, n)
        for pc in ("multigrid", "jacobi", "none"):
            record(f"n{n}_{pc}", a, store_u=n <= 33, tol=1e-12, max_iter=200_000, preconditioner=pc)
    # cycle / sweep variants
    a = field(48, 4)
    for cyc in (1, 2):
        for sw in (1, 2, 3):
            record(f"n48_c{cyc}_s{sw}", a, store_u=True, tol=1e-10, cycle_index=cyc,
                   pre_sweeps=sw, post_sweeps=sw)
    # variable forcing (test_correctness.py:47-57)
    n = 32
    xs = np.linspace(0, 1, n)
    fvar = np.outer(np.sin(np.pi * xs), 1.0 + xs**2)
    arrays["f_var32"] = fvar
    record("fvar32", field(32, 3), fvar, store_u=True, tol=1e-12)
    # non-convergence (test_api.py:95-106)
    record("maxiter2_128", field(128, 0), store_u=False, tol=1e-14, max_iter=2)
    # 1e6 contrast at 64^2 (test_correctness.py:162-170)
    record("contrast1e6_64", field(64, 13, 1e6, 1.0), store_u=True, tol=1e-10, max_iter=2000)
    # iteration table seed 0 {12,3} (the reference's README.md:72-76)
    for n in (128, 256, 512):
        record(f"table{n}", field(n, 0), tol=1e-10)
    # cfg2 at 1024^2 seed 1, 1e6 contrast
    record("cfg2_1024", field(1024, 1, 1e3, 1e-3), tol=1e-10)
    # cfg5 sizes
    record("cfg5_128_s3", field(128, 3, 1e2, 1e-2), tol=1e-10)

    # operator / preconditioner / level kernels on fixed inputs
    rng = np.random.default_rng(20240724)
    a17 = field(17, 11)
    x17 = rng.standard_normal((17, 17))
    arrays["a_op17"], arrays["x_op17"] = a17, x17
    arrays["y_op17"] = oracle.ref_apply_operator(a17, x17)
    a32 = field(32, 8)
    r32 = rng.standard_normal((32, 32))
    arrays["a_pc32"], arrays["r_pc32"] = a32, r32
    for cyc in (1, 2):
        for sw in (1, 2, 3):
            arrays[f"z_pc32_c{cyc}_s{sw}"] = oracle.ref_apply_preconditioner(
                a32, r32, pre_sweeps=sw, post_sweeps=sw, cycle_index=cyc)
    a33 = field(33, 2)
    r33 = rng.standard_normal((33, 33))
    arrays["a_pc33"], arrays["r_pc33"] = a33, r33
    arrays["z_pc33"] = oracle.ref_apply_preconditioner(a33, r33)
    # hierarchy (level.hpp:79-97, :171-211) at an odd size with random phases
    a13 = np.where(rng.random((13, 13)) < 0.5, 3.0, 12.0)
    arrays["a_h13"] = a13
    for lvl, L in enumerate(oracle.ref_hierarchy(a13)):
        for k in ("e", "w", "n", "s", "diag", "inv_diag"):
            arrays[f"h13_l{lvl}_{k}"] = L[k]

    # batch (test_api.py:109-116)
    batch_a = np.stack([field(32, s) for s in range(6)])
    arrays["batch_a32"] = batch_a
    meta["batch32_iterations"] = [int(oracle.ref_solve(x, tol=1e-12)["iterations"]) for x in batch_a]

    out = Path(__file__).resolve().parent
    np.savez_compressed(out / "golden.npz", **arrays)
    (out / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True))
    print("wrote", out / "golden.npz", "and golden.json;",
          {k: meta["solves"][k]["iterations"] for k in ("cfg1", "cfg2_1024", "table512")})


if __name__ == "__main__":
    main()
