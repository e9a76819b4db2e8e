"""CPU oracle for the darcy MG-PCG path -- test infrastructure only.

`oracle/darcy_oracle.c` restates the reference solver (darcy-cpp v1.0.0,
include/darcy/*.hpp, src/bindings.cpp) in plain C with the same loop order and
OpenMP structure. This module loads it through ctypes. Only the tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import it; the GPU
package never does.

When ``oracle/_ref/libdarcy_ref.so`` exists (built by ``oracle/build_ref.py``
from the reference's own headers, only possible where the reference checkout
is present) the ``ref_*`` helpers run the reference itself.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_PATH = HERE / "_ref" / "libdarcy_ref.so"

PRECONDITIONERS = {"none": 0, "jacobi": 1, "multigrid": 2, "mg": 2}

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int_p = ctypes.POINTER(ctypes.c_int)


class _Options(ctypes.Structure):
    _fields_ = [
        ("tol", ctypes.c_double),
        ("max_iter", ctypes.c_int),
        ("preconditioner", ctypes.c_int),
        ("pre_sweeps", ctypes.c_int),
        ("post_sweeps", ctypes.c_int),
        ("cycle_index", ctypes.c_int),
        ("record_history", ctypes.c_int),
    ]


class _Result(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("residual", ctypes.c_double),
        ("converged", ctypes.c_int),
        ("levels", ctypes.c_int),
        ("history_len", ctypes.c_int),
    ]


class OracleError(ValueError):
    pass


def build() -> Path:
    """Compile liboracle.so with the Makefile beside this file."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        _lib = ctypes.CDLL(str(LIB_PATH))
    return _lib


def _dp(arr: np.ndarray):
    return arr.ctypes.data_as(_c_double_p)


def _f64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


def _rhs(f, n: int) -> np.ndarray:
    if np.isscalar(f):
        return np.full((n, n), float(f))
    arr = _f64(f)
    if arr.shape != (n, n):
        raise OracleError("f must be a scalar or an array with the same shape as a")
    return arr


def _opts(tol, max_iter, preconditioner, pre_sweeps, post_sweeps, cycle_index, record_history):
    return _Options(
        float(tol), int(max_iter), PRECONDITIONERS[preconditioner], int(pre_sweeps), int(post_sweeps),
        int(cycle_index), int(bool(record_history)),
    )


def solve(a, f=1.0, *, tol=1e-10, max_iter=10000, preconditioner="multigrid", pre_sweeps=1,
          post_sweeps=1, cycle_index=2, record_history=False, u0=None) -> dict:
    """darcy::solve (solver.hpp:83-174) on the CPU; optional warm start u0."""
    a = _f64(a)
    n = a.shape[0]
    rhs = _rhs(f, n)
    u = np.empty((n, n))
    hist = np.empty(max_iter + 2) if record_history else None
    res = _Result()
    err = ctypes.create_string_buffer(256)
    o = _opts(tol, max_iter, preconditioner, pre_sweeps, post_sweeps, cycle_index, record_history)
    if u0 is None:
        rc = lib().oracle_solve(_dp(a), _dp(rhs), ctypes.c_int64(n), ctypes.byref(o), _dp(u),
                                _dp(hist) if hist is not None else None, ctypes.byref(res), err, 256)
    else:
        u0 = _f64(u0)
        rc = lib().oracle_solve_x0(_dp(a), _dp(rhs), _dp(u0), ctypes.c_int64(n), ctypes.byref(o),
                                   _dp(u), ctypes.byref(res), err, 256)
    if rc != 0:
        raise OracleError(err.value.decode())
    return {
        "u": u,
        "iterations": res.iterations,
        "residual": res.residual,
        "converged": bool(res.converged),
        "levels": res.levels,
        "history": hist[: res.history_len].copy() if hist is not None else np.empty(0),
    }


def solve_batch(a, f=1.0, *, tol=1e-10, max_iter=10000, preconditioner="multigrid", pre_sweeps=1,
                post_sweeps=1, cycle_index=2, threads=0) -> dict:
    """_core.solve_batch (bindings.cpp:140-197): OpenMP over samples."""
    a = _f64(a)
    batch, n = a.shape[0], a.shape[1]
    rhs = _rhs(f, n)
    u = np.empty_like(a)
    iters = np.zeros(batch, dtype=np.int32)
    res = np.zeros(batch)
    conv = np.zeros(batch, dtype=np.int32)
    err = ctypes.create_string_buffer(256)
    o = _opts(tol, max_iter, preconditioner, pre_sweeps, post_sweeps, cycle_index, False)
    rc = lib().oracle_solve_batch(_dp(a), _dp(rhs), ctypes.c_int64(batch), ctypes.c_int64(n),
                                  ctypes.byref(o), int(threads), _dp(u), iters.ctypes.data_as(_c_int_p),
                                  _dp(res), conv.ctypes.data_as(_c_int_p), err, 256)
    if rc != 0:
        raise OracleError(err.value.decode())
    return {"u": u, "iterations": iters.astype(np.int64), "residuals": res, "converged": conv.astype(bool)}


def apply_operator(a, x) -> np.ndarray:
    a, x = _f64(a), _f64(x)
    y = np.empty_like(x)
    err = ctypes.create_string_buffer(256)
    if lib().oracle_apply_operator(_dp(a), _dp(x), ctypes.c_int64(a.shape[0]), _dp(y), err, 256):
        raise OracleError(err.value.decode())
    return y


def apply_preconditioner(a, r, *, pre_sweeps=1, post_sweeps=1, cycle_index=2) -> np.ndarray:
    a, r = _f64(a), _f64(r)
    z = np.empty_like(r)
    err = ctypes.create_string_buffer(256)
    if lib().oracle_apply_preconditioner(_dp(a), _dp(r), ctypes.c_int64(a.shape[0]), int(pre_sweeps),
                                         int(post_sweeps), int(cycle_index), _dp(z), err, 256):
        raise OracleError(err.value.decode())
    return z


def num_levels(n: int) -> int:
    return int(lib().oracle_num_levels(ctypes.c_int64(n)))


def level_sides(n: int) -> list[int]:
    sides = [n]
    while sides[-1] > 1 and len(sides) < 32:
        sides.append((sides[-1] + 1) // 2)
    return sides


def _split_hierarchy(buf: np.ndarray, n: int) -> list[dict]:
    out, off = [], 0
    for side in level_sides(n):
        m = side * side
        chunk = buf[off: off + 6 * m].reshape(6, side, side)
        out.append(dict(zip(("e", "w", "n", "s", "diag", "inv_diag"), chunk)))
        off += 6 * m
    return out


def hierarchy(a) -> list[dict]:
    """Every level's e, w, n, s, diag, inv_diag (level.hpp:79-97, :171-211)."""
    a = _f64(a)
    n = a.shape[0]
    cap = sum(6 * s * s for s in level_sides(n))
    buf = np.empty(cap)
    got = lib().oracle_hierarchy(_dp(a), ctypes.c_int64(n), _dp(buf), ctypes.c_int64(cap))
    if got != cap:
        raise OracleError("hierarchy dump failed")
    return _split_hierarchy(buf, n)


def level_gs(a, x, b, colour: int) -> np.ndarray:
    a, b = _f64(a), _f64(b)
    x = _f64(x).copy()
    lib().oracle_level_gs(_dp(a), ctypes.c_int64(a.shape[0]), _dp(x), _dp(b), int(colour))
    return x


def level_residual(a, x, b) -> np.ndarray:
    a, x, b = _f64(a), _f64(x), _f64(b)
    r = np.empty_like(x)
    lib().oracle_level_residual(_dp(a), ctypes.c_int64(a.shape[0]), _dp(x), _dp(b), _dp(r))
    return r


def level_restrict(fine) -> np.ndarray:
    fine = _f64(fine)
    n = fine.shape[0]
    nc = (n + 1) // 2
    coarse = np.empty((nc, nc))
    lib().oracle_level_restrict(ctypes.c_int64(n), _dp(fine), _dp(coarse))
    return coarse


def level_prolong_add(coarse, fine) -> np.ndarray:
    coarse = _f64(coarse)
    fine = _f64(fine).copy()
    lib().oracle_level_prolong_add(ctypes.c_int64(fine.shape[0]), _dp(coarse), _dp(fine))
    return fine


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def set_threads(t: int) -> None:
    lib().oracle_set_threads(int(t))


# ---------------------------------------------------------------- reference


_ref = None


def have_ref() -> bool:
    return REF_PATH.exists()


def ref_lib() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(str(REF_PATH))
    return _ref


def ref_solve(a, f=1.0, *, tol=1e-10, max_iter=10000, preconditioner="multigrid", pre_sweeps=1,
              post_sweeps=1, cycle_index=2, record_history=False) -> dict:
    """The reference's own darcy::solve, through oracle/ref_driver.cpp."""
    a = _f64(a)
    n = a.shape[0]
    rhs = _rhs(f, n)
    u = np.empty((n, n))
    hist = np.empty(max_iter + 2)
    it, conv, lev, hl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    res = ctypes.c_double()
    err = ctypes.create_string_buffer(256)
    rc = ref_lib().ref_solve(
        _dp(a), _dp(rhs), ctypes.c_int64(n), ctypes.c_double(tol), int(max_iter),
        PRECONDITIONERS[preconditioner], int(pre_sweeps), int(post_sweeps), int(cycle_index),
        int(bool(record_history)), _dp(u), _dp(hist), ctypes.byref(it), ctypes.byref(res),
        ctypes.byref(conv), ctypes.byref(lev), ctypes.byref(hl), err, 256)
    if rc != 0:
        raise OracleError(err.value.decode())
    return {
        "u": u, "iterations": it.value, "residual": res.value, "converged": bool(conv.value),
        "levels": lev.value, "history": hist[: hl.value].copy(),
    }


def ref_apply_operator(a, x) -> np.ndarray:
    a, x = _f64(a), _f64(x)
    y = np.empty_like(x)
    ref_lib().ref_apply_operator(_dp(a), _dp(x), ctypes.c_int64(a.shape[0]), _dp(y))
    return y


def ref_apply_preconditioner(a, r, *, pre_sweeps=1, post_sweeps=1, cycle_index=2) -> np.ndarray:
    a, r = _f64(a), _f64(r)
    z = np.empty_like(r)
    ref_lib().ref_apply_preconditioner(_dp(a), _dp(r), ctypes.c_int64(a.shape[0]), int(pre_sweeps),
                                       int(post_sweeps), int(cycle_index), _dp(z))
    return z


def ref_hierarchy(a) -> list[dict]:
    a = _f64(a)
    n = a.shape[0]
    cap = sum(6 * s * s for s in level_sides(n))
    buf = np.empty(cap)
    got = ref_lib().ref_hierarchy(_dp(a), ctypes.c_int64(n), _dp(buf), ctypes.c_int64(cap))
    if got != cap:
        raise OracleError("reference hierarchy dump failed")
    return _split_hierarchy(buf, n)


def ref_set_threads(t: int) -> None:
    ref_lib().ref_set_threads(int(t))


def cpu_count() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
