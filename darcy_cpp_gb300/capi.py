"""ctypes binding of the C ABI (include/darcy_gpu.h).

This is the binding a caller without the pybind11 extension would write, and
the route the benchmark and the C-ABI tests use: plain pointers and sizes,
host or device buffers, status codes, `dgpu_last_error()` for messages.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libdarcy_gpu.so"

OK, INVALID_INPUT, CUDA_ERROR, NO_MEMORY, TIMEOUT = 0, 1, 2, 3, 4
PC = {"none": 0, "jacobi": 1, "multigrid": 2, "mg": 2}
FORM = {"fp64": 0, "plain": 0, "mixed": 1}


class Options(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iter", ctypes.c_int), ("preconditioner", ctypes.c_int),
                ("pre_sweeps", ctypes.c_int), ("post_sweeps", ctypes.c_int), ("cycle_index", ctypes.c_int),
                ("record_history", ctypes.c_int), ("form", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("residual", ctypes.c_double), ("converged", ctypes.c_int),
                ("levels", ctypes.c_int), ("history_len", ctypes.c_int), ("true_residual", ctypes.c_double),
                ("device_ms", ctypes.c_double), ("kernel_launches", ctypes.c_int64)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("avg_ms", ctypes.c_double), ("bytes", ctypes.c_double),
                ("launches_per_iteration", ctypes.c_double)]


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_lib = None


class DarcyGpuError(RuntimeError):
    pass


class InvalidInput(ValueError):
    pass


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(str(LIB_PATH))
        L.dgpu_last_error.restype = ctypes.c_char_p
        L.dgpu_create.argtypes = [ctypes.c_int, ctypes.POINTER(_P)]
        L.dgpu_destroy.argtypes = [_P]
        L.dgpu_destroy.restype = None
        L.dgpu_device_info.argtypes = [_P, ctypes.c_char_p, ctypes.c_int]
        L.dgpu_solve.argtypes = [_P, _P, _P, ctypes.c_double, ctypes.c_int64, ctypes.POINTER(Options), _P, _P, _P,
                                 ctypes.POINTER(Stats)]
        L.dgpu_solve_device.argtypes = [_P, _P, _P, ctypes.c_double, ctypes.c_int64, ctypes.POINTER(Options), _P,
                                        _P, ctypes.POINTER(Stats), _P]
        L.dgpu_solve_batch.argtypes = [_P, _P, _P, ctypes.c_double, ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                       ctypes.POINTER(Options), _P, _P, _P, _P, _P, _P]
        L.dgpu_solve_batch_device.argtypes = [_P, _P, _P, ctypes.c_double, ctypes.c_int, ctypes.c_int64,
                                              ctypes.c_int64, ctypes.POINTER(Options), _P, _P, _P, _P, _P, _P, _P, _P]
        L.dgpu_last_launches.argtypes = [_P]
        L.dgpu_last_launches.restype = ctypes.c_int64
        L.dgpu_solve_uneven.argtypes = [_P, ctypes.c_int64, _P, _P, _P, ctypes.c_double, ctypes.POINTER(Options),
                                        _P, _P, _P, _P, _P, _P]
        L.dgpu_apply_operator.argtypes = [_P, _P, _P, ctypes.c_int64, _P]
        L.dgpu_apply_preconditioner.argtypes = [_P, _P, _P, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, _P]
        L.dgpu_hierarchy.argtypes = [_P, _P, ctypes.c_int64, _P, ctypes.c_int64]
        L.dgpu_hierarchy.restype = ctypes.c_int64
        L.dgpu_num_levels.argtypes = [ctypes.c_int64]
        L.dgpu_profile_kernels.argtypes = [_P, _P, ctypes.c_int64, ctypes.POINTER(Options), ctypes.c_int,
                                           ctypes.POINTER(KernelTime), ctypes.c_int, _I]
        L.dgpu_flush_l2.argtypes = [_P, ctypes.c_int64]
        L.dgpu_check_conversions.argtypes = [_P, _P, ctypes.c_int64, _P, _P, _P, _P]
        L.dgpu_check_conversions.restype = ctypes.c_int64
        L.dgpu_apply_preconditioner_noalloc.argtypes = [_P, _P, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                                        ctypes.c_int, _P, _P]
        L.dgpu_random_fields.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_ulonglong, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, _P,
                                         ctypes.c_int, _P]
        # learned warm start
        L.dgpu_net_create.argtypes = [ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(_P)]
        L.dgpu_net_destroy.argtypes = [_P]
        L.dgpu_net_destroy.restype = None
        L.dgpu_net_num_params.argtypes = [_P]
        L.dgpu_net_num_params.restype = ctypes.c_int64
        L.dgpu_net_side.argtypes = [_P]
        L.dgpu_net_get_params.argtypes = [_P, _P]
        L.dgpu_net_set_params.argtypes = [_P, _P]
        L.dgpu_net_get_scaling.argtypes = [_P, _P]
        L.dgpu_net_set_scaling.argtypes = [_P, _P]
        L.dgpu_net_set_engine.argtypes = [_P, ctypes.c_int]
        L.dgpu_net_set_loss.argtypes = [_P, ctypes.c_int]
        L.dgpu_net_set_first_wait.argtypes = [_P, ctypes.c_longlong]
        L.dgpu_net_load_pairs.argtypes = [_P, _P, _P, _P, ctypes.c_int64]
        L.dgpu_net_train.argtypes = [_P, ctypes.c_int64, ctypes.c_int, ctypes.c_float, ctypes.c_ulonglong, _P]
        L.dgpu_net_gradients.argtypes = [_P, _P, _P, _P, ctypes.c_int64, _P, _P]
        L.dgpu_net_predict.argtypes = [_P, _P, _P, ctypes.c_int64, _P]
        L.dgpu_net_features.argtypes = [_P, _P, _P, ctypes.c_int64, _P]
        L.dgpu_net_predict_device.argtypes = [_P, _P, _P, ctypes.c_int64, _P, _P]
        L.dgpu_net_last_launches.argtypes = [_P]
        L.dgpu_net_last_launches.restype = ctypes.c_int64
        L.dgpu_net_info.argtypes = [_P, ctypes.c_char_p, ctypes.c_int]
        L.dgpu_solve_batch_learned.argtypes = [_P, _P, _P, ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
                                               ctypes.POINTER(Options), _P, _P, _P, _P, _P]
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc == OK:
        return
    msg = lib().dgpu_last_error().decode()
    if rc == INVALID_INPUT:
        raise InvalidInput(msg)
    raise DarcyGpuError(f"status {rc}: {msg}")


def options(tol=1e-10, max_iter=10000, preconditioner="multigrid", pre_sweeps=1, post_sweeps=1, cycle_index=2,
            record_history=False, form="fp64") -> Options:
    return Options(float(tol), int(max_iter), PC[preconditioner], int(pre_sweeps), int(post_sweeps),
                   int(cycle_index), int(bool(record_history)), FORM[form])


def _ptr(arr: np.ndarray | None):
    return None if arr is None else ctypes.c_void_p(arr.ctypes.data)


def _f64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


def apply_preconditioner_noalloc(d_a: int, d_r: int, n: int, d_z: int, pre_sweeps: int = 1, post_sweeps: int = 1,
                                 cycle_index: int = 2, stream: int | None = None) -> None:
    """z = M r on caller-owned device buffers with no device allocation
    (dgpu_apply_preconditioner_noalloc; n <= 128, calls must not overlap)."""
    check(lib().dgpu_apply_preconditioner_noalloc(ctypes.c_void_p(d_a), ctypes.c_void_p(d_r), int(n), int(pre_sweeps),
                                                  int(post_sweeps), int(cycle_index), ctypes.c_void_p(d_z),
                                                  ctypes.c_void_p(stream) if stream else None))


def random_fields(n: int, count: int, seed: int = 0, alpha: float = 2.0, tau: float = 3.0, hi: float = 12.0,
                  lo: float = 3.0, raw: bool = False) -> np.ndarray:
    """`count` two-phase fields (or raw Gaussian fields) generated on the GPU
    (dgpu_random_fields; same distribution as the host generator, other bits)."""
    out = np.empty((int(count), int(n), int(n)))
    check(lib().dgpu_random_fields(int(n), int(count), int(seed) & ((1 << 64) - 1), float(alpha), float(tau),
                                   float(hi), float(lo), int(bool(raw)), _ptr(out), 0, None))
    return out


class Context:
    """Owns one dgpu_context (stream, device buffers, captured graphs)."""

    def __init__(self, device: int = -1) -> None:
        self.handle = _P()
        check(lib().dgpu_create(int(device), ctypes.byref(self.handle)))

    def close(self) -> None:
        if self.handle:
            lib().dgpu_destroy(self.handle)
            self.handle = _P()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> str:
        buf = ctypes.create_string_buffer(512)
        check(lib().dgpu_device_info(self.handle, buf, 512))
        return buf.value.decode()

    def solve(self, a, f=1.0, x0=None, **kw) -> dict:
        a = _f64(a)
        n = a.shape[0]
        fa = None if np.isscalar(f) else _f64(f)
        u = np.empty_like(a)
        opt = options(**kw)
        hist = np.empty(opt.max_iter + 1) if opt.record_history else None
        st = Stats()
        check(lib().dgpu_solve(self.handle, _ptr(a), _ptr(fa), float(f) if fa is None else 0.0, n,
                               ctypes.byref(opt), _ptr(None if x0 is None else _f64(x0)), _ptr(u), _ptr(hist),
                               ctypes.byref(st)))
        return {"u": u, "iterations": st.iterations, "residual": st.residual, "converged": bool(st.converged),
                "levels": st.levels, "true_residual": st.true_residual, "device_ms": st.device_ms,
                "kernel_launches": st.kernel_launches,
                "history": hist[: st.history_len].copy() if hist is not None else np.empty(0)}

    def solve_device(self, d_a: int, n: int, d_u: int, stream: int | None = None, f_scalar: float = 1.0,
                     **kw) -> Stats:
        """Solve on device-resident buffers (raw device pointers)."""
        opt = options(**kw)
        st = Stats()
        check(lib().dgpu_solve_device(self.handle, ctypes.c_void_p(d_a), None, float(f_scalar), int(n),
                                      ctypes.byref(opt), None, ctypes.c_void_p(d_u), ctypes.byref(st),
                                      ctypes.c_void_p(stream) if stream else None))
        return st

    def solve_batch(self, a, f=1.0, **kw) -> dict:
        a = _f64(a)
        batch, n = a.shape[0], a.shape[1]
        fa = None if np.isscalar(f) else _f64(f)
        u = np.empty_like(a)
        it = np.zeros(batch, dtype=np.int32)
        res = np.zeros(batch)
        conv = np.zeros(batch, dtype=np.int32)
        lev = np.zeros(batch, dtype=np.int32)
        opt = options(**kw)
        check(lib().dgpu_solve_batch(self.handle, _ptr(a), _ptr(fa), float(f) if fa is None else 0.0, 0, batch, n,
                                     ctypes.byref(opt), None, _ptr(u), _ptr(it), _ptr(res), _ptr(conv), _ptr(lev)))
        return {"u": u, "iterations": it, "residuals": res, "converged": conv.astype(bool), "levels": lev}

    def solve_batch_device(self, d_a: int, batch: int, n: int, d_u: int, stream: int | None = None,
                           f_scalar: float = 1.0, **kw) -> dict:
        """Batched solve on device-resident packed arrays (raw device pointers)."""
        it = np.zeros(batch, dtype=np.int32)
        res = np.zeros(batch)
        conv = np.zeros(batch, dtype=np.int32)
        ms = np.zeros(1)
        opt = options(**kw)
        check(lib().dgpu_solve_batch_device(self.handle, ctypes.c_void_p(d_a), None, float(f_scalar), 0, int(batch),
                                            int(n), ctypes.byref(opt), None, ctypes.c_void_p(d_u), _ptr(it),
                                            _ptr(res), _ptr(conv), None, _ptr(ms),
                                            ctypes.c_void_p(stream) if stream else None))
        return {"iterations": it, "residuals": res, "converged": conv.astype(bool), "device_ms": float(ms[0]),
                "kernel_launches": int(lib().dgpu_last_launches(self.handle))}

    def solve_uneven(self, fields, f=None, x0=None, f_scalar: float = 1.0, **kw) -> dict:
        """Problems of different sides in one call (dgpu_solve_uneven); f and
        x0 are None or one array per problem."""
        arrays = [_f64(x) for x in fields]
        sides = np.array([x.shape[0] for x in arrays], dtype=np.int64)
        a = np.concatenate([x.ravel() for x in arrays])
        fa = None if f is None else np.concatenate([_f64(x).ravel() for x in f])
        u0 = None if x0 is None else np.concatenate([_f64(x).ravel() for x in x0])
        u = np.empty_like(a)
        count = len(arrays)
        it = np.zeros(count, dtype=np.int32)
        res = np.zeros(count)
        conv = np.zeros(count, dtype=np.int32)
        lev = np.zeros(count, dtype=np.int32)
        opt = options(**kw)
        check(lib().dgpu_solve_uneven(self.handle, count, _ptr(sides), _ptr(a), _ptr(fa), float(f_scalar),
                                      ctypes.byref(opt), _ptr(u0), _ptr(u), _ptr(it), _ptr(res), _ptr(conv),
                                      _ptr(lev)))
        out, at = [], 0
        for n in sides:
            out.append(u[at:at + n * n].reshape(n, n))
            at += n * n
        return {"u": out, "iterations": it, "residuals": res, "converged": conv.astype(bool), "levels": lev}

    def apply_operator(self, a, x) -> np.ndarray:
        a, x = _f64(a), _f64(x)
        y = np.empty_like(x)
        check(lib().dgpu_apply_operator(self.handle, _ptr(a), _ptr(x), a.shape[0], _ptr(y)))
        return y

    def apply_preconditioner(self, a, r, pre_sweeps=1, post_sweeps=1, cycle_index=2, form="fp64") -> np.ndarray:
        a, r = _f64(a), _f64(r)
        z = np.empty_like(r)
        check(lib().dgpu_apply_preconditioner(self.handle, _ptr(a), _ptr(r), a.shape[0], pre_sweeps, post_sweeps,
                                              cycle_index, FORM[form], _ptr(z)))
        return z

    def profile_kernels(self, a, reps: int = 20, **kw) -> list[dict]:
        a = _f64(a)
        rows = (KernelTime * 64)()
        count = ctypes.c_int()
        opt = options(**kw)
        check(lib().dgpu_profile_kernels(self.handle, _ptr(a), a.shape[0], ctypes.byref(opt), int(reps), rows, 64,
                                         ctypes.byref(count)))
        return [{"name": r.name.decode(), "avg_ms": r.avg_ms, "bytes": r.bytes,
                 "launches_per_iteration": r.launches_per_iteration} for r in rows[: count.value]]

    def flush_l2(self, nbytes: int = 512 << 20) -> None:
        check(lib().dgpu_flush_l2(self.handle, int(nbytes)))

    def check_conversions(self, x):
        """The engine's integer-pipe FP64<->FP32 conversions on the values x:
        (mismatches against the conversion instructions, hi, lo, rounded,
        widened)."""
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        hi = np.empty(x.size, np.float32)
        lo = np.empty(x.size, np.float32)
        rd = np.empty(x.size, np.float32)
        wd = np.empty(x.size, np.float64)
        mism = lib().dgpu_check_conversions(self.handle, _ptr(x), x.size, _ptr(hi), _ptr(lo), _ptr(rd), _ptr(wd))
        if mism < 0:
            check(-1)
        return int(mism), hi, lo, rd, wd

    def solve_batch_learned(self, net: "Net", a, f: float = 1.0, **kw) -> dict:
        """solve_batch with the warm start predicted on the device by `net`."""
        a = _f64(a)
        batch, n = a.shape[0], a.shape[1]
        u = np.empty_like(a)
        it = np.zeros(batch, dtype=np.int32)
        res = np.zeros(batch)
        conv = np.zeros(batch, dtype=np.int32)
        lev = np.zeros(batch, dtype=np.int32)
        opt = options(**kw)
        check(lib().dgpu_solve_batch_learned(self.handle, net.handle, _ptr(a), float(f), batch, n, ctypes.byref(opt),
                                             _ptr(u), _ptr(it), _ptr(res), _ptr(conv), _ptr(lev)))
        return {"u": u, "iterations": it, "residuals": res, "converged": conv.astype(bool), "levels": lev}


ENGINE = {"tensor": 0, "simt": 1}
LOSS = {"energy": 0, "mse": 1}


class Net:
    """Owns one dgpu_net (the warm-start network of include/darcy_gpu.h)."""

    def __init__(self, side: int, seed: int = 0) -> None:
        self.handle = _P()
        check(lib().dgpu_net_create(int(side), int(seed) & ((1 << 64) - 1), ctypes.byref(self.handle)))
        self.side = int(side)

    def close(self) -> None:
        if self.handle:
            lib().dgpu_net_destroy(self.handle)
            self.handle = _P()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(lib().dgpu_net_num_params(self.handle))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        check(lib().dgpu_net_get_params(self.handle, _ptr(out)))
        return out

    def set_params(self, w) -> None:
        w = np.ascontiguousarray(np.asarray(w, dtype=np.float32))
        if w.shape != (self.num_params,):
            raise InvalidInput(f"expected {self.num_params} parameters, got shape {w.shape}")
        check(lib().dgpu_net_set_params(self.handle, _ptr(w)))

    def get_scaling(self) -> np.ndarray:
        out = np.empty(4)
        check(lib().dgpu_net_get_scaling(self.handle, _ptr(out)))
        return out

    def set_scaling(self, s) -> None:
        s = _f64(s)
        if s.shape != (4,):
            raise InvalidInput("scaling has four entries: mean and std of log a, RMS of u, fref")
        check(lib().dgpu_net_set_scaling(self.handle, _ptr(s)))

    def set_engine(self, engine: str) -> None:
        check(lib().dgpu_net_set_engine(self.handle, ENGINE[engine]))

    def set_first_wait(self, polls: int) -> None:
        """Test hook: polls of each tensor-core convolution CTA's first MMA
        wait (dgpu_net_set_first_wait; default 1 << 24, 0 = run out at once)."""
        check(lib().dgpu_net_set_first_wait(self.handle, int(polls)))

    def set_loss(self, kind: str) -> None:
        check(lib().dgpu_net_set_loss(self.handle, LOSS[kind]))

    def _pack(self, a, u=None, f=None):
        a = _f64(a)
        if a.ndim == 2:
            a = a[None]
        if a.ndim != 3 or a.shape[1] != self.side or a.shape[2] != self.side:
            raise InvalidInput(f"a must have shape (count, {self.side}, {self.side})")
        uu = None if u is None else _f64(u).reshape(a.shape)
        ff = None
        if f is not None and not np.isscalar(f):
            ff = _f64(f).reshape(a.shape[0])
        elif f is not None and float(f) != 1.0:
            ff = np.full(a.shape[0], float(f))
        return a, uu, ff

    def load_pairs(self, a, u, f=None) -> None:
        a, u, ff = self._pack(a, u, f)
        check(lib().dgpu_net_load_pairs(self.handle, _ptr(a), _ptr(u), _ptr(ff), a.shape[0]))

    def train(self, steps: int, batch: int = 256, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.empty(int(steps), dtype=np.float32)
        check(lib().dgpu_net_train(self.handle, int(steps), int(batch), float(lr), int(seed) & ((1 << 64) - 1),
                                   _ptr(losses)))
        return losses

    def gradients(self, a, u, f=None) -> tuple[np.ndarray, float]:
        a, u, ff = self._pack(a, u, f)
        g = np.empty(self.num_params, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        check(lib().dgpu_net_gradients(self.handle, _ptr(a), _ptr(u), _ptr(ff), a.shape[0], _ptr(g), _ptr(loss)))
        return g, float(loss[0])

    def features(self, a, f=None) -> np.ndarray:
        a, _, ff = self._pack(a, None, f)
        out = np.empty(a.shape + (2,), dtype=np.float32)
        check(lib().dgpu_net_features(self.handle, _ptr(a), _ptr(ff), a.shape[0], _ptr(out)))
        return out

    def predict(self, a, f=None) -> np.ndarray:
        a, _, ff = self._pack(a, None, f)
        u0 = np.empty_like(a)
        check(lib().dgpu_net_predict(self.handle, _ptr(a), _ptr(ff), a.shape[0], _ptr(u0)))
        return u0

    def predict_device(self, d_a: int, count: int, d_u0: int, d_f: int | None = None,
                       stream: int | None = None) -> None:
        check(lib().dgpu_net_predict_device(self.handle, ctypes.c_void_p(d_a), ctypes.c_void_p(d_f) if d_f else None,
                                            int(count), ctypes.c_void_p(d_u0),
                                            ctypes.c_void_p(stream) if stream else None))

    def info(self) -> str:
        buf = ctypes.create_string_buffer(1024)
        check(lib().dgpu_net_info(self.handle, buf, 1024))
        return buf.value.decode()

    def last_launches(self) -> int:
        return int(lib().dgpu_net_last_launches(self.handle))
