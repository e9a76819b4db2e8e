"""Host-side checks that need no GPU: the C-ABI library loads and exports every
symbol include/darcy_gpu.h declares, and the extension validates its inputs
before touching the device (reference src/bindings.cpp:33-78 messages)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def built():
    import __graft_entry__

    builder = __graft_entry__._builder()
    if not builder.LIB.exists() or not builder.EXT.exists():
        builder.build()
    return builder.LIB


def declared_symbols() -> list[str]:
    text = (ROOT / "include" / "darcy_gpu.h").read_text()
    return sorted(set(re.findall(r"\b(dgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_reference_entry_points() -> None:
    names = declared_symbols()
    for want in ("dgpu_solve", "dgpu_solve_batch", "dgpu_apply_operator", "dgpu_apply_preconditioner",
                 "dgpu_last_error", "dgpu_create", "dgpu_destroy"):
        assert want in names


def test_library_exports_every_declared_symbol(built) -> None:
    lib = ctypes.CDLL(str(built))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_num_levels_without_a_device(built) -> None:
    lib = ctypes.CDLL(str(built))
    lib.dgpu_num_levels.argtypes = [ctypes.c_int64]
    for n, want in [(1, 1), (2, 2), (4, 3), (8, 4), (16, 5), (64, 7), (128, 8), (1024, 11), (2048, 12),
                    (17, 6), (33, 7), (47, 7), (63, 7)]:
        assert lib.dgpu_num_levels(n) == want


def test_build_info_has_exactly_the_reference_keys(built) -> None:
    import darcy_cpp_gb300 as darcy

    info = darcy.build_info()
    assert set(info) == {"version", "compiler", "openmp", "max_threads", "numpy"}
    assert isinstance(info["openmp"], bool) and info["max_threads"] >= 1
    assert darcy.__version__.count(".") == 2


@pytest.mark.parametrize("call, match", [
    (lambda d: d.solve(np.ones((4, 8))), "square"),
    (lambda d: d.solve(np.ones((4, 4, 4))), "square"),
    (lambda d: d.solve(np.ones((0, 0))), "square"),
    (lambda d: d.solve(np.ones((8, 8)), np.ones((4, 4))), "same shape"),
    (lambda d: d.solve(np.ones((8, 8)), preconditioner="ilu"), "unknown preconditioner"),
    (lambda d: d.solve(np.ones((8, 8)), tol=0.0), "tol"),
    (lambda d: d.solve(np.ones((8, 8)), tol=-1e-3), "tol"),
    (lambda d: d.solve(np.ones((8, 8)), max_iter=0), "max_iter"),
    (lambda d: d.solve(np.ones((8, 8)), pre_sweeps=0), "sweeps"),
    (lambda d: d.solve(np.ones((8, 8)), post_sweeps=0), "sweeps"),
    (lambda d: d.solve(np.ones((8, 8)), cycle_index=3), "cycle_index"),
    (lambda d: d.solve(np.ones((8, 8)), form="fp16"), "unknown form"),
    (lambda d: d.solve_batch(np.ones((8, 8))), r"batch, n, n"),
    (lambda d: d.apply_operator(np.ones((8, 8)), np.ones((4, 4))), "same shape"),
    (lambda d: d.apply_preconditioner(np.ones((8, 8)), np.ones((8, 4))), "square"),
    (lambda d: d.solve(np.ones((8, 8)), x0=np.ones((4, 4))), "same shape"),
])
def test_validation_happens_on_the_host(built, call, match) -> None:
    import darcy_cpp_gb300 as darcy

    with pytest.raises(ValueError, match=match):
        call(darcy)


def test_fields_are_exported(built) -> None:
    import darcy_cpp_gb300 as darcy

    a = darcy.two_phase_permeability(darcy.gaussian_random_field(16, seed=1), hi=9.0, lo=2.0)
    assert set(np.unique(a)) == {2.0, 9.0}
    with pytest.raises(ValueError, match="positive"):
        darcy.two_phase_permeability(np.zeros((8, 8)), hi=1.0, lo=-1.0)
    with pytest.raises(ValueError):
        darcy.gaussian_random_field(0)


# The reference binding's argument lists (src/bindings.cpp:135-137, :194-196,
# :215, :242-243, :258): names and defaults, positional-or-keyword. Arguments
# this engine adds (form, x0) come after them, keyword-only.
REFERENCE_ARGS = {
    "solve": [("a", None), ("f", "1.0"), ("tol", "1e-10"), ("max_iter", "10000"),
              ("preconditioner", "'multigrid'"), ("pre_sweeps", "1"), ("post_sweeps", "1"),
              ("cycle_index", "2"), ("record_history", "False")],
    "solve_batch": [("a", None), ("f", "1.0"), ("tol", "1e-10"), ("max_iter", "10000"),
                    ("preconditioner", "'multigrid'"), ("pre_sweeps", "1"), ("post_sweeps", "1"),
                    ("cycle_index", "2"), ("threads", "0")],
    "apply_operator": [("a", None), ("x", None)],
    "apply_preconditioner": [("a", None), ("r", None), ("pre_sweeps", "1"), ("post_sweeps", "1"),
                             ("cycle_index", "2")],
    "set_num_threads": [("threads", None)],
    "num_threads": [],
    "has_openmp": [],
}


def _signature(fn) -> tuple[list[tuple[str, str | None]], list[str]]:
    """(positional-or-keyword (name, default) pairs, keyword-only names) from
    the first line of a pybind11 docstring."""
    line = fn.__doc__.splitlines()[0]
    inner = line[line.index("(") + 1: line.rindex(")")]
    parts, depth, cur = [], 0, ""
    for ch in inner:  # split at commas outside brackets
        depth += ch == "["
        depth -= ch == "]"
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur.strip())
    positional, keyword, kw = [], [], False
    for p in parts:
        if p == "*":
            kw = True
            continue
        name = p.split(":")[0].strip()
        default = p.split(" = ", 1)[1].strip() if " = " in p else None
        (keyword if kw else positional).append(name if kw else (name, default))
    return positional, keyword


@pytest.mark.parametrize("name", sorted(REFERENCE_ARGS))
def test_core_signatures_match_the_reference_binding(built, name: str) -> None:
    from darcy_cpp_gb300 import _core

    positional, keyword = _signature(getattr(_core, name))
    assert positional == REFERENCE_ARGS[name]
    assert set(keyword) <= {"form", "x0"}


def test_core_module_attributes(built) -> None:
    from darcy_cpp_gb300 import _core

    assert issubclass(_core.InvalidInput, ValueError)
    assert isinstance(_core.__version__, str) and isinstance(_core.__compiler__, str)
    for field in ("u", "iterations", "residual", "converged", "levels", "history"):
        assert hasattr(_core.SolveResult, field)


# python/darcy/__init__.py:119-278: the package functions' positional
# arguments, keyword-only arguments and defaults (tol defaults to 1e-10).
PACKAGE_ARGS = {
    "solve": (["a", "f"], {"f": 1.0, "tol": 1e-10, "max_iter": 10000, "preconditioner": "multigrid",
                           "pre_sweeps": 1, "post_sweeps": 1, "cycle_index": 2, "record_history": False}),
    "solve_batch": (["a", "f"], {"f": 1.0, "tol": 1e-10, "max_iter": 10000, "preconditioner": "multigrid",
                                 "pre_sweeps": 1, "post_sweeps": 1, "cycle_index": 2, "threads": 0}),
    "apply_operator": (["a", "x"], {}),
    "apply_preconditioner": (["a", "r"], {"pre_sweeps": 1, "post_sweeps": 1, "cycle_index": 2}),
    "num_threads": ([], {}),
    "set_num_threads": (["threads"], {}),
    "has_openmp": ([], {}),
    "build_info": ([], {}),
}


@pytest.mark.parametrize("name", sorted(PACKAGE_ARGS))
def test_package_signatures_match_the_reference(built, name: str) -> None:
    import inspect

    import darcy_cpp_gb300 as darcy

    params = inspect.signature(getattr(darcy, name)).parameters.values()
    positional = [p.name for p in params if p.kind == p.POSITIONAL_OR_KEYWORD]
    defaults = {p.name: p.default for p in params if p.default is not p.empty}
    want_pos, want_defaults = PACKAGE_ARGS[name]
    assert positional == want_pos
    extra = {k: v for k, v in defaults.items() if k not in want_defaults}
    assert {k: v for k, v in defaults.items() if k in want_defaults} == want_defaults
    assert set(extra) <= {"form", "x0"}
    assert all(p.kind == p.KEYWORD_ONLY for p in params if p.name in extra)


def test_result_classes_keep_the_reference_fields(built) -> None:
    """python/darcy/__init__.py:63-114: frozen dataclasses with these fields in
    this order; fields added here come last and have defaults, so code that
    builds a result positionally or reads these fields works unchanged."""
    import dataclasses

    import darcy_cpp_gb300 as darcy

    for cls, want in ((darcy.SolveResult, ["u", "iterations", "residual", "converged", "levels", "history"]),
                      (darcy.BatchResult, ["u", "iterations", "residuals", "converged"])):
        fields = dataclasses.fields(cls)
        assert [f.name for f in fields][: len(want)] == want
        assert cls.__dataclass_params__.frozen
        for f in fields[len(want):]:
            assert f.default is not dataclasses.MISSING or f.default_factory is not dataclasses.MISSING
    r = darcy.BatchResult(u=np.zeros((2, 1, 1)), iterations=np.array([1, 2]), residuals=np.zeros(2),
                          converged=np.array([True, False]))
    assert r.all_converged is False


def test_package_exports_every_reference_name(built) -> None:
    """python/darcy/__init__.py:38-52 (__all__): every name is exported here too."""
    import darcy_cpp_gb300 as darcy

    for name in ("BatchResult", "SolveResult", "__version__", "apply_operator", "apply_preconditioner",
                 "build_info", "gaussian_random_field", "has_openmp", "num_threads", "set_num_threads",
                 "solve", "solve_batch", "two_phase_permeability"):
        assert name in darcy.__all__ and hasattr(darcy, name), name
