"""Independent direct solve for the acceptance tests (assembled CSR + spsolve):
a second oracle built a different way from the matrix-free path
(darcy_cpp_gb300/reference.py, after the reference's python/darcy/reference.py),
loaded by path so that it does not need the compiled extension."""

from __future__ import annotations

import importlib.util
from pathlib import Path

_spec = importlib.util.spec_from_file_location(
    "_darcy_reference", Path(__file__).resolve().parents[1] / "darcy_cpp_gb300" / "reference.py")
_mod = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(_mod)

assemble = _mod.assemble_matrix
direct_solve = _mod.solve_reference
