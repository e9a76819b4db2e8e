"""The reference's own acceptance suite (tests/test_correctness.py,
tests/test_multigrid.py, tests/test_api.py of darcy-cpp), restated against the
GPU package. Same properties and thresholds; the independent oracle is an
assembled sparse direct solve (tests/scipy_direct.py)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import two_phase

pytestmark = pytest.mark.gpu
scipy = pytest.importorskip("scipy")
from scipy_direct import assemble, direct_solve  # noqa: E402


@pytest.fixture(scope="module")
def darcy():
    import darcy_cpp_gb300

    return darcy_cpp_gb300


# ---------------------------------------------------- test_correctness.py


@pytest.mark.parametrize("n", [16, 31, 32, 48, 64])
def test_matches_sparse_direct_solve(darcy, n, preconditioner) -> None:
    a = two_phase(n, seed=n)
    res = darcy.solve(a, tol=1e-12, max_iter=200_000, preconditioner=preconditioner)
    assert res.converged
    exp = direct_solve(a)
    assert np.linalg.norm(res.u - exp) / np.linalg.norm(exp) < 1e-8


def test_preconditioners_agree(darcy) -> None:
    a = two_phase(40, seed=7)
    sols = [darcy.solve(a, tol=1e-13, max_iter=200_000, preconditioner=p).u for p in ("multigrid", "jacobi", "none")]
    for other in sols[1:]:
        assert np.allclose(sols[0], other, rtol=1e-7, atol=1e-14)


def test_operator_matches_assembled_matrix(darcy) -> None:
    rng = np.random.default_rng(0)
    a = two_phase(17, seed=11)
    mat = assemble(a)
    for _ in range(5):
        x = rng.standard_normal((17, 17))
        assert np.allclose(darcy.apply_operator(a, x), (mat @ x.ravel()).reshape(17, 17), atol=1e-12)


def test_solution_positive_and_bounded(darcy) -> None:
    res = darcy.solve(two_phase(48, seed=9), f=1.0, tol=1e-12)
    assert (res.u > 0).all()
    slowest = darcy.solve(np.full((48, 48), 3.0), f=1.0, tol=1e-12)
    assert res.u.max() <= slowest.u.max() * (1 + 1e-9)


def test_symmetric_problem_symmetric_solution(darcy) -> None:
    res = darcy.solve(np.full((40, 40), 5.0), tol=1e-13)
    assert np.allclose(res.u, res.u.T, atol=1e-11)
    assert np.allclose(res.u, res.u[::-1, :], atol=1e-11)


def test_scales_inversely_with_permeability(darcy) -> None:
    u1 = darcy.solve(np.full((40, 40), 1.0), tol=1e-13).u
    u2 = darcy.solve(np.full((40, 40), 2.0), tol=1e-13).u
    assert np.allclose(u1, 2.0 * u2, rtol=1e-8)


def test_residual_is_actually_achieved(darcy) -> None:
    n, tol = 64, 1e-11
    a = two_phase(n, seed=2)
    res = darcy.solve(a, tol=tol)
    b = np.full((n, n), (1.0 / (n + 1)) ** 2)
    true = np.linalg.norm(b - darcy.apply_operator(a, res.u)) / np.linalg.norm(b)
    assert true < 10 * tol
    assert res.residual == pytest.approx(true, rel=0.05, abs=1e-13)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_tiny_grids(darcy, n) -> None:
    res = darcy.solve(np.full((n, n), 2.0), tol=1e-13)
    assert res.converged
    assert np.allclose(res.u, direct_solve(np.full((n, n), 2.0)), atol=1e-12)


def test_extreme_contrast(darcy) -> None:
    a = darcy.two_phase_permeability(darcy.gaussian_random_field(64, seed=13), hi=1e6, lo=1.0)
    res = darcy.solve(a, tol=1e-10, max_iter=2000)
    assert res.converged
    exp = direct_solve(a)
    assert np.linalg.norm(res.u - exp) / np.linalg.norm(exp) < 1e-6


# ------------------------------------------------------ test_multigrid.py


def test_hierarchy_depth_is_logarithmic(darcy) -> None:
    for n, exp in [(1, 1), (2, 2), (4, 3), (8, 4), (16, 5), (64, 7), (128, 8)]:
        assert darcy.solve(np.full((n, n), 1.0), tol=1e-10).levels == exp


def test_odd_grids_coarsen_fully(darcy) -> None:
    for n in (17, 33, 47, 63):
        assert darcy.solve(np.full((n, n), 1.0), tol=1e-10).levels >= 5


@pytest.mark.parametrize("cycle_index", [1, 2])
def test_beats_jacobi_by_an_order_of_magnitude(darcy, cycle_index) -> None:
    a = two_phase(128, seed=0)
    mg = darcy.solve(a, tol=1e-10, cycle_index=cycle_index)
    jac = darcy.solve(a, tol=1e-10, preconditioner="jacobi", max_iter=100_000)
    assert mg.converged and jac.converged
    assert mg.iterations * 10 < jac.iterations


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_w_cycle_near_grid_independent(darcy, form) -> None:
    counts = {}
    for n in (32, 64, 128, 256, 512):
        res = darcy.solve(two_phase(n, seed=0), tol=1e-10, cycle_index=2, form=form)
        assert res.converged
        counts[n] = res.iterations
    assert counts[512] / counts[32] < 2.0, counts
    assert counts[512] < 50, counts


def test_more_smoothing_never_hurts(darcy) -> None:
    a = two_phase(128, seed=1)
    assert darcy.solve(a, tol=1e-10, pre_sweeps=3, post_sweeps=3).iterations <= darcy.solve(a, tol=1e-10).iterations


def test_w_beats_v(darcy) -> None:
    a = two_phase(256, seed=2)
    assert darcy.solve(a, tol=1e-10, cycle_index=2).iterations < darcy.solve(a, tol=1e-10, cycle_index=1).iterations


def test_residual_history_converges_steadily(darcy) -> None:
    res = darcy.solve(two_phase(128, seed=3), tol=1e-10, record_history=True)
    h = res.history
    assert h[0] == 1.0 and len(h) == res.iterations + 1 and h[-1] < 1e-10
    ratios = h[1:] / h[:-1]
    assert ratios[1:].max() < 1.0
    assert np.median(ratios) < 0.6


@pytest.mark.parametrize("cycle_index", [1, 2])
@pytest.mark.parametrize("sweeps", [1, 2, 3])
def test_preconditioner_is_symmetric(darcy, cycle_index, sweeps) -> None:
    rng = np.random.default_rng(4)
    a = two_phase(32, seed=8)
    for _ in range(5):
        r, s = rng.standard_normal((32, 32)), rng.standard_normal((32, 32))
        mr = darcy.apply_preconditioner(a, r, pre_sweeps=sweeps, post_sweeps=sweeps, cycle_index=cycle_index)
        ms = darcy.apply_preconditioner(a, s, pre_sweeps=sweeps, post_sweeps=sweeps, cycle_index=cycle_index)
        left, right = float(np.sum(mr * s)), float(np.sum(ms * r))
        assert abs(left - right) / max(abs(left), abs(right), 1e-300) < 1e-10


def test_preconditioner_approximates_inverse(darcy) -> None:
    rng = np.random.default_rng(6)
    a = two_phase(64, seed=10)
    worst = 0.0
    for _ in range(10):
        x = rng.standard_normal((64, 64))
        e = x - darcy.apply_preconditioner(a, darcy.apply_operator(a, x))
        worst = max(worst, float(np.linalg.norm(e) / np.linalg.norm(x)))
    assert worst < 0.5


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_scales_to_a_million_cells(darcy, form) -> None:
    res = darcy.solve(two_phase(1024, seed=0), tol=1e-10, form=form)
    assert res.converged and res.iterations < 60 and res.levels == 11


# ------------------------------------------------------------ test_api.py


def test_accepts_awkward_inputs(darcy) -> None:
    a = two_phase(32, seed=0)
    assert np.allclose(darcy.solve(a.astype(np.float32)).u, darcy.solve(a).u, rtol=1e-6)
    assert darcy.solve(np.full((16, 16), 4, dtype=np.int32)).converged
    b = two_phase(32, seed=1)
    assert np.allclose(darcy.solve(np.asfortranarray(b)).u, darcy.solve(b).u, atol=1e-12)
    assert darcy.solve(two_phase(64, seed=2)[::2, ::2]).converged
    assert darcy.solve([[1.0, 2.0], [2.0, 1.0]]).converged


def test_does_not_mutate_input_and_output_is_fresh(darcy) -> None:
    a = two_phase(32, seed=3)
    orig = a.copy()
    darcy.solve(a)
    assert np.array_equal(a, orig)
    res = darcy.solve(two_phase(16, seed=4))
    assert res.u.flags.writeable and res.u.flags.c_contiguous
    res.u[0, 0] = 123.0
    assert darcy.solve(two_phase(16, seed=4)).u[0, 0] != 123.0


def test_scalar_and_uniform_array_forcing_agree(darcy) -> None:
    a = two_phase(24, seed=5)
    assert np.allclose(darcy.solve(a, 2.5, tol=1e-12).u, darcy.solve(a, np.full((24, 24), 2.5), tol=1e-12).u,
                       atol=1e-13)


def test_single_sample_batch(darcy) -> None:
    a = two_phase(16, seed=1)
    assert np.allclose(darcy.solve_batch(a[None], tol=1e-12).u[0], darcy.solve(a, tol=1e-12).u, atol=1e-12)


def test_repr_and_history(darcy) -> None:
    text = repr(darcy.solve(two_phase(16, seed=0)))
    for token in ("SolveResult", "iterations", "residual", "converged"):
        assert token in text
    assert darcy.solve(two_phase(16, seed=0)).history.size == 0
    assert darcy.solve(two_phase(16, seed=0), record_history=True).history.size > 0
