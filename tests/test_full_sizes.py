"""GPU parity at the full sizes of the benchmark configurations, through
properties that do not need the CPU oracle to solve the whole workload:

* 2048 x 2048, a in {1e3, 1e-3} (the large single solve): 12 levels, the
  reference's published iteration count (380, bracketed by 10% for the
  plateau near tol), both forms within 1e-9 of the oracle's solution, and
  exact linearity in f (scaling f by 2 scales every operation of the solve by
  an exact power of two, so u doubles bit for bit);
* the 4096 uneven problems (sides 32..256 drawn per seed, {12, 3}): every
  problem converges in both forms, the mixed solutions are within 1e-9 of the
  FP64 ones, levels follow the side, and a sample agrees with the oracle.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import two_phase

pytestmark = pytest.mark.gpu

REL_L2 = 1e-9
SIDES = [32, 48, 64, 96, 128, 192, 256]


def rel_l2(x, y) -> float:
    return float(np.linalg.norm(np.asarray(x) - np.asarray(y)) / max(np.linalg.norm(y), 1e-300))


@pytest.fixture(scope="module")
def darcy():
    import darcy_cpp_gb300

    return darcy_cpp_gb300


def test_2048_known_answer_linearity_and_oracle_parity(darcy, orc) -> None:
    """2048^2 at 1e6 contrast (the second size of the large-solve workload):
    12 levels, the reference's published 380 iterations (bracketed by 10% for
    the plateau near tol, where the reduction order decides the last step),
    both forms within 1e-9 relative L2 of the oracle's solution, and exact
    linearity in f (scaling f by 2 scales every operation of the solve by an
    exact power of two, so u doubles bit for bit).

    The oracle runs on one thread (~2 min): at this size its multi-threaded
    solutions move with the order in which OpenMP combines the threads' dot
    products -- two 8-thread runs of the same field differ by 3.5e-10, 1, 4
    and 8 threads by up to 8e-10 (366, 380 and 379 iterations) -- so only the
    one-thread solution is a fixed target."""
    a = two_phase(2048, seed=1, hi=1e3, lo=1e-3)
    orc.set_threads(1)
    want = orc.solve(a, tol=1e-10)
    assert want["levels"] == 12 and want["converged"]
    fp64 = darcy.solve(a, tol=1e-10)
    assert fp64.converged and fp64.levels == 12 and fp64.residual < 1e-10
    assert 342 <= fp64.iterations <= 418  # the reference: 380
    assert rel_l2(fp64.u, want["u"]) < REL_L2
    mixed = darcy.solve(a, tol=1e-10, form="mixed")
    assert mixed.converged and mixed.residual < 1e-10
    assert rel_l2(mixed.u, want["u"]) < REL_L2
    doubled = darcy.solve(a, f=2.0, tol=1e-10, form="mixed")
    assert doubled.iterations == mixed.iterations
    assert np.array_equal(doubled.u, 2.0 * mixed.u)


def test_uneven_4096_batch(darcy, orc) -> None:
    sides = [SIDES[np.random.default_rng(s).integers(7)] for s in range(4096)]
    fields = [two_phase(n, seed=s) for s, n in enumerate(sides)]
    fp64 = darcy.solve_batch_uneven(fields, tol=1e-10)
    mixed = darcy.solve_batch_uneven(fields, tol=1e-10, form="mixed")
    assert fp64.converged.all() and mixed.converged.all()
    assert (fp64.residuals < 1e-10).all() and (mixed.residuals < 1e-10).all()
    from darcy_cpp_gb300 import capi

    assert [int(v) for v in fp64.levels] == [capi.lib().dgpu_num_levels(n) for n in sides]
    worst = max(rel_l2(mixed.u[q], fp64.u[q]) for q in range(len(fields)))
    assert worst < REL_L2
    orc.set_threads(1)
    for q in [0, 1, 2, 3, 4, 5]:
        want = orc.solve(fields[q], tol=1e-10)
        assert abs(int(fp64.iterations[q]) - want["iterations"]) <= max(1, round(0.1 * want["iterations"]))
        assert rel_l2(fp64.u[q], want["u"]) < REL_L2


def test_combined_16384x128_plus_64x512(darcy, orc) -> None:
    """16384 problems of 128^2 and 64 of 512^2 at contrast 1e4 in one call
    (the 512^2 ones ride in the same batched launch or go to the grid engine,
    as the routing decides): all converge, mixed within 1e-9 of FP64, and a
    sample of each size agrees with the oracle."""
    from darcy_cpp_gb300 import capi

    # the 128^2 fields from the GPU generator (same distribution as the
    # reference's, other bits; 16384 host-generated ones would take most of the
    # test's time), the 512^2 ones from the host generator
    big = list(capi.random_fields(128, 16384, seed=1, hi=1e2, lo=1e-2))
    big += [two_phase(512, seed=100000 + s, hi=1e2, lo=1e-2) for s in range(64)]
    fp64 = darcy.solve_batch_uneven(big, tol=1e-10)
    mixed = darcy.solve_batch_uneven(big, tol=1e-10, form="mixed")
    assert fp64.converged.all() and mixed.converged.all()
    assert (fp64.residuals < 1e-10).all() and (mixed.residuals < 1e-10).all()
    assert set(int(v) for v in fp64.levels[:16384]) == {8} and set(int(v) for v in fp64.levels[16384:]) == {10}
    small_u = np.stack(fp64.u[:16384])
    err = np.linalg.norm((np.stack(mixed.u[:16384]) - small_u).reshape(16384, -1), axis=1)
    assert (err < REL_L2 * np.linalg.norm(small_u.reshape(16384, -1), axis=1)).all()
    assert max(rel_l2(mixed.u[q], fp64.u[q]) for q in range(16384, len(big))) < REL_L2
    orc.set_threads(1)  # deterministic: several threads combine the dot products in arrival order
    for q in [0, 9999, 16384]:
        want = orc.solve(big[q], tol=1e-10)
        assert abs(int(fp64.iterations[q]) - want["iterations"]) <= max(1, round(0.1 * want["iterations"]))
        assert rel_l2(fp64.u[q], want["u"]) < REL_L2
