"""The allocation-free preconditioner entry point, checked through the C ABI.

dgpu_apply_preconditioner_noalloc exists for callers that cannot allocate
device memory while they run (a host that owns every allocation, a loop that
must not enter cudaMalloc/cudaFree): it keeps its scratch in a fixed array
inside the library and works on device buffers the caller already owns. Its
result must equal the regular entry point's z = M r, call after call, since
every call reuses (and so must fully rebuild) that one shared array.

This file is collected last so that a stop-at-first-failure run has already
run everything else; it also passes on its own in a fresh process.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import two_phase

pytestmark = pytest.mark.gpu

REL = 1e-12  # the preconditioner parity bar used in test_gpu_parity.py


def rel_l2(x, y) -> float:
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from darcy_cpp_gb300 import capi

    return torch, capi, capi.Context()


def device(torch, x: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()


@pytest.mark.parametrize("n", [1, 17, 64, 128])
def test_noalloc_matches_the_allocating_entry_point(env, n) -> None:
    torch, capi, ctx = env
    rng = np.random.default_rng(n)
    # two calls in a row with different fields and right-hand sides: the
    # second must not see anything the first left in the shared scratch
    for call, cycle in enumerate((2, 1)):
        a = two_phase(n, seed=n + 7 * call, hi=1e2, lo=1e-2) if n > 1 else np.full((1, 1), 3.0)
        r = rng.standard_normal((n, n))
        want = ctx.apply_preconditioner(a, r, cycle_index=cycle)
        d_a, d_r = device(torch, a), device(torch, r)
        d_z = torch.empty_like(d_r)
        capi.apply_preconditioner_noalloc(d_a.data_ptr(), d_r.data_ptr(), n, d_z.data_ptr(), cycle_index=cycle,
                                          stream=torch.cuda.current_stream().cuda_stream)
        got = d_z.cpu().numpy()
        assert rel_l2(got, want) < REL, (n, call)


def test_noalloc_more_sweeps_v_cycle_at_the_largest_side(env) -> None:
    """pre/post sweeps and the cycle index go through the shared setup (the
    dense tail is built with them): n = 128, 2 pre and 3 post sweeps, V-cycle,
    twice in a row against the allocating entry point with the same options."""
    torch, capi, ctx = env
    n = 128
    rng = np.random.default_rng(5)
    for call in range(2):
        a = two_phase(n, seed=40 + call, hi=1e2, lo=1e-2)
        r = rng.standard_normal((n, n))
        want = ctx.apply_preconditioner(a, r, pre_sweeps=2, post_sweeps=3, cycle_index=1)
        d_a, d_r = device(torch, a), device(torch, r)
        d_z = torch.empty_like(d_r)
        capi.apply_preconditioner_noalloc(d_a.data_ptr(), d_r.data_ptr(), n, d_z.data_ptr(), pre_sweeps=2,
                                          post_sweeps=3, cycle_index=1,
                                          stream=torch.cuda.current_stream().cuda_stream)
        assert rel_l2(d_z.cpu().numpy(), want) < REL, call


def test_noalloc_repeats_bit_for_bit(env) -> None:
    torch, capi, _ = env
    n = 48
    a, r = two_phase(n, seed=3), np.random.default_rng(0).standard_normal((n, n))
    d_a, d_r = device(torch, a), device(torch, r)
    outs = []
    for _ in range(2):
        d_z = torch.empty_like(d_r)
        capi.apply_preconditioner_noalloc(d_a.data_ptr(), d_r.data_ptr(), n, d_z.data_ptr())
        outs.append(d_z.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])


def test_noalloc_rejects_sizes_beyond_its_scratch(env) -> None:
    torch, capi, _ = env
    d = torch.zeros(129 * 129, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="allocation-free range 1..128"):
        capi.apply_preconditioner_noalloc(d.data_ptr(), d.data_ptr(), 129, d.data_ptr())


def test_noalloc_reports_invalid_permeability(env) -> None:
    torch, capi, _ = env
    n = 16
    a = np.full((n, n), 2.0)
    a[2, 3] = -1.0
    d_a, d_r = device(torch, a), device(torch, np.ones((n, n)))
    d_z = torch.empty_like(d_r)
    with pytest.raises(ValueError, match=f"positive.*flat index {2 * n + 3}"):
        capi.apply_preconditioner_noalloc(d_a.data_ptr(), d_r.data_ptr(), n, d_z.data_ptr())
    # a valid call afterwards succeeds (the status word is reset per call)
    a[2, 3] = 2.0
    d_a = device(torch, a)
    capi.apply_preconditioner_noalloc(d_a.data_ptr(), d_r.data_ptr(), n, d_z.data_ptr())
    assert np.isfinite(d_z.cpu().numpy()).all()
