"""GPU field generator: same distribution as the host generator (the
reference's construction), deterministic per seed, independent of chunking;
and the dataset command on top of it."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import two_phase


@pytest.fixture(scope="module")
def capi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from darcy_cpp_gb300 import capi as c

    return c


def host_raw(n: int, count: int, seed: int) -> np.ndarray:
    from darcy_cpp_gb300.fields import gaussian_random_field

    rng = np.random.default_rng(seed)
    return np.stack([gaussian_random_field(n, seed=rng) for _ in range(count)])


def lag1(x: np.ndarray) -> tuple[float, float]:
    x = x - x.mean()
    v = (x * x).mean()
    return float((x[:, 1:, :] * x[:, :-1, :]).mean() / v), float((x[:, :, 1:] * x[:, :, :-1]).mean() / v)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [16, 32, 64])
def test_gpu_fields_follow_the_host_distribution(capi, n) -> None:
    count = 3000
    gpu = capi.random_fields(n, count, seed=7, raw=True)
    host = host_raw(n, count, seed=7)
    vg, vh = gpu.var(axis=0), host.var(axis=0)
    # per-pixel variance map (boundary structure of the DCT basis included)
    assert abs(vg.mean() / vh.mean() - 1) < 0.05
    assert np.abs(vg / vh - 1).mean() < 0.08
    # zero mean, same spatial correlation
    se = np.sqrt(vh.mean() / (count * n * n)) * 10
    assert abs(gpu.mean()) < max(se, 0.05 * np.sqrt(vh.mean()))
    for g, h in zip(lag1(gpu), lag1(host)):
        assert abs(g - h) < 0.02
    # the thresholded media: same phase fraction
    two = capi.random_fields(n, count, seed=7)
    assert set(np.unique(two)) <= {3.0, 12.0}
    host_frac = (host >= 0).mean()
    assert abs((two == 12.0).mean() - host_frac) < 0.02


@pytest.mark.gpu
def test_gpu_fields_are_deterministic_and_chunk_independent(capi) -> None:
    a = capi.random_fields(32, 5, seed=11)
    b = capi.random_fields(32, 5, seed=11)
    c = capi.random_fields(32, 3, seed=11)
    d = capi.random_fields(32, 5, seed=12)
    assert np.array_equal(a, b) and np.array_equal(a[:3], c)
    assert not np.array_equal(a, d)
    # many fields: the host copy runs in chunks; field q is the same either way
    big = capi.random_fields(128, 4200, seed=3)
    assert np.array_equal(big[:5], capi.random_fields(128, 5, seed=3))


@pytest.mark.gpu
def test_gpu_fields_validation(capi) -> None:
    for bad in (0, 129):
        with pytest.raises(capi.InvalidInput, match="side"):
            capi.random_fields(bad, 1)
    with pytest.raises(capi.InvalidInput, match="positive"):
        capi.random_fields(8, 1, hi=-1.0)


@pytest.mark.gpu
def test_dataset_command_writes_reference_format(capi, orc, tmp_path) -> None:
    """The dataset command (python/darcy/cli.py:77-115): the reference's field
    loop, npz(a, u) in float32, every u equal to the oracle's solution of its
    field after the same float32 cast (rtol 1e-6: the GPU solve is within
    ~1e-12 of the oracle's, so the casts differ by at most one float32 ulp)."""
    from darcy_cpp_gb300 import dataset

    out = tmp_path / "d.npz"
    assert dataset.main(["--n-samples", "6", "--grid", "24", "--seed", "4", "--output", str(out)]) == 0
    with np.load(out) as z:
        assert z["a"].dtype == np.float32 and z["u"].dtype == np.float32
        assert z["a"].shape == (6, 24, 24)
        # the reference's field loop: one shared stream
        assert np.array_equal(z["a"], dataset.draw_fields(6, 24, seed=4).astype(np.float32))
    fields = dataset.draw_fields(6, 24, seed=4)
    with np.load(out) as z:
        for q in range(6):
            want = orc.solve(fields[q], tol=1e-10)["u"]
            assert np.allclose(z["u"][q], want.astype(np.float32), rtol=1e-6, atol=0), q
    gpu = tmp_path / "g.npz"
    assert dataset.main(["--n-samples", "4", "--grid", "24", "--gpu-fields", "--output", str(gpu)]) == 0
    with np.load(gpu) as z:
        assert set(np.unique(z["a"])) <= {3.0, 12.0}
    # non-convergence fails the command (cli.py:97-100)
    assert dataset.main(["--n-samples", "2", "--grid", "24", "--max-iter", "1", "--output",
                         str(tmp_path / "x.npz")]) == 1


@pytest.mark.gpu
def test_benchmark_harness_rows_and_table(capi) -> None:
    from darcy_cpp_gb300 import benchmark

    rows = benchmark.run_benchmark(grids=[32], repeats=1, verbose=False)
    assert {(r.preconditioner, r.form) for r in rows} == {("multigrid", "fp64"), ("multigrid", "mixed"),
                                                         ("jacobi", "fp64")}
    for r in rows:
        assert r.relative_error is not None and r.relative_error < 1e-8
        assert r.seconds > 0 and r.iterations > 0
    batch = benchmark.run_batch(32, 64, repeats=1, verbose=False)
    table = benchmark.format_table(rows, batch)
    assert table.startswith("| grid | preconditioner | form | CG iters |")
    assert "| 64 x 32² |" in table
    data = benchmark.to_json(rows, batch)
    assert len(data["single"]) == 3 and data["batch"][0]["solves_per_s"] > 0
