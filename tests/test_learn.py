"""Learned warm start: the network's kernels against a CPU float32 reference,
the tensor-core convolution against the CUDA-core one, training, and what the
trained network gains over a zero start (iterations to the same tolerance).

The CPU reference is the same network in torch (CPU, float32) with BF16
rounding applied where the GPU rounds: weights and inputs, each GELU output
in the forward pass, each pre-activation gradient in the backward pass. What
remains is float32 summation order, so gradients agree to ~1e-4 relative.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import two_phase

SIDE_CASES = [8, 16, 20, 48, 64, 128, 256]


def rel_l2(x, y) -> float:
    x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
    return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))


def fields(side: int, seeds) -> np.ndarray:
    return np.stack([two_phase(side, seed=int(s)) for s in seeds])


# ---------------------------------------------------------------- CPU side

def layer_shapes():
    cin = [2, 32, 32, 32, 32, 32]
    cout = [32, 32, 32, 32, 32, 1]
    return cin, cout


def split_params(w: np.ndarray):
    """Flat parameters -> per layer (weights [cout, cin, 3, 3], bias [cout])."""
    cin, cout = layer_shapes()
    out, at = [], 0
    for ci, co in zip(cin, cout):
        n = co * 9 * ci
        wl = w[at:at + n].reshape(co, 3, 3, ci).transpose(0, 3, 1, 2)  # [co][tap=(ky,kx)][ci]
        at += n
        bl = w[at:at + co]
        at += co
        out.append((wl, bl))
    assert at == w.size
    return out


def test_parameter_count_matches_the_layout() -> None:
    cin, cout = layer_shapes()
    assert sum(co * 9 * ci + co for ci, co in zip(cin, cout)) == 37_889


def energy(torch, e, a):
    """e^T A e per sample for the cell-centred operator of `a` (harmonic
    interior faces, the cell's own permeability on boundary faces)."""
    hx = 2 * a[:, :, 1:] * a[:, :, :-1] / (a[:, :, 1:] + a[:, :, :-1])
    hy = 2 * a[:, 1:, :] * a[:, :-1, :] / (a[:, 1:, :] + a[:, :-1, :])
    s = (hx * (e[:, :, 1:] - e[:, :, :-1]) ** 2).sum(dim=(1, 2))
    s = s + (hy * (e[:, 1:, :] - e[:, :-1, :]) ** 2).sum(dim=(1, 2))
    s = s + (a[:, :, 0] * e[:, :, 0] ** 2).sum(1) + (a[:, :, -1] * e[:, :, -1] ** 2).sum(1)
    s = s + (a[:, 0, :] * e[:, 0, :] ** 2).sum(1) + (a[:, -1, :] * e[:, -1, :] ** 2).sum(1)
    return s


def torch_reference(w, scaling, features, a, u, f=None, loss_kind="energy"):
    """Loss and parameter gradients of the network on the CPU (float32 with
    the GPU's BF16 rounding points)."""
    torch = pytest.importorskip("torch")
    F = torch.nn.functional

    class RoundFwd(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            return x.to(torch.bfloat16).to(torch.float32)

        @staticmethod
        def backward(ctx, g):
            return g

    class RoundBwd(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            return x.clone()

        @staticmethod
        def backward(ctx, g):
            return g.to(torch.bfloat16).to(torch.float32)

    mu, sd, us, fref = scaling
    count = a.shape[0]
    fs = np.ones(count) if f is None else np.asarray(f, dtype=np.float64)
    x = torch.tensor(np.ascontiguousarray(features.transpose(0, 3, 1, 2)))
    target = torch.tensor((u / (us * fs[:, None, None] / fref)).astype(np.float32))[:, None]
    params = []
    for wl, bl in split_params(np.asarray(w, dtype=np.float32)):
        wt = torch.tensor(np.ascontiguousarray(wl)).to(torch.bfloat16).to(torch.float32).requires_grad_(True)
        bt = torch.tensor(np.ascontiguousarray(bl)).requires_grad_(True)
        params.append((wt, bt))
    h = x
    for l, (wt, bt) in enumerate(params):
        pre = F.conv2d(h, wt, bt, padding=1)
        if l < 5:
            h = RoundFwd.apply(F.gelu(RoundBwd.apply(pre)))
        else:
            h = pre
    if loss_kind == "energy":
        at = torch.tensor(a.astype(np.float32))
        norm = energy(torch, target[:, 0], at).detach()
        loss = torch.mean(energy(torch, h[:, 0] - target[:, 0], at) / norm)
    else:
        loss = torch.mean((h - target) ** 2)
    loss.backward()
    grads = []
    for wt, bt in params:
        grads.append((wt.grad.numpy().transpose(0, 2, 3, 1).reshape(-1), bt.grad.numpy()))
    flat = np.concatenate([np.concatenate([gw, gb]) for gw, gb in grads])
    return float(loss.detach()), flat, h.detach().numpy()[:, 0]


def test_dataset_fields_follow_one_shared_stream() -> None:
    from darcy_cpp_gb300.dataset import draw_fields
    from darcy_cpp_gb300.fields import gaussian_random_field, two_phase_permeability

    a = draw_fields(3, 16, seed=5)
    rng = np.random.default_rng(5)
    want = np.stack([two_phase_permeability(gaussian_random_field(16, seed=rng)) for _ in range(3)])
    assert np.array_equal(a, want)
    assert set(np.unique(a)) <= {3.0, 12.0}


# ---------------------------------------------------------------- GPU side

@pytest.fixture(scope="module")
def learn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from darcy_cpp_gb300 import learn as L

    return L


def solved_pairs(learn, side, seeds):
    return learn.generate_pairs(list(seeds), side)


@pytest.mark.gpu
@pytest.mark.parametrize("side", SIDE_CASES)
def test_tensor_core_forward_matches_cuda_cores(learn, side) -> None:
    net = learn.WarmStartNet(side, seed=3)
    a = fields(side, range(4 if side <= 128 else 2))
    net.set_scaling([float(np.log(a).mean()), float(np.log(a).std()) or 1.0, 1e-2, 1.0])
    # random non-trivial weights so every layer contributes
    w = np.random.default_rng(side).standard_normal(net.num_params).astype(np.float32) * 0.2
    net.set_params(w)
    net.set_engine("simt")
    ref = net.predict(a)
    net.set_engine("tensor")
    got = net.predict(a)
    assert np.isfinite(got).all()
    assert rel_l2(got, ref) < 2e-3, rel_l2(got, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("engine, loss_kind", [("tensor", "energy"), ("simt", "energy"), ("tensor", "mse")])
def test_gradients_match_the_cpu_reference(learn, engine, loss_kind) -> None:
    side = 16
    a, u = solved_pairs(learn, side, range(40, 44))
    net = learn.WarmStartNet(side, seed=11)
    net.set_engine(engine)
    net.set_loss(loss_kind)
    w = net.params()
    w += np.random.default_rng(1).standard_normal(w.size).astype(np.float32) * 0.05  # biases non-zero too
    net.set_params(w)
    net.fit(a, u, steps=1, lr=1e-12)  # sets the scaling from the pairs; the update is negligible
    net.set_params(w)
    g, loss = net.gradients(a, u)
    ref_loss, ref_g, _ = torch_reference(w, net.scaling(), net.features(a), a, u, loss_kind=loss_kind)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss) + 1e-9, (loss, ref_loss)
    # per layer, relative to that layer's gradient norm
    at = 0
    cin, cout = layer_shapes()
    for l, (ci, co) in enumerate(zip(cin, cout)):
        n = co * 9 * ci + co
        err = rel_l2(g[at:at + n], ref_g[at:at + n])
        assert err < 2e-3, (l, err)
        at += n


def unit_solution(n: int) -> np.ndarray:
    """a = 1, f = 1 solution of the n x n grid by a dense solve, unit RMS."""
    m = n * n
    A = np.zeros((m, m))
    for i in range(n):
        for j in range(n):
            k = i * n + j
            A[k, k] = 4.0
            for di, dj in ((0, 1), (0, -1), (1, 0), (-1, 0)):
                if 0 <= i + di < n and 0 <= j + dj < n:
                    A[k, (i + di) * n + j + dj] = -1.0
    u = np.linalg.solve(A, np.full(m, 1.0 / (n + 1) ** 2)).reshape(n, n)
    return u / np.sqrt(np.mean(u * u))


@pytest.mark.gpu
def test_features_are_log_a_and_the_scaled_unit_solution(learn) -> None:
    side = 20
    a = fields(side, range(3))
    net = learn.WarmStartNet(side)
    net.set_scaling([1.5, 0.7, 1e-3, 2.0])
    fs = np.array([1.0, 2.0, 3.0])
    x = net.features(a, fs)
    bf = lambda v: np.asarray(v, dtype=np.float32)  # noqa: E731
    want0 = (np.log(a) - 1.5) / 0.7
    want1 = (fs / 2.0)[:, None, None] * unit_solution(side)[None]
    assert np.allclose(x[..., 0], bf(want0), rtol=2 ** -8, atol=1e-6)
    assert np.allclose(x[..., 1], bf(want1), rtol=2 ** -8, atol=1e-6)


@pytest.mark.gpu
def test_gradients_with_per_sample_forcing(learn) -> None:
    side = 32
    seeds = range(60, 63)
    a = fields(side, seeds)
    fs = np.array([1.0, 2.5, 0.5])
    import darcy_cpp_gb300 as darcy

    u = np.stack([darcy.solve(a[q], float(fs[q])).u for q in range(3)])
    net = learn.WarmStartNet(side, seed=2)
    net.fit(a, u, f=fs, steps=1, lr=1e-12)
    w = net.params()
    g, loss = net.gradients(a, u, f=fs)
    ref_loss, ref_g, _ = torch_reference(w, net.scaling(), net.features(a, fs), a, u, fs)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss) + 1e-9
    assert rel_l2(g, ref_g) < 2e-3


@pytest.mark.gpu
def test_training_reduces_the_loss_and_is_deterministic(learn) -> None:
    side = 32
    a, u = solved_pairs(learn, side, range(1000, 1512))
    losses = []
    params = []
    for _ in range(2):
        net = learn.WarmStartNet(side, seed=7)
        losses.append(net.fit(a, u, steps=150, batch=64, lr=1e-3, seed=3))
        params.append(net.params())
    first, again = losses
    assert np.isfinite(first).all()
    assert first[-10:].mean() < 0.2 * first[:10].mean(), (first[:10].mean(), first[-10:].mean())
    assert np.array_equal(first, again)
    assert np.array_equal(params[0], params[1])


@pytest.mark.gpu
def test_warm_start_saves_iterations_at_the_same_tolerance(learn, tmp_path) -> None:
    import darcy_cpp_gb300 as darcy

    side = 64
    a, u = solved_pairs(learn, side, range(10000, 12048))
    net = learn.WarmStartNet(side, seed=0)
    losses = net.fit(a, u, steps=400, batch=128, lr=1e-3)
    assert losses[-20:].mean() < losses[:20].mean()
    held = fields(side, range(30000, 30128))
    zero = darcy.solve_batch(held, 1.0, form="mixed")
    warm = learn.solve_batch_learned(net, held, 1.0, form="mixed")
    assert zero.all_converged and warm.all_converged
    assert (warm.residuals < 1e-10).all()
    # same answer as the FP64 zero start to the solver's accuracy
    ref = darcy.solve_batch(held, 1.0, form="fp64")
    for q in range(0, 128, 17):
        assert rel_l2(warm.u[q], ref.u[q]) < 1e-9
    # the prediction is a better start than zero: fewer iterations on average
    assert warm.iterations.mean() < zero.iterations.mean(), (warm.iterations.mean(), zero.iterations.mean())
    # the prediction alone is already close (relative L2 error of u0)
    u0 = net.predict(held)
    err = np.mean([rel_l2(u0[q], ref.u[q]) for q in range(held.shape[0])])
    assert err < 0.2, err
    # weights file round trip gives the same prediction
    path = tmp_path / "warm.npz"
    net.save(path)
    net2 = learn.WarmStartNet.load(path)
    assert np.array_equal(net2.predict(held[:4]), u0[:4])


@pytest.mark.gpu
def test_learned_batch_equals_host_warm_start(learn) -> None:
    import darcy_cpp_gb300 as darcy

    side = 64
    a, u = solved_pairs(learn, side, range(500, 756))
    net = learn.WarmStartNet(side, seed=1)
    net.fit(a, u, steps=40, batch=64)
    held = fields(side, range(900, 932))
    u0 = net.predict(held)
    host = darcy.solve_batch(held, 1.0, form="fp64", x0=u0)
    dev = learn.solve_batch_learned(net, held, 1.0, form="fp64")
    # same start, same solver; the two calls may run different autotuned block
    # shapes, which only reorders reductions
    assert np.abs(host.iterations - dev.iterations).max() <= 1
    for q in range(held.shape[0]):
        assert rel_l2(dev.u[q], host.u[q]) < 1e-10


@pytest.mark.gpu
def test_network_validation(learn) -> None:
    from darcy_cpp_gb300 import capi

    for bad_side in (6, 7, 33, 514):
        with pytest.raises(ValueError, match="side"):
            learn.WarmStartNet(bad_side)
    net = learn.WarmStartNet(32)
    with pytest.raises(ValueError, match="scaling"):
        net.predict(np.ones((1, 32, 32)))
    with pytest.raises(ValueError, match="shape"):
        net.fit(np.ones((2, 16, 16)), np.ones((2, 16, 16)))
    net.handle.load_pairs(np.ones((2, 32, 32)), np.ones((2, 32, 32)))
    with pytest.raises(ValueError, match="batch larger"):
        net.handle.train(1, batch=4)
    with pytest.raises(ValueError, match="permeability"):
        bad = np.ones((2, 32, 32))
        bad[1, 3, 4] = -1.0
        net2 = learn.WarmStartNet(32)
        net2.fit(bad, np.ones((2, 32, 32)), steps=1, batch=1)
    with pytest.raises(ValueError, match="parameters"):
        net.set_params(np.zeros(5, dtype=np.float32))
    with pytest.raises(ValueError, match="another grid side"):
        learn.solve_batch_learned(net, np.ones((1, 64, 64)))
    with pytest.raises(capi.InvalidInput, match="learning rate"):
        net.handle.train(1, 1, lr=0.0)


@pytest.mark.gpu
def test_mma_wait_that_runs_out_reports_timeout_and_the_net_recovers(learn) -> None:
    """The tensor-core convolution's bounded MMA-completion wait: with its
    first wait given no polls (test hook), every CTA records the lost wait,
    drains its MMA in flight with the full budget, frees its tensor memory and
    returns; the call reports DGPU_TIMEOUT. The context stays usable: with the
    default budget restored the prediction equals the one before, bit for bit,
    and the solver still runs."""
    from darcy_cpp_gb300 import capi

    side = 32
    net = learn.WarmStartNet(side, seed=7)
    a = fields(side, range(3))
    net.set_scaling([float(np.log(a).mean()), float(np.log(a).std()) or 1.0, 1e-2, 1.0])
    net.set_params(np.random.default_rng(1).standard_normal(net.num_params).astype(np.float32) * 0.2)
    before = net.predict(a)
    net.handle.set_first_wait(0)
    with pytest.raises(capi.DarcyGpuError, match=f"status {capi.TIMEOUT}: .*wait ran out"):
        net.predict(a)
    net.handle.set_first_wait(1 << 24)
    after = net.predict(a)
    assert np.array_equal(before, after)
    with pytest.raises(capi.InvalidInput, match="polls"):
        net.handle.set_first_wait(-1)
    import darcy_cpp_gb300 as darcy

    assert darcy.solve(a[0]).converged


@pytest.mark.gpu
def test_learned_start_no_better_than_zero_falls_back_to_zero(learn) -> None:
    """A predicted start no better than zero is replaced by the zero start in
    the batched solve (the fallback it is judged against; the test is the
    start's estimated energy-norm error r0 . M r0 against the solution's
    estimated energy b . u0): with predictions ~1e3 times too large, every
    problem takes the zero start's iterations and ends at its solution."""
    import darcy_cpp_gb300 as darcy

    side = 32
    a = fields(side, range(6))
    net = learn.WarmStartNet(side, seed=5)
    net.set_scaling([float(np.log(a).mean()), float(np.log(a).std()) or 1.0, 1e3, 1.0])
    net.set_params(np.random.default_rng(2).standard_normal(net.num_params).astype(np.float32) * 0.2)
    u0 = net.predict(a)
    b = np.full((side, side), 1.0 / (side + 1) ** 2)
    for q in range(len(a)):
        assert np.linalg.norm(b - darcy.apply_operator(a[q], u0[q])) > np.linalg.norm(b)
    warm = learn.solve_batch_learned(net, a, tol=1e-10, form="mixed")
    zero = darcy.solve_batch(a, tol=1e-10, form="mixed")
    assert warm.all_converged
    assert np.array_equal(warm.iterations, zero.iterations)
    for q in range(len(a)):
        assert rel_l2(warm.u[q], zero.u[q]) < 1e-12
