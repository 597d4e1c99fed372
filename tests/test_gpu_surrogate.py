"""The surrogate's tcgen05 kernels against plain PyTorch FP32 references of the same ops."""
import numpy as np
import pytest
import torch

from black_simulation_gb300 import bhk

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,splits", [
    (128, 256, 64, 1), (300, 256, 200, 1), (257, 64, 256, 1), (129, 16, 16, 1), (1000, 256, 256, 1),
    (256, 256, 4096, 8), (16, 256, 2048, 4),
])
def test_tc_gemm_matches_fp32_reference(cuda, M, N, K, splits):
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    C = bhk.tc_gemm(A, B, splits)
    ref = A.float() @ B.float().T
    err = (C - ref).abs().max().item() / max(1.0, ref.abs().max().item())
    assert err < 1e-5, err


# ------------------------------------------------------------------------ the surrogate network ----

def _batch(n, seed, device="cuda"):
    rng = np.random.default_rng(seed)
    x = np.stack([rng.uniform(0, 0.998, n), np.deg2rad(rng.uniform(5, 89, n)), rng.uniform(1.301, 3.0, n),
                  rng.uniform(-12, 12, n), rng.uniform(-12, 12, n)], axis=1).astype(np.float32)
    cls = rng.integers(0, 4, n).astype(np.uint8)
    tgt = np.zeros((n, 8), np.float32)
    tgt[:, 3] = rng.uniform(0.05, 1.0, n)
    tgt[:, 4] = rng.normal(0, 0.3, n)
    v = rng.normal(size=(n, 3))
    tgt[:, 5:8] = v / np.linalg.norm(v, axis=1, keepdims=True)
    t = lambda a: torch.from_numpy(a).to(device)
    return x, cls, tgt, t(x), t(cls), t(tgt)


@pytest.fixture(scope="module")
def sur(cuda):
    from black_simulation_gb300.surrogate import Surrogate
    s = Surrogate(0, seed=7, max_batch=2048)
    yield s
    s.close()


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("n", [128, 1024])
def test_gradients_match_cpu_fp64_network(sur, n):
    """The tcgen05 forward/backward chain against the CPU FP64 network with BF16 rounding emulated
    where the GPU stores BF16; per parameter tensor, relative Frobenius error <= 1e-2."""
    import surrogate_mlp as sm
    x, cls, tgt, xd, cd, td = _batch(n, 100 + n)
    w = (1.0, 3.0, 5.0, 7.0)
    sur.set_loss_weights(*w)
    g, loss = sur.gradients(xd, cd, td)
    p, B = sur.params(), sur.fourier()
    g_ref, terms = sm.gradients(p.astype(np.float64), B, x, cls, tgt, emulate_bf16=True, weights=w)
    assert np.allclose(loss, terms, rtol=2e-3, atol=1e-6), (loss, terms)
    offs = np.cumsum([0] + [fo * fi + fo for fo, fi in sm.LAYERS])
    for l, (fo, fi) in enumerate(sm.LAYERS):
        w0, b0, e = offs[l], offs[l] + fo * fi, offs[l + 1]
        assert _rel(g[w0:b0], g_ref[w0:b0]) < 1e-2, (l, "W", _rel(g[w0:b0], g_ref[w0:b0]))
        assert _rel(g[b0:e], g_ref[b0:e]) < 1e-2, (l, "b", _rel(g[b0:e], g_ref[b0:e]))
    # the padded head rows stay without gradient
    assert not np.any(g[offs[4] + 8 * 256:offs[4] + 16 * 256]) and not np.any(g[offs[5] - 8:offs[5]])
    # and against plain FP64 (no BF16): what BF16 storage costs the gradient
    g64, _ = sm.gradients(p.astype(np.float64), B, x, cls, tgt, weights=w)
    assert _rel(g, g64) < 5e-2


@pytest.fixture(scope="module")
def sur64(cuda):
    from black_simulation_gb300.surrogate import Surrogate
    s = Surrogate(0, seed=11, max_batch=2048, width=64)
    yield s
    s.close()


def test_width64_gradients_match_cpu_fp64_network(sur64):
    """The hidden-width-64 network through the same tcgen05 chain (N = 64 tiles, one K chunk per
    hidden layer) against the CPU FP64 network of that width, BF16 rounding emulated: <= 1e-2."""
    import surrogate_mlp as sm
    assert sur64.width == 64 and sur64.num_params() == sm.num_params(64)
    x, cls, tgt, xd, cd, td = _batch(1024, 77)
    w = (1.0, 3.0, 5.0, 7.0)
    sur64.set_loss_weights(*w)
    g, loss = sur64.gradients(xd, cd, td)
    p, B = sur64.params(), sur64.fourier()
    g_ref, terms = sm.gradients(p.astype(np.float64), B, x, cls, tgt, emulate_bf16=True, weights=w)
    assert np.allclose(loss, terms, rtol=2e-3, atol=1e-6), (loss, terms)
    offs = np.cumsum([0] + [fo * fi + fo for fo, fi in sm.layers(64)])
    for l, (fo, fi) in enumerate(sm.layers(64)):
        w0, b0, e = offs[l], offs[l] + fo * fi, offs[l + 1]
        assert _rel(g[w0:b0], g_ref[w0:b0]) < 1e-2, (l, "W", _rel(g[w0:b0], g_ref[w0:b0]))
        assert _rel(g[b0:e], g_ref[b0:e]) < 1e-2, (l, "b", _rel(g[b0:e], g_ref[b0:e]))
    y = sur64.predict(xd).cpu().numpy()
    Y, _ = sm.forward(p.astype(np.float64), B, x, emulate_bf16=True)
    assert np.abs(y - Y[:, :8]).max() <= 1e-2 * max(1.0, np.abs(Y[:, :8]).max())


def test_width_is_checked(cuda):
    from black_simulation_gb300 import bhk
    from black_simulation_gb300.surrogate import Surrogate
    with pytest.raises(ValueError):
        Surrogate(0, width=128)
    h = bhk.C.c_void_p()
    assert bhk.lib().bhk_surrogate_create_width(0, 1, 128, 128, bhk.C.byref(h)) == bhk.EINVAL


def test_predict_matches_cpu_forward(sur):
    import surrogate_mlp as sm
    x, _, _, xd, _, _ = _batch(3000, 9)   # more rows than the batch capacity, not a multiple of 128
    y = sur.predict(xd).cpu().numpy()
    Y, _ = sm.forward(sur.params().astype(np.float64), sur.fourier(), x, emulate_bf16=True)
    assert np.abs(y - Y[:, :8]).max() <= 1e-2 * max(1.0, np.abs(Y[:, :8]).max())


def test_params_round_trip(sur):
    p = sur.params()
    q = p.copy()
    q[:10] += 0.5
    sur.set_params(q)
    assert np.array_equal(sur.params(), q)
    sur.set_params(p)
    assert np.array_equal(sur.params(), p)


def test_invalid_batch_is_rejected(sur):
    from black_simulation_gb300 import bhk
    _, _, _, xd, cd, td = _batch(100, 1)   # not a multiple of 128
    with pytest.raises(bhk.BhkError):
        sur.gradients(xd, cd, td)


def test_training_on_traced_rays_reduces_loss(cuda, ctx):
    """A short run on rays the tracer labels: the loss falls and the held-out classification beats
    the class prior."""
    from black_simulation_gb300 import bhk
    from black_simulation_gb300.surrogate import Surrogate, inputs_from_rays, sample_rays, targets_from_rays
    rays = sample_rays(5 * 65536, seed=5)
    out = ctx.trace_rays(*rays, r_disk_in=0.0, r_disk_out=30.0, opts=bhk.TraceOpts("mixed"))
    torch.cuda.synchronize()
    x = inputs_from_rays(*rays)
    cls, tgt = targets_from_rays(out)
    n_train = 4 * 65536
    with Surrogate(0, seed=3, max_batch=65536) as s:
        hist = s.train(x[:n_train].contiguous(), cls[:n_train].contiguous(), tgt[:n_train].contiguous(),
                       batch=16384, steps=600, lr=1e-3)
        tot = hist.sum(axis=1)
        assert np.all(np.isfinite(tot))
        assert tot[-10:].mean() < 0.5 * tot[:3].mean(), (tot[:3], tot[-10:])
        y = s.predict(x[n_train:].contiguous())
        pred = y[:, :3].argmax(dim=1) + 1
        held = cls[n_train:].long()
        ok = held > 0
        acc = (pred[ok] == held[ok]).float().mean().item()
        prior = torch.bincount(held[ok]).max().item() / ok.sum().item()
        assert acc > prior + 0.2, (acc, prior)


@pytest.mark.parametrize("width", [256, 64])
def test_every_training_step_starts_from_zeroed_gradient_and_loss(cuda, width):
    """The optimiser step zeroes the gradient and the loss terms it has used, so that the next step
    accumulates from zero. Two steps on the same batch at a learning rate too small to move the BF16
    weights see the same gradient: the second step's loss terms equal the first's (not twice them), and
    Adam's first moment after them is (0.9 * 0.1 + 0.1) g = 1.9 times the one-step moment 0.1 g (2.9
    times, were the second gradient added to the first)."""
    from black_simulation_gb300.surrogate import Surrogate
    x, cls, tgt, xd, cd, td = _batch(1024, 31)
    with Surrogate(0, seed=5, max_batch=1024, width=width) as s:
        p0 = s.params()
        m0, v0, st0 = s.adam_state()
        h1 = s.train(xd, cd, td, batch=1024, steps=1, lr=1e-20)
        m1, _, _ = s.adam_state()
        s.set_params(p0)
        s.set_adam_state(m0, v0, st0)
        h2 = s.train(xd, cd, td, batch=1024, steps=2, lr=1e-20)
        m2, _, _ = s.adam_state()
    assert np.allclose(h2[1], h2[0], rtol=1e-4, atol=1e-7), h2
    assert np.allclose(h2[0], h1[0], rtol=1e-4, atol=1e-7), (h1, h2)
    big = np.abs(m1) > 1e-3 * np.abs(m1).max()
    assert big.sum() > 1000
    assert np.allclose(m2[big], 1.9 * m1[big], rtol=2e-3), np.abs(m2[big] / m1[big] - 1.9).max()


def test_checkpoint_round_trip(cuda, tmp_path):
    """Parameters, Fourier matrix and Adam state survive save/load; training resumes as before."""
    from black_simulation_gb300.surrogate import Surrogate
    x, cls, tgt, xd, cd, td = _batch(1024, 4)
    with Surrogate(0, seed=11, max_batch=1024) as a, Surrogate(0, seed=12, max_batch=1024) as b:
        a.train(xd, cd, td, batch=512, steps=5, lr=1e-3)
        a.save(str(tmp_path / "ck.npz"))
        b.load(str(tmp_path / "ck.npz"))
        assert np.array_equal(a.params(), b.params()) and np.array_equal(a.fourier(), b.fourier())
        ha = a.train(xd, cd, td, batch=512, steps=3, lr=1e-3)
        hb = b.train(xd, cd, td, batch=512, steps=3, lr=1e-3)
        # atomically summed bias gradients make the last bits order-dependent
        assert np.allclose(ha, hb, rtol=1e-4, atol=1e-7)
        assert np.allclose(a.params(), b.params(), rtol=1e-4, atol=1e-6)


def test_dataset_follows_the_training_distribution(cuda, ctx):
    """bhk_surrogate_dataset: inputs inside the stated ranges, (alpha, beta) within 1.5 x the shadow
    radius, and labels identical to tracing the same rays directly."""
    from black_simulation_gb300 import bhk
    from black_simulation_gb300.surrogate import make_dataset, shadow_radius, targets_from_rays
    n = 200_000
    x, cls, tgt, rays = make_dataset(ctx, n, seed=17, keep_rays=True)
    xs = x.cpu().numpy()
    assert xs[:, 0].min() >= 0 and xs[:, 0].max() <= 0.998
    assert np.deg2rad(5) - 1e-6 <= xs[:, 1].min() and xs[:, 1].max() <= np.deg2rad(89) + 1e-6
    assert np.log10(20) - 1e-6 <= xs[:, 2].min() and xs[:, 2].max() <= 3 + 1e-6
    # roughly uniform in log r and in a
    assert abs(np.median(xs[:, 2]) - 0.5 * (np.log10(20) + 3)) < 0.02
    rng = np.random.default_rng(0)
    for i in rng.choice(n, 25, replace=False):
        R = shadow_radius(float(rays[0, i]), float(rays[1, i]), float(rays[2, i]))
        rho = float(np.hypot(rays[3, i].item(), rays[4, i].item()))
        assert rho <= 1.5 * R * 1.01
    cnt = np.bincount(cls.cpu().numpy(), minlength=4)
    assert cnt[1] > 0.1 * n and cnt[2] > 0.1 * n and cnt[3] > 0.01 * n
    out = ctx.trace_rays(*[rays[k].contiguous() for k in range(5)], r_disk_in=0.0, r_disk_out=30.0,
                         opts=bhk.TraceOpts("mixed"))
    c2, t2 = targets_from_rays(out)
    assert torch.equal(c2, cls)
    assert torch.allclose(t2, tgt, rtol=1e-6, atol=1e-7)
