"""Surrogate + integrator-fallback rendering: the pixel-list tracer, the fused tcgen05 inference
kernel against the layer-by-layer network, and the fallback rules (confidence, critical-curve band)."""
import math

import numpy as np
import pytest
import torch

from black_simulation_gb300 import bhk
from black_simulation_gb300.surrogate import Surrogate, pixel_inputs, shadow_radius

pytestmark = pytest.mark.gpu

FIELDS_D = ("r_disk", "phi_disk", "g", "theta_inf", "phi_inf")


def _frame(width=192, height=108, theta_deg=60.0):
    th = math.radians(theta_deg)
    hw = 1.2 * shadow_radius(0.998, 30.0, th)
    return bhk.Frame(0.998, 30.0, th, width, height, -hw, hw, -hw * height / width, hw * height / width, 0.0, 30.0)


def _same(a, b):
    """Bitwise equality of float64 arrays with NaN == NaN."""
    return np.array_equal(a.view(np.int64), b.view(np.int64))


def test_trace_pixels_matches_full_frame(ctx):
    f = _frame()
    full = ctx.trace_frames([f], bhk.TraceOpts("mixed"))
    rng = np.random.default_rng(3)
    pix = np.sort(rng.choice(f.rays, 3000, replace=False)).astype(np.int32)
    sub = ctx.trace_pixels([f], torch.from_numpy(pix).cuda(), bhk.TraceOpts("mixed"))
    torch.cuda.synchronize()
    assert np.array_equal(sub["outcome"].cpu().numpy(), full["outcome"].cpu().numpy()[pix])
    for k in FIELDS_D:
        assert _same(sub[k].cpu().numpy(), full[k].cpu().numpy()[pix]), k
    assert np.array_equal(sub["steps"].cpu().numpy(), full["steps"].cpu().numpy()[pix])


def test_trace_pixels_over_two_frames(ctx):
    f1, f2 = _frame(64, 36, 80.0), _frame(48, 48, 50.0)
    full = ctx.trace_frames([f1, f2], bhk.TraceOpts("mixed"))
    pix = np.array([0, 5, f1.rays - 1, f1.rays, f1.rays + 777, f1.rays + f2.rays - 1], dtype=np.int32)
    sub = ctx.trace_pixels([f1, f2], torch.from_numpy(pix).cuda(), bhk.TraceOpts("mixed"))
    torch.cuda.synchronize()
    assert np.array_equal(sub["outcome"].cpu().numpy(), full["outcome"].cpu().numpy()[pix])
    assert _same(sub["g"].cpu().numpy(), full["g"].cpu().numpy()[pix])


def _train(ctx, width, seed):
    from black_simulation_gb300.surrogate import inputs_from_rays, sample_rays, targets_from_rays
    rays = sample_rays(8 * 65536, seed=21)
    out = ctx.trace_rays(*rays, r_disk_in=0.0, r_disk_out=30.0, opts=bhk.TraceOpts("mixed"))
    x = inputs_from_rays(*rays)
    cls, tgt = targets_from_rays(out)
    s = Surrogate(0, seed=seed, max_batch=65536, width=width)
    s.train(x, cls, tgt, batch=65536, steps=400, lr=1e-3)
    return s


@pytest.fixture(scope="module")
def trained(cuda, ctx):
    """A surrogate trained briefly on tracer labels around the test frames' poses."""
    s = _train(ctx, 256, 5)
    yield s
    s.close()


@pytest.fixture(scope="module")
def trained64(cuda, ctx):
    """The same with hidden width 64."""
    s = _train(ctx, 64, 6)
    yield s
    s.close()


@pytest.mark.parametrize("net", ["trained", "trained64"])
def test_fused_inference_matches_layerwise_network(ctx, request, net):
    trained = request.getfixturevalue(net)
    frames = [_frame(160, 90, 70.0), _frame(96, 96, 88.0)]
    out, st = trained.render(ctx, frames, p_min=0.0, band=0.0, fallback=False)
    assert st["rays"] == sum(f.rays for f in frames)
    x = torch.from_numpy(np.concatenate([pixel_inputs(f) for f in frames])).cuda()
    y = trained.predict(x).cpu().numpy().astype(np.float64)
    cls = y[:, :3].argmax(axis=1) + 1
    oc = out["outcome"].cpu().numpy()
    # classes agree except at near-ties (FP32 accumulation order differs between the two paths)
    srt = np.sort(y[:, :3], axis=1)
    clear = srt[:, 2] - srt[:, 1] > 1e-2
    assert np.array_equal(oc[clear], cls[clear])
    same = oc == cls
    disk = same & (cls == bhk.DISK)
    rd = out["r_disk"].cpu().numpy()
    assert np.allclose(rd[disk], 30.0 * y[disk, 3], rtol=1e-2, atol=2e-2)
    g = out["g"].cpu().numpy()
    assert np.allclose(g[disk], np.exp(y[disk, 4]), rtol=1e-2)
    esc = same & (cls == bhk.ESCAPED)
    v = y[esc, 5:8] / np.linalg.norm(y[esc, 5:8], axis=1, keepdims=True)
    th = out["theta_inf"].cpu().numpy()[esc]
    if esc.any():   # a camera at 30 M beside a disk out to 30 M sees few escaping rays
        assert np.abs(th - np.arccos(np.clip(v[:, 2], -1, 1))).max() < 1e-2
    assert np.all(out["steps"].cpu().numpy() == 0)
    assert np.all(np.isnan(out["phi_disk"].cpu().numpy()))


def test_untrained_network_falls_back_and_matches_tracer(ctx, cuda):
    """With an untrained network almost nothing is confident: the fallback rays carry exactly the
    tracer's results, the others the network's (steps 0)."""
    f = _frame(128, 72, 60.0)
    full = ctx.trace_frames([f], bhk.TraceOpts("mixed"))
    with Surrogate(0, seed=9, max_batch=128) as s:
        out, st = s.render(ctx, [f], bhk.TraceOpts("mixed"))
        fb = s.fallback_list().cpu().numpy()
    torch.cuda.synchronize()
    assert st["fallback"] == fb.size and st["fallback"] > 0.9 * f.rays
    assert np.unique(fb).size == fb.size and fb.min() >= 0 and fb.max() < f.rays
    assert np.array_equal(out["outcome"].cpu().numpy()[fb], full["outcome"].cpu().numpy()[fb])
    for k in FIELDS_D:
        assert _same(out[k].cpu().numpy()[fb], full[k].cpu().numpy()[fb]), k
    rest = np.setdiff1d(np.arange(f.rays), fb)
    assert np.all(out["steps"].cpu().numpy()[rest] == 0)


def test_band_rule_covers_the_critical_curve(ctx, trained, oracle):
    """Every pixel within 0.045 M of the analytic critical curve (the oracle's polyline) is handed to
    the integrator under the 0.05 M band rule; most pixels far from it are not."""
    f = _frame(384, 216, 60.0)
    out, st = trained.render(ctx, [f], p_min=0.0, band=0.05, fallback=False)
    fb = np.zeros(f.rays, bool)
    fb[trained.fallback_list().cpu().numpy()] = True
    ca, cb = oracle.critical_curve_finite(f.a, f.r_obs, f.theta_obs, samples=400)
    x = pixel_inputs(f).astype(np.float64)
    d = np.empty(f.rays)
    for i in range(0, f.rays, 1024):
        d[i:i + 1024] = band_distance(x[i:i + 1024, 3], x[i:i + 1024, 4], ca, cb)
    near = d < 0.045
    assert near.sum() > 100
    assert fb[near].all(), np.nonzero(near & ~fb)[0][:10]
    far = d > 0.08
    snap = np.abs(x[:, 3]) * math.sin(f.theta_obs) < 4e-3
    assert fb[far & ~snap].mean() < 1e-3


def band_distance(alpha, beta, ca, cb):
    import pyoracle
    return pyoracle.band_distance(alpha, beta, ca, cb)


def test_captured_only_acceptance_answers_exactly(ctx, trained):
    """accept="captured": the network answers only rays it classes captured (confident, outside the
    band); every other pixel carries exactly the tracer's results, and an accepted pixel has no
    continuous output, so it equals the tracer's wherever the tracer captured it too."""
    frames = [_frame(192, 108, 70.0), _frame(96, 96, 50.0)]
    full = ctx.trace_frames(frames, bhk.TraceOpts("mixed"))
    out, st = trained.render(ctx, frames, bhk.TraceOpts("mixed"), accept="captured")
    torch.cuda.synchronize()
    assert st["accept"] == 1
    n = sum(f.rays for f in frames)
    fb = np.zeros(n, bool)
    fb[trained.fallback_list().cpu().numpy()] = True
    oc, ref = out["outcome"].cpu().numpy(), full["outcome"].cpu().numpy()
    acc = ~fb
    assert acc.any() and np.all(oc[acc] == bhk.CAPTURED)
    assert np.all(out["steps"].cpu().numpy()[acc] == 0)
    assert np.array_equal(oc[fb], ref[fb])
    for k in FIELDS_D:
        o, r = out[k].cpu().numpy(), full[k].cpu().numpy()
        assert _same(o[fb], r[fb]), k
        assert np.all(np.isnan(o[acc])), k
    # the accepted answers agree with the tracer's outcome (a briefly trained network: >= 99 %)
    assert (ref[acc] == bhk.CAPTURED).mean() >= 0.99


def test_width64_network_renders_faster_than_the_tracer(ctx, cuda):
    """What the trained network gains over the tracer alone. A width-64 network trained on 8M rays
    the tracer labels renders 8 poses of the orbit sequence (1920 x 1080 each) with integrator fallback
    (class probability < 0.99 or within 0.05 M of the critical curve) in less time than the plain
    mixed tracer takes for the same pixels, CUDA events on one stream, medians of 5. The price is
    accuracy: where it answers, the network is ~1e-2 accurate (outcomes here >= 98.5 % the tracer's),
    while the fallback pixels carry exactly the tracer's outcomes."""
    from black_simulation_gb300.surrogate import Surrogate, make_dataset, orbit_frames
    x, cls, tgt = make_dataset(ctx, 8 * 1024 * 1024, seed=3)
    frames = orbit_frames(8, 1920, 1080)
    n = sum(f.rays for f in frames)
    opts = bhk.TraceOpts("mixed", rtol=1e-6)
    full = bhk.alloc_outputs(n, "cuda")
    out = bhk.alloc_outputs(n, "cuda")
    with Surrogate(0, seed=3, max_batch=65536, width=64) as s:
        s.train(x, cls, tgt, batch=65536, steps=6000, lr=1e-3)
        del x, cls, tgt

        def median_ms(fn):
            for _ in range(2):
                fn()
            torch.cuda.synchronize()
            ms = []
            for _ in range(5):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                fn()
                b.record()
                torch.cuda.synchronize()
                ms.append(a.elapsed_time(b))
            return float(np.median(ms))

        t_trace = median_ms(lambda: ctx.trace_frames(frames, opts, out=full))
        t_sur = median_ms(lambda: s.render(ctx, frames, opts, out=out))
        _, st = s.render(ctx, frames, opts, out=out)
        fb = s.fallback_list().cpu().numpy()
    torch.cuda.synchronize()
    oc, ref = out["outcome"].cpu().numpy(), full["outcome"].cpu().numpy()
    agree = float(np.mean(oc == ref))
    print(f"plain tracer {t_trace:.2f} ms, width-64 surrogate + fallback {t_sur:.2f} ms "
          f"({t_trace / t_sur:.2f}x), fallback {st['fallback'] / n:.3f}, outcome agreement {agree:.4f}")
    assert t_sur < 0.9 * t_trace
    assert agree >= 0.985
    assert np.array_equal(oc[fb], ref[fb])
