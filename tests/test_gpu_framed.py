"""Per-ray cameras with arbitrary frames (bhk_trace_rays_framed): trajectory::traceRay's call shape,
including moving cameras and cameras inside the horizon, against the oracle and the reference's
own loop (tests/golden/framed_ref.npz)."""
import numpy as np
import pytest
import torch

import pyoracle as po
from black_simulation_gb300 import bhk

pytestmark = pytest.mark.gpu

KEYS = ("r_disk", "phi_disk", "g", "theta_inf", "phi_inf")


def _rays(g):
    cams, frames, looks = g["cameras"], g["frames"], g["looks"]
    nl = len(looks)
    rep = lambda col: np.repeat(cams[:, col], nl)
    arr = dict(a=rep(0), r=rep(1), theta=rep(2), phi=rep(3), r_in=rep(4),
               frames=np.repeat(frames, nl, axis=0), look=np.tile(looks, (len(cams), 1)))
    return arr


def _trace(ctx, g, opts):
    arr = _rays(g)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    outs = []
    # one call per camera (its own ISCO as the disk's inner edge)
    nl = len(g["looks"])
    for c in range(len(g["cameras"])):
        sl = slice(c * nl, (c + 1) * nl)
        o = ctx.trace_rays_framed(t(arr["a"][sl]), t(arr["r"][sl]), t(arr["theta"][sl]), t(arr["phi"][sl]),
                                  t(arr["frames"][sl]), t(arr["look"][sl]), r_disk_in=float(arr["r_in"][sl][0]),
                                  r_disk_out=20.0, opts=opts)
        torch.cuda.synchronize()
        outs.append({k: v.cpu().numpy() for k, v in o.items()})
    return {k: np.concatenate([o[k] for o in outs]) for k in outs[0]}


def _close(x, y, tol):
    both = ~np.isnan(x) & ~np.isnan(y)
    assert np.array_equal(np.isnan(x), np.isnan(y))
    return np.abs(x[both] - y[both]).max(initial=0.0) <= tol * max(1.0, np.abs(y[both]).max(initial=0.0))


def test_fp64_framed_matches_oracle_dp5(ctx, golden, oracle):
    """Same algorithm on both sides (FP64 Dormand-Prince, rtol 1e-10): identical outcomes, values to 1e-8."""
    g = golden("framed_ref.npz")
    got = _trace(ctx, g, bhk.TraceOpts("fp64", rtol=1e-10))
    arr = _rays(g)
    for i in range(len(arr["a"])):
        sc = po.Scene(arr["a"][i], arr["r"][i], arr["theta"][i], arr["phi"][i], arr["r_in"][i], 20.0, 1000.0, 1e-6,
                      1e-10, 20000, po.DP5)
        ray = oracle.trace_framed(sc, arr["frames"][i], arr["look"][i])
        assert got["outcome"][i] == ray.outcome, (i, got["outcome"][i], ray.outcome)
        for k in KEYS:
            w, x = getattr(ray, k), got[k][i]
            assert (np.isnan(w) and np.isnan(x)) or abs(x - w) <= 1e-8 * max(1.0, abs(w)), (i, k, x, w)


def test_fp64_framed_matches_reference_loop_fixture(ctx, golden):
    """Against the reference's own loop at tolerance 1e-4 (error ~1e-8): outcomes agree and disk radius,
    g and sky angles to 1e-6 (the bar of the FP64 mode)."""
    g = golden("framed_ref.npz")
    got = _trace(ctx, g, bhk.TraceOpts("fp64", rtol=1e-10))
    assert np.array_equal(got["outcome"], g["outcome"].astype(np.uint8))
    for k in KEYS:
        assert _close(got[k], g[k], 1e-6), k


def test_inside_horizon_rule_and_rise(ctx, golden):
    """Cameras inside the horizon: photons with 2 r_+ E - a L < 0 end captured with no step; the
    others are integrated back out through r_+ (some reach the disk or the sky)."""
    g = golden("framed_ref.npz")
    got = _trace(ctx, g, bhk.TraceOpts("fp64", rtol=1e-10))
    arr = _rays(g)
    rp = 1.0 + np.sqrt(1.0 - arr["a"] ** 2)
    inside = arr["r"] < rp
    assert inside.sum() == 80
    dead = inside & (got["steps"] == 0)
    assert dead.sum() > 0 and np.all(got["outcome"][dead] == bhk.CAPTURED)
    out_of_hole = inside & (got["outcome"] != bhk.CAPTURED)
    assert out_of_hole.sum() > 40 and np.all(got["steps"][out_of_hole] > 0)


def test_mixed_framed_against_fp64(ctx, golden):
    """Mixed precision (FP32 integration) on moving and inside-horizon cameras: outcomes agree with
    FP64 and the outputs to 1e-4."""
    g = golden("framed_ref.npz")
    ref = _trace(ctx, g, bhk.TraceOpts("fp64", rtol=1e-10))
    got = _trace(ctx, g, bhk.TraceOpts("mixed", rtol=1e-6))
    agree = got["outcome"] == ref["outcome"]
    assert agree.mean() >= 0.99, np.nonzero(~agree)
    for k in KEYS:
        assert _close(got[k][agree], ref[k][agree], 1e-4), k


def test_zamo_frame_equals_pinhole_call(ctx, golden, oracle):
    """A ZAMO frame with look = normalize(-1, -beta/r, alpha/r) is the pinhole of bhk_trace_rays."""
    n = 64
    rng = np.random.default_rng(2)
    a, r, th = 0.9, 30.0, np.deg2rad(70.0)
    al, be = rng.uniform(-12, 12, n), rng.uniform(-12, 12, n)
    fr = np.ctypeslib.as_array(oracle.zamo_frame(a, r, th).e).copy()
    lk = np.stack([-np.ones(n), -be / r, al / r], 1)
    lk /= np.linalg.norm(lk, axis=1, keepdims=True)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    opts = bhk.TraceOpts("fp64", rtol=1e-10)
    f = ctx.trace_rays_framed(t(np.full(n, a)), t(np.full(n, r)), t(np.full(n, th)), t(np.zeros(n)),
                              t(np.repeat(fr[None], n, axis=0)), t(lk), r_disk_out=20.0, opts=opts)
    p = ctx.trace_rays(t(np.full(n, a)), t(np.full(n, r)), t(np.full(n, th)), t(al), t(be), r_disk_out=20.0, opts=opts)
    torch.cuda.synchronize()
    assert torch.equal(f["outcome"], p["outcome"])
    for k in KEYS:
        assert _close(f[k].cpu().numpy(), p[k].cpu().numpy(), 1e-9), k


def test_framed_rejects_bad_arguments(ctx):
    z = torch.zeros(4, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        ctx.trace_rays_framed(z, z, z, z, torch.zeros(4, 4, dtype=torch.float64, device="cuda"),
                              torch.zeros(4, 3, dtype=torch.float64, device="cuda"))
    with pytest.raises(bhk.BhkError):
        ctx.trace_rays_framed(z, z, z, z, torch.zeros(4, 4, 4, dtype=torch.float64, device="cuda"),
                              torch.zeros(4, 3, dtype=torch.float64, device="cuda"), r_disk_out=-1.0)


def test_rayreport_fields_against_reference_traceRay(ctx, golden, oracle):
    """energy, gCamera, b, q, rMin, turns and delay of trajectory::traceRay's RayReport: traced with its
    own event settings (escape past 250 M, horizon r_+ + 0.01) in FP64, against the reference's values
    at its product tolerance 0.01 (so to that tolerance's accuracy for the step-sampled quantities)."""
    g = golden("framed_ref.npz")
    arr = _rays(g)
    nl = len(g["looks"])
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    outs = []
    for c in range(len(g["cameras"])):
        sl = slice(c * nl, (c + 1) * nl)
        rp = 1.0 + np.sqrt(1.0 - arr["a"][sl][0] ** 2)
        opts = bhk.TraceOpts("fp64", rtol=1e-10, r_escape=250.0, capture_eps=0.01 / rp)
        o = ctx.trace_rays_framed(t(arr["a"][sl]), t(arr["r"][sl]), t(arr["theta"][sl]), t(arr["phi"][sl]),
                                  t(arr["frames"][sl]), t(arr["look"][sl]), r_disk_in=float(arr["r_in"][sl][0]),
                                  r_disk_out=20.0, opts=opts, out=bhk.alloc_outputs(nl, "cuda", extras=True))
        torch.cuda.synchronize()
        outs.append({k: v.cpu().numpy() for k, v in o.items()})
    got = {k: np.concatenate([o[k] for o in outs]) for k in outs[0]}
    tv = g["tr_values"]
    end_map = np.array([bhk.ESCAPED, bhk.CAPTURED, bhk.DISK])
    want_end = end_map[g["tr_end"]]
    same = got["outcome"] == want_end
    assert same.mean() >= 0.99
    E = tv[:, 7]
    assert np.allclose(got["energy"], E, rtol=1e-12)
    assert np.allclose(got["g_camera"], 1.0 / E, rtol=1e-12)
    for i in range(len(E)):  # b, q against the oracle's launch of the same camera and look
        sc = po.Scene(arr["a"][i], arr["r"][i], arr["theta"][i], arr["phi"][i], arr["r_in"][i], 20.0, 1000.0, 1e-6,
                      1e-10, 10, po.DP5)
        ray = oracle.trace_framed(sc, arr["frames"][i], arr["look"][i])
        assert abs(got["b"][i] - ray.L / ray.E) <= 1e-12 * max(1.0, abs(ray.L / ray.E))
        assert abs(got["q"][i] - ray.Q / ray.E ** 2) <= 1e-11 * max(1.0, abs(ray.Q / ray.E ** 2))
    # rMin: ours is refined at the turning point, the reference's is the smallest step end. Where the
    # path is cut by an event (a capture, a disk crossing) both include the last step's end, and the
    # reference's coarse step reaches a little further past the event.
    ref_rmin = tv[:, 5]
    esc = same & (want_end == bhk.ESCAPED)
    assert np.all(got["r_min"][esc] <= ref_rmin[esc] * (1 + 1e-9))
    assert np.all(ref_rmin[esc] - got["r_min"][esc] <= 1e-2 * ref_rmin[esc] + 1e-3)
    cut = same & ~esc
    assert np.all(np.abs(got["r_min"][cut] - ref_rmin[cut]) <= 5e-2 * ref_rmin[cut])
    # turns: the same chord sum, finer steps; from inside the horizon the azimuth turns fast as the ray
    # rises through r_+, and the reference's coarse chords there are not converged, so compare outside
    # (rays that wind round the photon sphere are chaotic in their constants: compared below 3/4 turn)
    outside = same & (arr["r"] > 1.0 + np.sqrt(1.0 - arr["a"] ** 2))
    calm = outside & (tv[:, 6] < 0.75)
    assert calm.sum() > 100
    assert np.allclose(got["turns"][calm], tv[calm, 6], rtol=2e-2, atol=2e-3)
    assert np.all(np.isfinite(got["turns"][same])) and np.all(got["turns"][same] >= 0)
    # delay: disk crossings are interpolated in both; the reference reports escapes and captures at the
    # first step past the event (later, so longer)
    disk = calm & (want_end == bhk.DISK)
    assert np.allclose(got["delay"][disk], tv[disk, 8], rtol=2e-3)
    other = calm & (want_end != bhk.DISK) & (got["steps"] > 0)
    assert np.all(got["delay"][other] <= tv[other, 8] * (1 + 1e-6) + 1e-9)
    assert np.all(got["delay"][other] >= 0.8 * tv[other, 8] - 1e-9)


def test_mixed_mode_reports_rmin_but_not_delay(ctx, golden):
    g = golden("framed_ref.npz")
    arr = _rays(g)
    nl = len(g["looks"])
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x[:nl])).cuda()
    o = ctx.trace_rays_framed(t(arr["a"]), t(arr["r"]), t(arr["theta"]), t(arr["phi"]), t(arr["frames"]),
                              t(arr["look"]), r_disk_in=float(arr["r_in"][0]), r_disk_out=20.0,
                              opts=bhk.TraceOpts("mixed"), out=bhk.alloc_outputs(nl, "cuda", extras=True))
    torch.cuda.synchronize()
    assert torch.isfinite(o["r_min"]).all() and torch.isfinite(o["energy"]).all()
    assert torch.isnan(o["delay"]).all() and torch.isnan(o["turns"]).all()
