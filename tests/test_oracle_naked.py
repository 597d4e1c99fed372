"""Naked singularities (|a| > 1) in the oracle: the radii against the reference's own values, the
reference's known-answer checks (tests/test_kerr.cpp:2456-2507) restated on the oracle's per-step
functions, and the oracle's tracers against frames the reference loop traced with the renderer's
rules for a spacetime without a horizon (shaders/trace.frag:1768-1787): no capture, the ring
singularity where Sigma < 4e-4, and the sky of the r < 0 region beyond the ring's disk."""
import math

import numpy as np
import pytest

import pyoracle as po

FRAMES = [0, 1, 2]


def _scene(g, i, method, tol, max_steps=200000):
    sc = g[f"f{i}_scene"]
    return po.scene(a=sc[0], r_obs=sc[1], theta_obs_deg=math.degrees(sc[2]), r_disk_out=sc[5], tol=tol,
                    method=method, max_steps=max_steps)


def _frame(g, i):
    return {k[len(f"f{i}_"):]: g[k] for k in g.keys() if k.startswith(f"f{i}_")}


def interior(outcome, w, h):
    """Pixels whose four neighbours share their outcome: away from the boundaries between outcomes,
    where a ray's fate depends on the step sequence (the ring, the edge of the ring's disk)."""
    o = outcome.reshape(h, w)
    m = np.ones_like(o, bool)
    m[1:, :] &= o[1:, :] == o[:-1, :]
    m[:-1, :] &= o[:-1, :] == o[1:, :]
    m[:, 1:] &= o[:, 1:] == o[:, :-1]
    m[:, :-1] &= o[:, :-1] == o[:, 1:]
    return m.ravel()


def test_naked_radii_match_reference(oracle, golden):
    g = golden("naked_ref.npz")
    for a, isco, ph in zip(g["spins"], g["isco"], g["photon_orbit"]):
        np.testing.assert_allclose([oracle.isco_radius_raw(a, 1), oracle.isco_radius_raw(a, 0)], isco, rtol=1e-12)
        np.testing.assert_allclose([oracle.photon_orbit_radius_raw(a, 1), oracle.photon_orbit_radius_raw(a, 0)], ph,
                                   rtol=1e-12)
        assert oracle.horizon_radius_raw(a) == 0.0


def _circular_energy(a, r):
    """Closed-form energy of the prograde circular equatorial orbit (Bardeen, Press & Teukolsky 1972)."""
    q = math.sqrt(r)
    return (r * q - 2 * q + a) / (r ** 0.75 * math.sqrt(r * q - 3 * q + 2 * a))


def test_naked_known_answers(oracle):
    """testNakedSingularity's closed-form checks (tests/test_kerr.cpp:2457-2483) at a = 1.2."""
    a, b = 1.2, math.sqrt(1.2 ** 2 - 1)
    r = np.arange(-20.0, 20.0, 0.001)
    assert abs(np.min(r * r - 2 * r + a * a) - b * b) < 1e-9
    rph = oracle.photon_orbit_radius_raw(a, 0)
    assert abs(rph * (rph - 3) ** 2 - 4 * a * a) < 1e-10
    assert oracle.photon_orbit_radius_raw(a, 1) == 0.0
    ri, h = oracle.isco_radius_raw(a, 1), 1e-4
    assert abs((_circular_energy(a, ri + h) - _circular_energy(a, ri - h)) / (2 * h)) < 1e-6
    e = _circular_energy(a, ri)
    assert e < _circular_energy(a, 0.9 * ri) and e < _circular_energy(a, 1.1 * ri) and ri < 1.0


def test_ray_through_the_ring_disk_comes_out_at_negative_r(oracle):
    """tests/test_kerr.cpp:2484-2506 on the oracle's per-step functions: a Q < 0 photon through the
    ring's disk reaches r <= -8 away from the ring, keeping vr^2 = R and vtheta^2 = Theta."""
    a = 1.2
    c = po.Constants(1.0, 0.0, -1.2, 0.0)
    s = po.State(0.0, 8.0, 0.3, 0.0, 0.0, 0.0)
    s.vr = -math.sqrt(oracle.radial_potential_raw(a, c, s.r))
    s.vtheta = math.sqrt(max(oracle.polar_potential_raw(a, c, s.theta), 0.0))
    least, drift = 1e30, 0.0
    for _ in range(200000):
        if not (-8.0 < s.r < 1e3):
            break
        s = oracle.step_mino(a, c, s, oracle.photon_step_size(a, c, s, 0.005))
        s = oracle.enforce_constraints(a, c, s)
        s = oracle.normalize_angles(s)
        cs = math.cos(s.theta)
        least = min(least, s.r * s.r + a * a * cs * cs)
        R, Th = oracle.radial_potential_raw(a, c, s.r), oracle.polar_potential_raw(a, c, s.theta)
        drift = max(drift, abs(s.vr ** 2 - R) / (1 + abs(R)), abs(s.vtheta ** 2 - Th) / (1 + abs(Th)))
    assert s.r <= -8.0 and least > 0.05
    assert drift < 1e-6


@pytest.mark.parametrize("i", FRAMES)
def test_dp5_oracle_matches_reference_naked_frames(oracle, golden, i):
    """The FP64 Dormand-Prince tracer against the reference loop at tolerance 1e-4: the same outcome
    away from outcome boundaries, r_disk and g to 1e-6, both skies' exit angles to 1e-6 rad."""
    g = golden("naked_ref.npz")
    f = _frame(g, i)
    w, h = int(f["width"]), int(f["height"])
    out = oracle.trace_frame(_scene(g, i, po.DP5, 1e-10), w, h, *f["extents"])
    inner = interior(f["outcome"], w, h)
    assert inner.mean() > 0.8
    np.testing.assert_array_equal(out["outcome"][inner], f["outcome"][inner].astype(np.int32))
    assert np.all(np.isin(out["outcome"], (po.DISK, po.ESCAPED, po.ESCAPED_BEYOND, po.RING)))
    d = (out["outcome"] == po.DISK) & (f["outcome"] == po.DISK)
    if d.any():
        assert np.max(np.abs(out["r_disk"][d] / f["r_disk"][d] - 1)) < 1e-6
        assert np.max(np.abs(out["g"][d] / f["g"][d] - 1)) < 1e-6
    for sky in (po.ESCAPED, po.ESCAPED_BEYOND):
        e = (out["outcome"] == sky) & (f["outcome"] == sky)
        if e.any():
            assert np.max(np.abs(out["theta_inf"][e] - f["theta_inf"][e])) < 1e-6
            assert np.max(np.abs(np.angle(np.exp(1j * (out["phi_inf"][e] - f["phi_inf"][e]))))) < 1e-6


def test_naked_frames_show_both_skies_and_the_ring(golden):
    g = golden("naked_ref.npz")
    counts = sum(np.bincount(g[f"f{i}_outcome"], minlength=6) for i in FRAMES)
    assert counts[po.CAPTURED] == 0 and counts[po.UNFINISHED] == 0
    assert counts[po.ESCAPED_BEYOND] > 100 and counts[po.RING] >= 1 and counts[po.DISK] > 1000


def test_rk4_restatement_bit_exact_on_naked_rays(oracle, golden):
    """The oracle's RK4 loop with the naked rules gives the reference's numbers bit for bit (sampled
    rays of the no-disk frame: both skies)."""
    g = golden("naked_ref.npz")
    f = _frame(g, 2)
    w, h = int(f["width"]), int(f["height"])
    al, be = po.pixel_grid(w, h, *f["extents"])
    beyond = np.nonzero(f["outcome"] == po.ESCAPED_BEYOND)[0][:4]
    idx = np.concatenate([np.arange(0, w * h, 211), beyond])
    sc = _scene(g, 2, po.RK4, 1e-4, max_steps=5_000_000)
    n = len(idx)
    out = oracle.trace_rays(sc, np.full(n, sc.a), np.full(n, sc.r_obs), np.full(n, sc.theta_obs), al[idx], be[idx])
    np.testing.assert_array_equal(out["outcome"], f["outcome"][idx])
    for k in ("theta_inf", "phi_inf"):
        np.testing.assert_array_equal(out[k], f[k][idx])
