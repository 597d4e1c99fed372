"""Pins the oracle (oracle/kerr_oracle.c) to the reference before it is trusted as the checker.

Golden vectors come from the reference's own kerr.cpp / trajectory.cpp / eht.cpp / central.cpp
(tests/golden/make_golden.py). Where the reference library itself is present (this container),
the restatement is also compared with it directly, bit for bit.
"""
import math

import numpy as np
import pytest

import pyoracle as po


def _st(row):
    return po.State(*row)


def _c(row):
    return po.Constants(*row)


def test_per_step_functions_match_reference_vectors(oracle, golden):
    g = golden("steps_ref.npz")
    for i in range(len(g["a"])):
        a, c, s = g["a"][i], _c(g["cons"][i]), _st(g["state"][i])
        d = oracle.derivatives(a, c, s)
        np.testing.assert_array_equal([d.dt, d.dr, d.dtheta, d.dphi, d.dvr, d.dvtheta], g["derivatives"][i])
        x = oracle.step_mino(a, c, s, g["h"][i])
        np.testing.assert_array_equal([x.t, x.r, x.theta, x.phi, x.vr, x.vtheta], g["step_mino"][i])
        assert oracle.photon_step_size(a, c, s, g["tol"][i]) == g["step_size"][i]
        x = oracle.enforce_constraints(a, c, s)
        np.testing.assert_array_equal([x.t, x.r, x.theta, x.phi, x.vr, x.vtheta], g["enforced"][i])
        row = g["state"][i].copy()
        row[2] *= 3.0
        x = oracle.normalize_angles(_st(row))
        np.testing.assert_array_equal([x.t, x.r, x.theta, x.phi, x.vr, x.vtheta], g["normalized"][i])


def test_frames_photons_and_zamo_launch_match_reference(oracle, golden):
    g = golden("steps_ref.npz")
    for i in range(len(g["frame_a"])):
        a, r, th = g["frame_a"][i], g["frame_r"][i], g["frame_theta"][i]
        f = oracle.zamo_frame(a, r, th)
        got = np.array([[f.e[k][j] for j in range(4)] for k in range(4)])
        np.testing.assert_array_equal(got, g["frames"][i])
        c, s = oracle.photon_from_frame(a, r, th, 0.25, f, g["look"][i])
        np.testing.assert_array_equal([c.E, c.L, c.Q, c.mu], g["photon_cons"][i])
        np.testing.assert_array_equal([s.t, s.r, s.theta, s.phi, s.vr, s.vtheta], g["photon_state"][i])
        c, s = oracle.launch_from_zamo(a, r, th, 0.0, g["zamo_v"][i], 0.0)
        np.testing.assert_array_equal([c.E, c.L, c.Q, c.mu], g["zamo_cons"][i])
        np.testing.assert_array_equal([s.t, s.r, s.theta, s.phi, s.vr, s.vtheta], g["zamo_state"][i])


def test_radii_and_critical_curves_match_reference(oracle, golden):
    g = golden("steps_ref.npz")
    for spin, row in zip(g["spins"], g["radii"]):
        got = [oracle.horizon_radius_raw(spin), oracle.isco_radius_raw(spin, 1), oracle.isco_radius_raw(spin, 0),
               oracle.photon_orbit_radius_raw(spin, 1), oracle.photon_orbit_radius_raw(spin, 0)]
        np.testing.assert_array_equal(got, row)
    assert len(g["cc_params"]) == 5
    for i, (sa, incl) in enumerate(g["cc_params"]):
        al, be = oracle.critical_curve(sa, incl, 400)
        np.testing.assert_array_equal(al, g[f"cc{i}_alpha"])
        np.testing.assert_array_equal(be, g[f"cc{i}_beta"])


def test_known_answers_radii():
    # testRadii (tests/test_kerr.cpp:65-81): closed forms.
    o = po.Oracle()
    assert abs(o.horizon_radius_raw(0.0) - 2.0) < 1e-14
    assert abs(o.horizon_radius_raw(0.6) - 1.8) < 1e-14
    assert abs(o.isco_radius_raw(0.0, 1) - 6.0) < 1e-12
    assert abs(o.isco_radius_raw(0.5, 1) - 4.233003) < 1e-5
    assert abs(o.isco_radius_raw(1.0, 1) - 1.0) < 1e-12
    assert abs(o.isco_radius_raw(1.0, 0) - 9.0) < 1e-12
    assert abs(o.photon_orbit_radius_raw(0.0, 1) - 3.0) < 1e-12
    assert abs(o.photon_orbit_radius_raw(1.0, 0) - 4.0) < 1e-12


def test_rk4_loop_reproduces_reference_traceRay(oracle, golden):
    """With traceRay's own settings (tolerance 0.01, horizon r_+ + 0.01, escape max(250, 1.5 r)),
    the oracle's RK4 loop ends every ray as src/trajectory.cpp:214-396 does, at the same radius and g."""
    g = golden("trajectory_ref.npz")
    end_map = {1: po.CAPTURED, 2: po.DISK, 0: po.ESCAPED}  # RayEnd: Sky=0, Horizon=1, Disk=2
    for i in range(len(g["a"])):
        a, r, th = g["a"][i], g["r"][i], g["theta"][i]
        rp = oracle.horizon_radius_raw(a)
        sc = po.Scene(a, r, th, 0.0, g["r_in"][i], 20.0, 250.0, 0.01 / rp, 0.01, 200000, po.RK4)
        look = g["look"][i]
        # pinhole look = normalize(-1, -beta/r, alpha/r)  =>  alpha = r l_phi / -l_r, beta = r l_theta / l_r
        alpha = r * look[2] / -look[0]
        beta = r * look[1] / look[0]
        ray = oracle.trace_ray(sc, alpha, beta)
        want = end_map[int(g["end"][i])]
        assert ray.outcome == want, (i, ray.outcome, want)
        if want == po.DISK:
            assert abs(ray.r_disk - g["values"][i][0]) < 1e-9 * max(1.0, g["values"][i][0])
            assert abs(ray.g - g["values"][i][1]) < 1e-9


def test_rk4_at_1e4_matches_reference_frame_fixture(oracle, golden):
    """The restated RK4 loop at tolerance 1e-4 gives the reference fixture's numbers bit for bit
    (sampled rays; the full frame is the fixture)."""
    g = golden("c1_rk4_1e-4.npz")
    w, h = int(g["width"]), int(g["height"])
    ext = g["extents"]
    al, be = po.pixel_grid(w, h, *ext)
    idx = np.arange(0, w * h, 331)
    sc = po.scene(a=0.9, r_obs=50.0, theta_obs_deg=80.0, r_disk_out=20.0, tol=1e-4, method=po.RK4,
                  max_steps=5_000_000)
    out = oracle.trace_rays(sc, np.full(len(idx), 0.9), np.full(len(idx), 50.0), np.full(len(idx), sc.theta_obs),
                            al[idx], be[idx])
    np.testing.assert_array_equal(out["outcome"], g["outcome"][idx])
    for k in ("r_disk", "phi_disk", "g", "theta_inf", "phi_inf"):
        np.testing.assert_array_equal(out[k], g[k][idx])


def _band(oracle, frame_npz, a, r_obs, theta):
    w, h = int(frame_npz["width"]), int(frame_npz["height"])
    al, be = po.pixel_grid(w, h, *frame_npz["extents"])
    ca, cb = oracle.critical_curve_finite(a, r_obs, theta, 800)
    return po.band_distance(al, be, ca, cb)


@pytest.mark.parametrize("name,a,r_obs,deg,r_out", [
    ("c1_rk4_1e-4.npz", 0.9, 50.0, 80.0, 20.0),
    ("c2_rk4_1e-4.npz", 0.998, 1000.0, 60.0, 30.0),
])
def test_dp5_oracle_matches_reference_rk4(oracle, golden, name, a, r_obs, deg, r_out):
    """The FP64 Dormand-Prince tracer (what the GPU FP64 mode implements) against the reference RK4
    at tolerance 1e-4: 100% outcome agreement outside 1e-3 M of the critical curve, r_disk and g
    to 1e-6 relative, exit angles to 1e-6 rad."""
    g = golden(name)
    w, h = int(g["width"]), int(g["height"])
    sc = po.scene(a=a, r_obs=r_obs, theta_obs_deg=deg, r_disk_out=r_out, tol=1e-10, method=po.DP5)
    out = oracle.trace_frame(sc, w, h, *g["extents"])
    band = _band(oracle, g, a, r_obs, math.radians(deg))
    outside = band > 1e-3
    assert outside.mean() > 0.99
    np.testing.assert_array_equal(out["outcome"][outside], g["outcome"][outside].astype(np.int32))
    d = (out["outcome"] == po.DISK) & (g["outcome"] == po.DISK)
    assert np.max(np.abs(out["r_disk"][d] / g["r_disk"][d] - 1)) < 1e-6
    assert np.max(np.abs(out["g"][d] / g["g"][d] - 1)) < 1e-6
    dphi = np.angle(np.exp(1j * (out["phi_disk"][d] - g["phi_disk"][d])))
    assert np.max(np.abs(dphi)) < 1e-6
    e = (out["outcome"] == po.ESCAPED) & (g["outcome"] == po.ESCAPED)
    if e.any():
        assert np.max(np.abs(out["theta_inf"][e] - g["theta_inf"][e])) < 1e-6
        assert np.max(np.abs(np.angle(np.exp(1j * (out["phi_inf"][e] - g["phi_inf"][e]))))) < 1e-6
    assert out["steps"].max() < 20000


def test_finite_critical_curve_tends_to_bardeen(oracle):
    """The pinhole critical curve at r_obs -> infinity is eht::criticalCurve (src/eht.cpp:52-80)."""
    for a, deg in ((0.9, 60.0), (0.5, 17.0)):
        th = math.radians(deg)
        fa, fb = oracle.critical_curve_finite(a, 1e7, th, 400)
        ba, bb = oracle.critical_curve(a, th, 400)
        assert np.max(np.abs(fa - ba)) < 1e-4 and np.max(np.abs(fb - bb)) < 1e-4


def test_capture_zone_test_agrees_with_sampling(oracle):
    rng = np.random.default_rng(5)
    for _ in range(300):
        a = rng.uniform(0, 0.998)
        E, L, Q = 1.0, rng.uniform(-7, 7), rng.uniform(-1, 30)
        rp = oracle.horizon_radius_raw(a)
        r = rp + rng.uniform(0.001, 0.05)
        proven = oracle.no_radial_root_below_raw(a, E, L, Q, r, 1e-6)
        xs = np.linspace(rp * (1 + 1e-6), r, 2001)
        c = po.Constants(E, L, Q, 0.0)
        Rs = np.array([oracle.radial_potential_raw(a, c, x) for x in xs])
        if proven:  # a "no root" answer must never be wrong
            assert Rs.min() > 0


@pytest.mark.skipif(not po.reference_available(), reason="reference library not built here")
def test_restatement_bit_exact_against_reference_library(oracle):
    R = po.Oracle(reference=True)
    sc = po.scene(tol=1e-2, method=po.RK4)
    o1 = oracle.trace_frame(sc, 24, 24, -15, 15, -15, 15)
    o2 = R.trace_frame(sc, 24, 24, -15, 15, -15, 15)
    for k in o1:
        np.testing.assert_array_equal(o1[k], o2[k])


def test_framed_launch_reproduces_reference_loop(oracle, golden):
    """Cameras with arbitrary frames (ZAMO, boosted, free-falling inside the horizon): the oracle's
    photonFromFrame launch, inside-horizon rule and RK4 loop at tolerance 1e-4 give the reference's
    numbers bit for bit."""
    g = golden("framed_ref.npz")
    looks = g["looks"]
    i = 0
    for cam, fr in zip(g["cameras"], g["frames"]):
        a, r, th, ph, r_in = cam
        sc = po.Scene(a, r, th, ph, r_in, 20.0, 1000.0, 1e-6, 1e-4, 5_000_000, po.RK4)
        for lk in looks:
            ray = oracle.trace_framed(sc, fr, lk)
            assert ray.outcome == g["outcome"][i], (i, ray.outcome, g["outcome"][i])
            for k in ("r_disk", "phi_disk", "g", "theta_inf", "phi_inf"):
                want = g[k][i]
                got = getattr(ray, k)
                assert (np.isnan(want) and np.isnan(got)) or got == want, (i, k, got, want)
            i += 1


def test_framed_rk4_reproduces_reference_traceRay(oracle, golden):
    """With traceRay's own settings the oracle ends every framed ray as src/trajectory.cpp:214-396
    does -- including cameras inside the horizon (its dead-zone rule and the rise through r_+)."""
    g = golden("framed_ref.npz")
    end_map = {1: po.CAPTURED, 2: po.DISK, 0: po.ESCAPED}
    i = 0
    inside = 0
    for cam, fr in zip(g["cameras"], g["frames"]):
        a, r, th, ph, r_in = cam
        rp = oracle.horizon_radius_raw(a)
        inside += r < rp
        sc = po.Scene(a, r, th, ph, r_in, 20.0, 250.0, 0.01 / rp, 0.01, 200000, po.RK4)
        for lk in g["looks"]:
            ray = oracle.trace_framed(sc, fr, lk)
            want = end_map[int(g["tr_end"][i])]
            assert ray.outcome == want, (i, ray.outcome, want)
            if want == po.DISK:
                assert abs(ray.r_disk - g["tr_values"][i][0]) < 1e-9 * max(1.0, g["tr_values"][i][0])
                assert abs(ray.g - g["tr_values"][i][1]) < 1e-9
            i += 1
    assert inside == 2
