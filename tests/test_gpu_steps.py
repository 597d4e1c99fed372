"""GPU per-step mirrors (bhk_derivatives, bhk_step_mino, ...) against the reference's golden
vectors, and the reference's known-answer tests for the photon path (tests/test_kerr.cpp)
re-run through the C ABI: the same loop shapes, with libbhk's kernels doing every step."""
import math

import numpy as np
import pytest
import torch

from black_simulation_gb300 import bhk

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def dev(x):
    return torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def close(got, want, rtol=RTOL, atol=1e-12):
    np.testing.assert_allclose(got, want, rtol=rtol, atol=atol)


def test_per_step_mirrors_match_reference_vectors(cuda, golden):
    """Every one of the 512 reference rows, each with its own spin (one launch of n = 1 per row)."""
    g = golden("steps_ref.npz")
    n = len(g["a"])
    for i in range(n):
        a = float(g["a"][i])  # the batch shares one spin: rows of different spins go one at a time
        c = dev(g["cons"][i:i + 1])
        s = dev(g["state"][i:i + 1])
        close(bhk.derivatives(a, c, s).cpu().numpy()[0], g["derivatives"][i])
        s2 = s.clone()
        bhk.step_mino(a, c, s2, dev([g["h"][i]]))
        close(s2.cpu().numpy()[0], g["step_mino"][i])
        close(bhk.photon_step_size(a, c, s, float(g["tol"][i])).cpu().numpy()[0], g["step_size"][i])
        s3 = s.clone()
        bhk.enforce_constraints(a, c, s3)
        close(s3.cpu().numpy()[0], g["enforced"][i])
    # normalizeAngles is spin-free: the whole table in one launch.
    st = g["state"].copy()
    st[:, 2] *= 3.0
    s = dev(st)
    bhk.normalize_angles(s)
    close(s.cpu().numpy(), g["normalized"])


def test_batched_mirrors_match_reference_vectors_per_spin_block(cuda, golden):
    """The batched launch path (n = 64 rows sharing a spin, as the reference call shape has it): each
    mirror once per spin over its 64 rows, all 8 x 64 reference rows checked (src/kerr.cpp:331-575)."""
    g = golden("steps_blocks_ref.npz")
    per, tol = int(g["per"]), float(g["tol"])
    for b, a in enumerate(g["spins"]):
        sl = slice(b * per, (b + 1) * per)
        assert np.all(g["a"][sl] == a)
        c, s = dev(g["cons"][sl]), dev(g["state"][sl])
        close(bhk.derivatives(float(a), c, s).cpu().numpy(), g["derivatives"][sl])
        s2 = s.clone()
        bhk.step_mino(float(a), c, s2, dev(g["h"][sl]))
        close(s2.cpu().numpy(), g["step_mino"][sl])
        close(bhk.photon_step_size(float(a), c, s, tol).cpu().numpy(), g["step_size"][sl])
        s3 = s.clone()
        bhk.enforce_constraints(float(a), c, s3)
        close(s3.cpu().numpy(), g["enforced"][sl])
        R, Th = bhk.potentials(float(a), c, s)
        close(R.cpu().numpy(), g["potentials"][sl, 0])
        # Theta = Q - cos^2 (...) cancels: absolute tolerance on the scale of its terms
        close(Th.cpu().numpy(), g["potentials"][sl, 1], atol=1e-10)


def test_frames_and_photon_launches_match_reference(cuda, golden):
    g = golden("steps_ref.npz")
    for i in range(0, len(g["frame_a"]), 8):
        a, r, th = float(g["frame_a"][i]), float(g["frame_r"][i]), float(g["frame_theta"][i])
        f = bhk.observer_frame(a, dev([r]), dev([th]))
        close(f.cpu().numpy()[0], g["frames"][i])
        c, s = bhk.photon_from_frame(a, r, th, 0.25, f[0], dev(g["look"][i:i + 1]))
        close(c.cpu().numpy()[0], g["photon_cons"][i], rtol=1e-11, atol=1e-11)
        close(s.cpu().numpy()[0], g["photon_state"][i], rtol=1e-11, atol=1e-11)
        c, s = bhk.launch_from_zamo(a, r, th, 0.0, dev(g["zamo_v"][i:i + 1]), 0.0)
        close(c.cpu().numpy()[0], g["zamo_cons"][i], rtol=1e-11, atol=1e-11)
        close(s.cpu().numpy()[0], g["zamo_state"][i], rtol=1e-11, atol=1e-11)


def _ks_metric(a, r, th):
    """The Kerr-Schild metric g_mn at (r, theta) (kerr::metricTensor, src/kerr.cpp:238-254) and Sigma."""
    sn, cs = math.sin(th), math.cos(th)
    sigma = r * r + a * a * cs * cs
    A = (r * r + a * a) ** 2 - a * a * (r * r - 2 * r + a * a) * sn * sn
    f = 2 * r / sigma
    gm = np.zeros((4, 4))
    gm[0, 0] = -(1 - f); gm[0, 1] = gm[1, 0] = f; gm[0, 3] = gm[3, 0] = -f * a * sn * sn
    gm[1, 1] = 1 + f; gm[1, 3] = gm[3, 1] = -a * sn * sn * (1 + f); gm[2, 2] = sigma; gm[3, 3] = A * sn * sn / sigma
    return gm, sigma


def _observed_photon(a, r, th, v, look):
    """kerr::observedPhoton (src/kerr.cpp:485-500) composed from the GPU mirrors: the observer moving
    with 3-velocity v relative to the ZAMO (launchFromZamo with mu = 1, its 4-velocity as
    kerr::fourVelocity forms it, src/kerr.cpp:418-422), its frame, the photon seen along look,
    normalised to E = 1. Returns the frequency the observer measures (1 / E before normalising),
    the constants, the state and the observer's 4-velocity."""
    oc, os_ = bhk.launch_from_zamo(a, r, th, 0.0, dev([v]), 1.0)
    d = bhk.derivatives(a, oc, os_).cpu().numpy()[0]
    _, sigma = _ks_metric(a, r, th)
    u = d[:4] / sigma
    f = bhk.observer_frame(a, dev([r]), dev([th]), dev([u]))
    c, s = bhk.photon_from_frame(a, r, th, 0.0, f[0], dev([look]))
    cv, sv = c.cpu().numpy()[0].copy(), s.cpu().numpy()[0].copy()
    inv = 1.0 / cv[0]
    cv[1] *= inv; cv[2] *= inv * inv; sv[4] *= inv; sv[5] *= inv; cv[0] = 1.0
    return inv, cv, sv, u


def test_moving_observer(cuda):
    """testMovingObserver (tests/test_kerr.cpp:349-381): a boosted observer measures the energy the
    boost predicts (1e-10), the aberrated photon is null (1e-9), flying at 0.6 c straight at what it
    looks at blueshifts it by sqrt(1.6 / 0.4) = 2 (1e-12), and an observer at rest is deterministic."""
    a, r, th = 0.9, 7.0, 1.2
    look = [-0.6, 0.48, 0.64]
    g0, _, _, _ = _observed_photon(a, r, th, [0.0, 0.0, 0.0], look)
    g, c, s, u = _observed_photon(a, r, th, [-0.3, 0.2, 0.5], look)
    cd, sd = dev([c]), dev([s])
    d = bhk.derivatives(a, cd, sd).cpu().numpy()[0]
    gm, sigma = _ks_metric(a, r, th)
    assert abs(-(d[:4] / sigma) @ gm @ u - g) < 1e-10
    R, Th = bhk.potentials(a, cd, sd)
    assert abs(s[4] ** 2 - R.item()) < 1e-9
    assert abs(s[5] ** 2 - Th.item()) < 1e-9
    still, _, _, _ = _observed_photon(a, r, th, [0.0, 0.0, 0.0], [-1.0, 0.0, 0.0])
    moving, _, _, _ = _observed_photon(a, r, th, [-0.6, 0.0, 0.0], [-1.0, 0.0, 0.0])
    assert abs(moving / still - 2.0) < 1e-12
    assert _observed_photon(a, r, th, [0.0, 0.0, 0.0], look)[0] == g0


def test_observer_frames_orthonormal_and_photons_null(cuda):
    """testObserverFrames (tests/test_kerr.cpp:703-800): ZAMO frames orthonormal to 1e-12, photons
    from them null to 1e-9, and a ZAMO photon equals launchFromZamo to 1e-12."""
    a = 0.9
    rs = dev([6.0, 7.0, 30.0, 500.0])
    ths = dev([1.1, 1.2, 0.3, 2.9])
    F = bhk.observer_frame(a, rs, ths).cpu().numpy()
    for k in range(4):
        gm, _ = _ks_metric(a, float(rs[k]), float(ths[k]))
        G = F[k] @ gm @ F[k].T
        assert np.max(np.abs(G - np.diag([-1.0, 1, 1, 1]))) < 1e-12
    look = np.array([[-0.48, 0.6, 0.64]])
    c, s = bhk.photon_from_frame(a, 7.0, 1.2, 0.0, dev(F[1]), dev(look))
    R, Th = bhk.potentials(a, c, s)
    sv = s.cpu().numpy()[0]
    assert abs(sv[4] ** 2 - R.item()) < 1e-9 * max(1.0, abs(R.item()))
    assert abs(sv[5] ** 2 - Th.item()) < 1e-9
    zc, zs = bhk.launch_from_zamo(a, 7.0, 1.2, 0.0, dev(-look), 0.0)
    cv, zcv, zsv = c.cpu().numpy()[0], zc.cpu().numpy()[0], zs.cpu().numpy()[0]
    assert abs(cv[1] / cv[0] - zcv[1]) < 1e-12
    assert abs(cv[2] / cv[0] ** 2 - zcv[2]) < 1e-12
    assert abs(sv[4] / cv[0] - zsv[4]) < 1e-12


def _photon_fate_batch(a, bs, tol=1e-3, r0=1000.0, max_iter=400000):
    """photonFate (tests/test_kerr.cpp:222-241) for a batch of impact parameters, every step on the GPU."""
    th = math.pi / 2
    sigma = r0 * r0
    delta = r0 * r0 - 2 * r0 + a * a
    A = (r0 * r0 + a * a) ** 2 - a * a * delta
    omega = 2 * a * r0 / A
    v = []
    for b in bs:
        vphi = b * math.sqrt(sigma * delta / A) / (math.sqrt(A / sigma) * (1.0 - omega * b))
        v.append([-math.sqrt(1 - vphi * vphi), 0.0, vphi])
    c, s = bhk.launch_from_zamo(a, r0, th, 0.0, dev(v), 0.0)
    rh = 1 + math.sqrt(1 - a * a)
    fate = np.zeros(len(bs), int)
    measured_b = (c[:, 1] / c[:, 0]).cpu().numpy()
    active = torch.ones(len(bs), dtype=torch.bool, device="cuda")
    for it in range(max_iter):
        h = bhk.photon_step_size(a, c, s, tol)
        h = torch.where(active, h, torch.zeros_like(h))
        bhk.step_mino(a, c, s, h)
        bhk.enforce_constraints(a, c, s)
        if it % 256 == 255:
            r = s[:, 1].cpu().numpy()
            for k in range(len(bs)):
                if fate[k] == 0 and r[k] < rh + 1e-3:
                    fate[k] = -1
                elif fate[k] == 0 and r[k] > 2000.0:
                    fate[k] = 1
            active = torch.tensor(fate == 0, device="cuda")
            if np.all(fate != 0):
                break
    return fate, measured_b


def test_shadow_capture_and_escape_at_critical_impact_parameters(cuda):
    """testShadow (tests/test_kerr.cpp:243-262)."""
    bc = 3 * math.sqrt(3)
    fate, mb = _photon_fate_batch(0.0, [bc * 0.999, bc * 1.001])
    assert list(fate) == [-1, 1]
    assert abs(mb[0] - bc * 0.999) < 1e-10
    a = 0.9
    xi = lambda r: -(r ** 3 - 3 * r * r + a * a * r + a * a) / (a * (r - 1))  # noqa: E731
    r_pro = 2 * (1 + math.cos(2 / 3 * math.acos(-a)))
    r_ret = 2 * (1 + math.cos(2 / 3 * math.acos(a)))
    b_pro, b_ret = xi(r_pro), xi(r_ret)
    assert abs(b_pro - 2.844) < 2e-3 and abs(b_ret + 6.834) < 2e-3
    fate, _ = _photon_fate_batch(a, [b_pro * 0.999, b_pro * 1.001, b_ret * 0.999, b_ret * 1.001])
    assert list(fate) == [-1, 1, -1, 1]


def test_traced_light_bending_matches_exact_integral(cuda, golden):
    """testSurfaceLightBending (tests/test_kerr.cpp:984-1013): integrator bending from R = 5.8 M to
    r = 1e6 against central::bendingAngle to 1e-6 (reference values in the golden fixture)."""
    g = golden("steps_ref.npz")
    alphas = g["bend_alpha"]
    v = np.stack([np.cos(alphas), np.zeros_like(alphas), np.sin(alphas)], 1)
    c, s = bhk.launch_from_zamo(0.0, 5.8, math.pi / 2, 0.0, dev(v), 0.0)
    done = torch.zeros(len(alphas), dtype=torch.bool, device="cuda")
    for it in range(2_000_000):
        h = bhk.photon_step_size(0.0, c, s, 2e-4)
        h = torch.where(done, torch.zeros_like(h), h)
        bhk.step_mino(0.0, c, s, h)
        bhk.enforce_constraints(0.0, c, s)
        if it % 512 == 511:
            done = s[:, 1] >= 1e6
            if bool(done.all()):
                break
    sv, cv = s.cpu().numpy(), c.cpu().numpy()
    traced = sv[:, 3] + np.arcsin(cv[:, 1] / cv[:, 0] / sv[:, 1])
    np.testing.assert_allclose(traced, g["bend"], rtol=0, atol=1e-6)


def _escape_direction(a, r, theta, vs, tol):
    """escapeDirection (tests/test_kerr.cpp:266-281) for a batch of launch directions."""
    c, s = bhk.launch_from_zamo(a, r, theta, 0.0, dev(vs), 0.0)
    rh = 1 + math.sqrt(1 - a * a)
    for it in range(100000):
        rr = s[:, 1]
        live = rr < 500.0
        if it % 64 == 0 and not bool(live.any()):
            break
        h = bhk.photon_step_size(a, c, s, tol)
        h = torch.where(live, h, torch.zeros_like(h))
        bhk.step_mino(a, c, s, h)
        bhk.normalize_angles(s)
        bhk.enforce_constraints(a, c, s)
    assert bool((s[:, 1] > rh + 1e-3).all())
    d = bhk.cartesian_velocity(a, c, s).cpu().numpy()
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def test_near_axis_photons_leave_together(cuda):
    """testNearAxisPhotons (tests/test_kerr.cpp:283-325)."""
    a, r, theta = 0.94, 32.0, 1.48
    for eps in (0.0011, 0.003):
        vs = []
        for z in (eps, -eps):
            x = np.array([-1.0, -0.53, z])
            vs.append(x / np.linalg.norm(x))
        d = _escape_direction(a, r, theta, vs, 0.04)
        assert abs(d[0, 0] - d[1, 0]) < 2e-3
        assert abs(d[0, 1] - d[1, 1]) < 1e-2
        assert abs(d[0, 2] - d[1, 2]) < 2e-3
    vs = []
    for k in range(6):
        eps = 1e-6 * 10.0 ** k
        x = np.array([-0.8, -0.6, eps])
        vs.append(x / np.linalg.norm(x))
    d = _escape_direction(a, r, 0.035, vs, 0.04)
    for k in range(1, 6):
        eps = 1e-6 * 10.0 ** k
        assert np.linalg.norm(d[k] - d[k - 1]) < 2e-3 + 2 * eps


def test_predict_matches_reference_paths(cuda, golden):
    """trajectory::predict batched on the GPU against the reference's own paths (bound and precessing,
    near-circular, plunging, escaping; tests/golden/predict_ref.npz)."""
    import torch
    g = golden("predict_ref.npz")
    sc = g["scalars"]
    for i, (a, r, th) in enumerate(g["cases"]):
        c = torch.tensor(g["constants"][i:i + 1], dtype=torch.float64, device="cuda")
        s = torch.tensor(g["states"][i:i + 1], dtype=torch.float64, device="cuda")
        o = bhk.predict(float(a), c, s, float(g["max_time"]), float(g["min_spacing"]), int(g["max_points"]),
                        escape_radius=float(g["escape_radius"]))
        torch.cuda.synchronize()
        assert int(o["fate"][0]) == int(sc[i, 0]), (i, int(o["fate"][0]), sc[i, 0])
        assert int(o["periapses"][0]) == int(sc[i, 4])
        assert abs(float(o["duration"][0]) / sc[i, 1] - 1.0) < 1e-9
        assert abs(float(o["r_min"][0]) / sc[i, 2] - 1.0) < 1e-8
        assert abs(float(o["r_max"][0]) / sc[i, 3] - 1.0) < 1e-8
        assert abs(float(o["precession_deg"][0]) - sc[i, 5]) < 1e-5
        npts = int(o["n_points"][0])
        assert npts == int(sc[i, 6])
        pts = o["points"][0, :npts].cpu().numpy()
        want = g["points"][i, :npts]
        assert np.abs(pts - want).max() <= 1e-6 * max(1.0, np.abs(want).max())


def test_predict_batch_equals_single_particles(cuda, golden):
    import torch
    g = golden("predict_ref.npz")
    # the same particles, several spins in one call are not possible (one a per call): batch per spin
    idx = [i for i, row in enumerate(g["cases"]) if row[0] == 0.9]
    c = torch.tensor(g["constants"][idx], dtype=torch.float64, device="cuda")
    s = torch.tensor(g["states"][idx], dtype=torch.float64, device="cuda")
    o = bhk.predict(0.9, c, s, 3000.0, 0.5, 2000, points=False)
    torch.cuda.synchronize()
    for j, i in enumerate(idx):
        assert int(o["fate"][j]) == int(g["scalars"][i, 0])
        assert int(o["n_points"][j]) == int(g["scalars"][i, 6])
    with pytest.raises(bhk.BhkError):
        bhk.predict(1.5, c, s, 10.0)
