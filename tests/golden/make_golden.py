"""Generates the golden fixtures in this folder from the reference itself.

Run where the reference tree exists (it builds oracle/_ref/libkerr_ref.so from the reference's
unmodified kerr.cpp, trajectory.cpp, central.cpp and eht.cpp through oracle/Makefile):

    python tests/golden/make_golden.py

Fixtures (all produced by the reference's own functions, never by this project's code):
  steps_blocks_ref.npz  per-step vectors in 8 spin blocks of 64 states (derivatives, stepMino,
                      photonStepSize, enforceConstraints, radialPotential/polarPotential), for batched checks
  steps_ref.npz       per-step vectors: derivatives, stepMino, photonStepSize, enforceConstraints,
                      normalizeAngles, ZAMO frames + photonFromFrame, launchFromZamo, radii, critical
                      curves, central::bendingAngle (src/kerr.cpp, src/eht.cpp, src/central.cpp)
  trajectory_ref.npz  trajectory::traceRay end and values (rEnd, g, skyDirection, rMin, turns, energy,
                      delay) for ZAMO cameras with a disk
                      (src/trajectory.cpp:214-396), to pin the loop shape of the oracle
  c1_rk4_1e-4.npz     128x128 frame, a=0.9, r_obs=50, theta=80 deg, alpha,beta in [-15,15], disk
                      ISCO..20, escape 1000, capture r_+(1+1e-6): the reference RK4 loop at tolerance 1e-4
  c2_rk4_1e-4.npz     96x54 frame with the 1080p geometry (a=0.998, r_obs=1000, theta=60 deg,
                      alpha in +-20, beta in +-11.25, disk ISCO..30) at tolerance 1e-4
  framed_ref.npz      cameras with arbitrary frames -- ZAMO, boosted from the ZAMO (Camera::frame's
                      drift recipe, src/camera.cpp:23-36) and free-falling inside the horizon
                      (kerr::fourVelocity) -- frames from kerr::observerFrame, 40 look directions each:
                      trajectory::traceRay's end/rEnd/g (src/trajectory.cpp:214-396) and the reference
                      loop at tolerance 1e-4 from kerr::photonFromFrame with traceRay's inside-horizon rule
  predict_ref.npz     trajectory::predict paths of massive particles launched from ZAMOs (bound and
                      precessing, near-circular, plunging, escaping; src/trajectory.cpp:130-185)
  naked_ref.npz       past |a| = 1 (no horizon): kerr::iscoRadius / photonOrbitRadius of naked spins;
                      frames traced by the reference loop at tolerance 1e-4 with the renderer's rules
                      for naked singularities (ring where Sigma < 4e-4, the sky of the r < 0 region;
                      shaders/trace.frag:1768-1787); an eht::render image at a = 1.2
  eht_ref.npz         eht::render images (src/eht.cpp:260-347): the M87* view of the reference's
                      calibration test (a = 0.9 at 60 deg, 48 px, density from eht::calibrate at 0.5 Jy),
                      a = 0.5 at 163 deg (32 px) and a = 0.99 at 30 deg (40 px), default flow
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import pyoracle as po  # noqa: E402


def steps_blocks_fixture(R: po.Oracle) -> dict:
    """Per-step vectors in spin blocks (8 spins x 64 states), so that each mirror is checked through
    one batched launch per spin (the reference call shape shares a by the batch)."""
    rng = np.random.default_rng(20261204)
    spins = np.array([0.0, 0.3, 0.5, 0.7, 0.9, 0.95, 0.99, 0.998])
    per = 64
    n = spins.size * per
    a = np.repeat(spins, per)
    cons = np.stack([rng.uniform(0.5, 1.5, n), rng.uniform(-8, 8, n), rng.uniform(-2, 40, n), np.zeros(n)], 1)
    st = np.stack([rng.uniform(-5, 5, n), rng.uniform(1.2, 1000, n), rng.uniform(-0.3, np.pi + 0.3, n),
                   rng.uniform(-10, 10, n), rng.uniform(-1e3, 1e3, n), rng.uniform(-10, 10, n)], 1)
    h = rng.uniform(-0.02, 0.02, n)
    tol = float(10.0 ** rng.uniform(-4, -1))  # one tolerance per batch, as photonStepSize takes it
    der = np.zeros((n, 6))
    stepped = np.zeros((n, 6))
    hstep = np.zeros(n)
    enforced = np.zeros((n, 6))
    pot = np.zeros((n, 2))
    for i in range(n):
        c = po.Constants(*cons[i])
        s = po.State(*st[i])
        d = R.derivatives(a[i], c, s)
        der[i] = [d.dt, d.dr, d.dtheta, d.dphi, d.dvr, d.dvtheta]
        x = R.step_mino(a[i], c, s, h[i])
        stepped[i] = [x.t, x.r, x.theta, x.phi, x.vr, x.vtheta]
        hstep[i] = R.photon_step_size(a[i], c, s, tol)
        x = R.enforce_constraints(a[i], c, s)
        enforced[i] = [x.t, x.r, x.theta, x.phi, x.vr, x.vtheta]
        pot[i] = [R.radial_potential_raw(a[i], C.byref(c), st[i][1]), R.polar_potential_raw(a[i], C.byref(c), st[i][2])]
    return dict(spins=spins, per=np.array(per), a=a, cons=cons, state=st, h=h, tol=np.array(tol), derivatives=der,
                step_mino=stepped, step_size=hstep, enforced=enforced, potentials=pot)


def steps_fixture(R: po.Oracle) -> dict:
    rng = np.random.default_rng(20261203)
    n = 512
    a = rng.uniform(0.0, 0.999, n)
    cons = np.stack([rng.uniform(0.5, 1.5, n), rng.uniform(-8, 8, n), rng.uniform(-2, 40, n), np.zeros(n)], 1)
    st = np.stack([rng.uniform(-5, 5, n), rng.uniform(1.2, 1000, n), rng.uniform(-0.3, np.pi + 0.3, n),
                   rng.uniform(-10, 10, n), rng.uniform(-1e3, 1e3, n), rng.uniform(-10, 10, n)], 1)
    h = rng.uniform(-0.02, 0.02, n)
    tol = 10.0 ** rng.uniform(-4, -1, n)
    der = np.zeros((n, 6))
    stepped = np.zeros((n, 6))
    hstep = np.zeros(n)
    enforced = np.zeros((n, 6))
    normalized = np.zeros((n, 6))
    for i in range(n):
        c = po.Constants(*cons[i])
        s = po.State(*st[i])
        d = R.derivatives(a[i], c, s)
        der[i] = [d.dt, d.dr, d.dtheta, d.dphi, d.dvr, d.dvtheta]
        x = R.step_mino(a[i], c, s, h[i])
        stepped[i] = [x.t, x.r, x.theta, x.phi, x.vr, x.vtheta]
        hstep[i] = R.photon_step_size(a[i], c, s, tol[i])
        x = R.enforce_constraints(a[i], c, s)
        enforced[i] = [x.t, x.r, x.theta, x.phi, x.vr, x.vtheta]
        big = po.State(st[i][0], st[i][1], st[i][2] * 3.0, st[i][3], st[i][4], st[i][5])
        x = R.normalize_angles(big)
        normalized[i] = [x.t, x.r, x.theta, x.phi, x.vr, x.vtheta]
    # ZAMO frames and the photons they launch
    m = 128
    fa = rng.uniform(0.0, 0.999, m)
    fr = 10.0 ** rng.uniform(0.4, 3.0, m)
    fth = rng.uniform(0.02, np.pi - 0.02, m)
    look = rng.normal(size=(m, 3))
    look /= np.linalg.norm(look, axis=1, keepdims=True)
    frames = np.zeros((m, 4, 4))
    pcons = np.zeros((m, 4))
    pstate = np.zeros((m, 6))
    for i in range(m):
        f = R.zamo_frame(fa[i], fr[i], fth[i])
        frames[i] = np.array([[f.e[k][j] for j in range(4)] for k in range(4)])
        c, s = R.photon_from_frame(fa[i], fr[i], fth[i], 0.25, f, look[i])
        pcons[i] = [c.E, c.L, c.Q, c.mu]
        pstate[i] = [s.t, s.r, s.theta, s.phi, s.vr, s.vtheta]
    zv = rng.normal(size=(m, 3))
    zv /= np.linalg.norm(zv, axis=1, keepdims=True)
    zcons = np.zeros((m, 4))
    zstate = np.zeros((m, 6))
    for i in range(m):
        c, s = R.launch_from_zamo(fa[i], fr[i], fth[i], 0.0, zv[i], 0.0)
        zcons[i] = [c.E, c.L, c.Q, c.mu]
        zstate[i] = [s.t, s.r, s.theta, s.phi, s.vr, s.vtheta]
    spins = np.array([0.0, 0.3, 0.6, 0.9, 0.94, 0.998, 1.0])
    radii = np.array([[R.horizon_radius_raw(x), R.isco_radius_raw(x, 1), R.isco_radius_raw(x, 0),
                       R.photon_orbit_radius_raw(x, 1), R.photon_orbit_radius_raw(x, 0)] for x in spins])
    cc_params = np.array([(0.0, 1.0), (0.9, np.deg2rad(17)), (0.9, np.deg2rad(60)), (0.998, np.deg2rad(60)),
                          (0.5, np.deg2rad(80))])
    cc = {"cc_params": cc_params}
    for i, (sa, incl) in enumerate(cc_params):
        al, be = R.critical_curve(sa, incl, 400)
        cc[f"cc{i}_alpha"] = al
        cc[f"cc{i}_beta"] = be
    bend_alpha = np.deg2rad([10.0, 40.0, 70.0, 89.0])
    bend = np.array([R.bending_angle_raw(5.8, x) for x in bend_alpha])
    return dict(a=a, cons=cons, state=st, h=h, tol=tol, derivatives=der, step_mino=stepped, step_size=hstep,
                enforced=enforced, normalized=normalized, frame_a=fa, frame_r=fr, frame_theta=fth, look=look,
                frames=frames, photon_cons=pcons, photon_state=pstate, zamo_v=zv, zamo_cons=zcons,
                zamo_state=zstate, spins=spins, radii=radii, bend_alpha=bend_alpha, bend=bend, **cc)


def trajectory_fixture(R: po.Oracle) -> dict:
    rng = np.random.default_rng(7)
    n = 96
    a = rng.uniform(0.0, 0.998, n)
    r = 10.0 ** rng.uniform(1.2, 2.0, n)
    th = rng.uniform(0.2, np.pi - 0.2, n)
    look = np.stack([-np.ones(n), rng.uniform(-0.35, 0.35, n), rng.uniform(-0.35, 0.35, n)], 1)
    look /= np.linalg.norm(look, axis=1, keepdims=True)
    end = np.zeros(n, np.int32)
    vals = np.zeros((n, 9))
    r_in = np.array([R.isco_radius_raw(x, 1) for x in a])
    for i in range(n):
        out = np.zeros(9)
        end[i] = R.trajectory_trace_raw(a[i], r[i], th[i], 0.0, po._ptr(np.ascontiguousarray(look[i])), 1, r_in[i],
                                        20.0, 250.0, po._ptr(out))
        vals[i] = out
    return dict(a=a, r=r, theta=th, look=look, r_in=r_in, end=end, values=vals)


FRAMED_CAMERAS = (
    # (a, r, theta, phi, kind, parameters)
    (0.9, 50.0, np.deg2rad(80.0), 0.0, "zamo", ()),
    (0.9, 20.0, np.deg2rad(60.0), 0.3, "boost", (0.0, 0.0, 0.5)),
    (0.9, 15.0, np.deg2rad(100.0), 1.0, "boost", (-0.6, 0.1, 0.0)),
    (0.998, 8.0, np.deg2rad(45.0), 0.0, "boost", (0.2, -0.3, 0.4)),
    (0.9, 1.3, np.deg2rad(70.0), 0.0, "fall", (1.0, 0.0, 0.0)),      # inside r_+ = 1.436: E, L, extra Q
    (0.5, 1.6, np.deg2rad(30.0), 2.0, "fall", (1.0, 0.5, 0.1)),      # inside r_+ = 1.866
)


def framed_camera(R: po.Oracle, a, r, th, kind, par):
    """The camera frame (4 x 4) the reference builds for one of FRAMED_CAMERAS."""
    u = np.zeros(4)
    R.zamo_four_velocity_raw(a, r, th, po._ptr(u))
    if kind == "boost":
        z = po.Frame()
        R.observer_frame_raw(a, r, th, po._ptr(u), C.byref(z))
        e = np.ctypeslib.as_array(z.e)
        v = np.array(par)
        gamma = 1.0 / np.sqrt(1.0 - v @ v)
        u = gamma * (e[0] + v[0] * e[1] + v[1] * e[2] + v[2] * e[3])
    elif kind == "fall":  # a massive geodesic observer (mu = 1), falling inward
        E, L, dq = par
        c = po.Constants(E, L, 0.0, 1.0)
        st, ct = np.sin(th), np.cos(th)
        c.Q = ct * ct * (a * a * (1.0 - E * E) + L * L / (st * st)) + dq
        Rr = R.radial_potential_raw(a, C.byref(c), r)
        Th = R.polar_potential_raw(a, C.byref(c), th)
        s = po.State(0.0, r, th, 0.0, -np.sqrt(max(Rr, 0.0)), np.sqrt(max(Th, 0.0)))
        d = po.Derivs()
        R.derivatives_raw(a, C.byref(c), C.byref(s), C.byref(d))
        sigma = r * r + a * a * ct * ct
        u = np.array([d.dt, d.dr, d.dtheta, d.dphi]) / sigma
    f = po.Frame()
    R.observer_frame_raw(a, r, th, po._ptr(np.ascontiguousarray(u)), C.byref(f))
    return np.ctypeslib.as_array(f.e).copy()


def fibonacci_looks(n):
    k = np.arange(n) + 0.5
    z = 1.0 - 2.0 * k / n
    ph = np.pi * (1.0 + 5.0 ** 0.5) * k
    rr = np.sqrt(1.0 - z * z)
    return np.stack([z, rr * np.cos(ph), rr * np.sin(ph)], 1)  # (l_r, l_theta, l_phi)


def framed_fixture(R: po.Oracle) -> dict:
    looks = fibonacci_looks(40)
    cams, frames = [], []
    tr_end, tr_val = [], []
    keys = ("outcome", "r_disk", "phi_disk", "g", "theta_inf", "phi_inf", "steps")
    rk = {k: [] for k in keys}
    for a, r, th, ph, kind, par in FRAMED_CAMERAS:
        f = framed_camera(R, a, r, th, kind, par)
        r_in = R.isco_radius_raw(a, 1)
        frames.append(f)
        cams.append([a, r, th, ph, r_in])
        sc = po.Scene(a, r, th, ph, r_in, 20.0, 1000.0, 1e-6, 1e-4, 5_000_000, po.RK4)
        for lk in looks:
            out = np.zeros(9)
            tr_end.append(R.trajectory_trace_framed_raw(a, r, th, ph, po._ptr(np.ascontiguousarray(f.reshape(16))),
                                                        po._ptr(np.ascontiguousarray(lk)), 1, r_in, 20.0, 250.0,
                                                        po._ptr(out)))
            tr_val.append(out)
            ray = R.trace_framed(sc, f, lk)
            for k in keys:
                rk[k].append(getattr(ray, k))
    out = dict(cameras=np.array(cams), frames=np.array(frames), looks=looks, tr_end=np.array(tr_end, np.int32),
               tr_values=np.array(tr_val))
    out.update({k: np.array(v) for k, v in rk.items()})
    print("  framed outcomes", np.bincount(out["outcome"].astype(int), minlength=4), "traceRay ends",
          np.bincount(out["tr_end"], minlength=5))
    return out


EHT_VIEWS = (  # (a, inclination deg, half width, size), frequency 230 GHz, M87* mass
    (0.9, 60.0, 16.0, 48),
    (0.5, 163.0, 16.0, 32),
    (0.99, 30.0, 16.0, 40),
)
EHT_FLOW = (1e5, 4e11, 10.0, 0.9, 1.0, 0.8165)  # eht::Flow defaults (src/eht.h)
M87_MASS, M87_DISTANCE_PC, M87_FLUX_JY = 6.5e9, 16.8e6, 0.5


def eht_fixture(R: po.Oracle) -> dict:
    lib = R.lib
    dp = C.POINTER(C.c_double)
    lib.ref_eht_render.argtypes = [C.c_double] * 3 + [C.c_int] + [C.c_double] * 2 + [dp, C.c_int, dp,
                                                                                        C.POINTER(C.c_ubyte)]
    lib.ref_eht_render.restype = None
    lib.ref_eht_calibrate.argtypes = [C.c_double] * 3 + [C.c_int] + [C.c_double] * 2 + [dp] + [C.c_double] * 2 + [C.c_int]
    lib.ref_eht_calibrate.restype = C.c_double
    lib.ref_eht_angular_scale.argtypes = [C.c_double, C.c_double]
    lib.ref_eht_angular_scale.restype = C.c_double
    lib.ref_eht_flux.argtypes = [dp, C.c_int, C.c_double, C.c_double]
    lib.ref_eht_flux.restype = C.c_double
    threads = os.cpu_count() or 1
    theta_g = lib.ref_eht_angular_scale(M87_MASS, M87_DISTANCE_PC)
    flow = np.array(EHT_FLOW)
    t = time.time()
    n0 = lib.ref_eht_calibrate(0.9, np.deg2rad(60.0), 16.0, 40, 230e9, M87_MASS, po._ptr(flow), M87_FLUX_JY, theta_g,
                               threads)
    print(f"  calibrated n0 = {n0:.6g} in {time.time() - t:.1f} s")
    out = dict(views=np.array(EHT_VIEWS), flow=flow, n0_calibrated=n0, theta_g=theta_g, mass=M87_MASS,
               target_jy=M87_FLUX_JY)
    for i, (a, inc, hw, size) in enumerate(EHT_VIEWS):
        fl = flow.copy()
        if i == 0:
            fl[0] = n0
        inten = np.zeros(size * size)
        shadow = np.zeros(size * size, np.uint8)
        t = time.time()
        lib.ref_eht_render(a, np.deg2rad(inc), hw, size, 230e9, M87_MASS, po._ptr(fl), threads, po._ptr(inten),
                           shadow.ctypes.data_as(C.POINTER(C.c_ubyte)))
        out[f"intensity_{i}"] = inten
        out[f"shadow_{i}"] = shadow
        out[f"flux_{i}"] = lib.ref_eht_flux(po._ptr(inten), size, hw, theta_g)
        print(f"  view {i}: {size}x{size} in {time.time() - t:.1f} s, flux {out[f'flux_{i}']:.4g} Jy, "
              f"shadow px {shadow.sum()}")
    return out


PREDICT_CASES = (  # (a, r, theta deg, ZAMO-frame velocity (r, theta, phi)), mu = 1
    (0.9, 12.0, 90.0, (0.0, 0.0, 0.38)),     # eccentric, equatorial: precesses
    (0.9, 10.0, 70.0, (0.05, 0.1, 0.36)),    # inclined, eccentric
    (0.5, 8.0, 90.0, (0.0, 0.0, 0.42)),      # near circular
    (0.9, 6.0, 80.0, (-0.3, 0.0, 0.2)),      # plunges
    (0.3, 20.0, 60.0, (0.7, 0.0, 0.2)),      # escapes
    (0.998, 4.0, 90.0, (0.0, 0.0, 0.55)),    # close to the hole
)


def predict_fixture(R: po.Oracle) -> dict:
    lib = R.lib
    lib.ref_predict.argtypes = [C.c_double, C.POINTER(po.Constants), C.POINTER(po.State), C.c_double, C.c_double,
                                C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
    lib.ref_predict.restype = None
    cap = 2001
    cons, states, scal, pts = [], [], [], []
    for a, r, th, v in PREDICT_CASES:
        c, s = R.launch_from_zamo(a, r, np.deg2rad(th), 0.0, np.array(v, dtype=np.float64), 1.0)
        out = np.zeros(7)
        p = np.zeros((cap, 3))
        lib.ref_predict(a, C.byref(c), C.byref(s), 3000.0, 0.5, cap - 1, 0.0, 2000.0, po._ptr(out), po._ptr(p), cap)
        cons.append([c.E, c.L, c.Q, c.mu])
        states.append([s.t, s.r, s.theta, s.phi, s.vr, s.vtheta])
        scal.append(out)
        pts.append(p)
        print(f"  a={a} r={r}: fate {int(out[0])}, {int(out[4])} periapses, precession {out[5]:.3f} deg, "
              f"{int(out[6])} points")
    return dict(cases=np.array([[a, r, th] for a, r, th, _ in PREDICT_CASES]), constants=np.array(cons),
                states=np.array(states), scalars=np.array(scal), points=np.array(pts), max_time=3000.0,
                min_spacing=0.5, max_points=cap - 1, escape_radius=2000.0)


NAKED_SPINS = (1.02, 1.05, 1.2, 1.5, 2.0, -1.3)
NAKED_FRAMES = (  # (a, r_obs, theta_obs deg, r_disk_out, width, height, (alpha_lo, alpha_hi, beta_lo, beta_hi))
    (1.2, 100.0, 30.0, 20.0, 64, 64, (-4.0, 4.0, -4.0, 4.0)),        # through the ring's disk, disk from ISCO < 1
    (1.05, 50.0, 75.0, 20.0, 48, 27, (-12.0, 12.0, -6.75, 6.75)),   # near edge-on
    (1.5, 30.0, 60.0, 0.0, 40, 40, (-6.0, 6.0, -6.0, 6.0)),         # no disk: both skies
)
NAKED_EHT = (1.2, 60.0, 16.0, 24)  # (a, inclination deg, half width, size)


def naked_fixture(R: po.Oracle) -> dict:
    lib = R.lib
    lib.ref_isco_radius.argtypes = [C.c_double, C.c_int]
    lib.ref_isco_radius.restype = C.c_double
    lib.ref_photon_orbit_radius.argtypes = [C.c_double, C.c_int]
    lib.ref_photon_orbit_radius.restype = C.c_double
    out = dict(spins=np.array(NAKED_SPINS),
               isco=np.array([[lib.ref_isco_radius(a, p) for p in (1, 0)] for a in NAKED_SPINS]),
               photon_orbit=np.array([[lib.ref_photon_orbit_radius(a, p) for p in (1, 0)] for a in NAKED_SPINS]))
    for i, (a, r, th, rout, w, h, ext) in enumerate(NAKED_FRAMES):
        sc = po.scene(a=a, r_obs=r, theta_obs_deg=th, r_disk_out=rout, tol=1e-4, method=po.RK4, max_steps=5_000_000)
        for k, v in frame_fixture(R, sc, w, h, ext).items():
            out[f"f{i}_{k}"] = v
    dp = C.POINTER(C.c_double)
    lib.ref_eht_render.argtypes = [C.c_double] * 3 + [C.c_int] + [C.c_double] * 2 + [dp, C.c_int, dp,
                                                                                        C.POINTER(C.c_ubyte)]
    lib.ref_eht_render.restype = None
    a, inc, hw, size = NAKED_EHT
    flow = np.array(EHT_FLOW)
    inten = np.zeros(size * size)
    shadow = np.zeros(size * size, np.uint8)
    t = time.time()
    lib.ref_eht_render(a, np.deg2rad(inc), hw, size, 230e9, M87_MASS, po._ptr(flow), os.cpu_count() or 1,
                       po._ptr(inten), shadow.ctypes.data_as(C.POINTER(C.c_ubyte)))
    print(f"  eht {size}x{size} at a = {a} in {time.time() - t:.1f} s, shadow px {shadow.sum()}")
    out.update(eht_view=np.array(NAKED_EHT), eht_flow=flow, eht_intensity=inten, eht_shadow=shadow)
    return out


def frame_fixture(R: po.Oracle, sc: po.Scene, w, h, ext) -> dict:
    t = time.time()
    out = R.trace_frame(sc, w, h, *ext)
    print(f"  traced {w}x{h} in {time.time() - t:.1f} s, outcomes {np.bincount(out['outcome'], minlength=6)}")
    return dict(outcome=out["outcome"].astype(np.uint8), r_disk=out["r_disk"], phi_disk=out["phi_disk"],
                g=out["g"], theta_inf=out["theta_inf"], phi_inf=out["phi_inf"], steps=out["steps"],
                width=w, height=h, extents=np.array(ext),
                scene=np.array([sc.a, sc.r_obs, sc.theta_obs, sc.phi_obs, sc.r_disk_in, sc.r_disk_out, sc.r_escape,
                                sc.capture_eps, sc.tol]))


def main() -> None:
    po.build(reference=True)
    R = po.Oracle(reference=True)
    print("naked_ref.npz")
    np.savez_compressed(os.path.join(HERE, "naked_ref.npz"), **naked_fixture(R))
    if os.environ.get("NAKED_ONLY"):
        return
    print("steps_blocks_ref.npz")
    np.savez_compressed(os.path.join(HERE, "steps_blocks_ref.npz"), **steps_blocks_fixture(R))
    if os.environ.get("BLOCKS_ONLY"):
        return
    print("steps_ref.npz")
    np.savez_compressed(os.path.join(HERE, "steps_ref.npz"), **steps_fixture(R))
    print("trajectory_ref.npz")
    np.savez_compressed(os.path.join(HERE, "trajectory_ref.npz"), **trajectory_fixture(R))
    print("framed_ref.npz")
    np.savez_compressed(os.path.join(HERE, "framed_ref.npz"), **framed_fixture(R))
    print("predict_ref.npz")
    np.savez_compressed(os.path.join(HERE, "predict_ref.npz"), **predict_fixture(R))
    print("eht_ref.npz")
    np.savez_compressed(os.path.join(HERE, "eht_ref.npz"), **eht_fixture(R))
    if os.environ.get("FRAMED_ONLY"):
        return
    print("c1_rk4_1e-4.npz")
    sc1 = po.scene(a=0.9, r_obs=50.0, theta_obs_deg=80.0, r_disk_out=20.0, tol=1e-4, method=po.RK4,
                   max_steps=5_000_000)
    np.savez_compressed(os.path.join(HERE, "c1_rk4_1e-4.npz"),
                        **frame_fixture(R, sc1, 128, 128, (-15.0, 15.0, -15.0, 15.0)))
    print("c2_rk4_1e-4.npz")
    sc2 = po.scene(a=0.998, r_obs=1000.0, theta_obs_deg=60.0, r_disk_out=30.0, tol=1e-4, method=po.RK4,
                   max_steps=5_000_000)
    np.savez_compressed(os.path.join(HERE, "c2_rk4_1e-4.npz"),
                        **frame_fixture(R, sc2, 96, 54, (-20.0, 20.0, -11.25, 11.25)))


if __name__ == "__main__":
    main()
