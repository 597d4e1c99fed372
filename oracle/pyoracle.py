"""ctypes access to the oracle libraries (TEST INFRASTRUCTURE ONLY).

`Oracle()` loads oracle/liboracle.so, the C restatement of the reference's photon path
(oracle/kerr_oracle.c). `Oracle(reference=True)` loads oracle/_ref/libkerr_ref.so, the reference's
own kerr.cpp / trajectory.cpp / central.cpp / eht.cpp behind oracle/ref_driver.cpp; that one only
exists where the reference tree was present at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libkerr_ref.so")

UNFINISHED, CAPTURED, DISK, ESCAPED = 0, 1, 2, 3
ESCAPED_BEYOND, RING = 4, 5  # past |a| = 1: the sky of the r < 0 region, the ring singularity
RK4, DP5 = 0, 1


class Constants(C.Structure):
    _fields_ = [("E", C.c_double), ("L", C.c_double), ("Q", C.c_double), ("mu", C.c_double)]


class State(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("t", "r", "theta", "phi", "vr", "vtheta")]


class Derivs(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dt", "dr", "dtheta", "dphi", "dvr", "dvtheta")]


class Frame(C.Structure):
    _fields_ = [("e", (C.c_double * 4) * 4)]


class Scene(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("a", "r_obs", "theta_obs", "phi_obs", "r_disk_in", "r_disk_out",
                                           "r_escape", "capture_eps", "tol")] + [
        ("max_steps", C.c_int), ("method", C.c_int)]


class Ray(C.Structure):
    _fields_ = [("outcome", C.c_int32), ("steps", C.c_int32), ("rejected", C.c_int32), ("pad", C.c_int32)] + [
        (n, C.c_double) for n in ("r_disk", "phi_disk", "g", "theta_inf", "phi_inf", "E", "L", "Q")]


def build(reference: bool = False) -> None:
    """Compiles the oracle (and, when asked and the reference tree exists, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def reference_available() -> bool:
    return os.path.exists(LIB_REF)


def scene(a=0.9, r_obs=50.0, theta_obs_deg=80.0, phi_obs=0.0, r_disk_in=0.0, r_disk_out=20.0,
          r_escape=1000.0, capture_eps=1e-6, tol=1e-10, max_steps=20000, method=DP5) -> Scene:
    return Scene(a, r_obs, np.deg2rad(theta_obs_deg), phi_obs, r_disk_in, r_disk_out, r_escape, capture_eps,
                 tol, max_steps, method)


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _ptr(x, ct=C.c_double):
    return None if x is None else x.ctypes.data_as(C.POINTER(ct))


class Oracle:
    def __init__(self, reference: bool = False):
        path = LIB_REF if reference else LIB_ORACLE
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.p = "ref_" if reference else "orc_"
        self.reference = reference
        L = self.lib
        f = self._f
        f("derivatives", None, [C.c_double, C.POINTER(Constants), C.POINTER(State), C.POINTER(Derivs)])
        f("step_mino", None, [C.c_double, C.POINTER(Constants), C.POINTER(State), C.c_double])
        f("photon_step_size", C.c_double, [C.c_double, C.POINTER(Constants), C.POINTER(State), C.c_double])
        f("enforce_constraints", None, [C.c_double, C.POINTER(Constants), C.POINTER(State)])
        f("normalize_angles", None, [C.POINTER(State)])
        f("radial_potential", C.c_double, [C.c_double, C.POINTER(Constants), C.c_double])
        f("polar_potential", C.c_double, [C.c_double, C.POINTER(Constants), C.c_double])
        f("inflow_factor", C.c_double, [C.c_double] * 4)
        f("horizon_radius", C.c_double, [C.c_double])
        f("isco_radius", C.c_double, [C.c_double, C.c_int])
        f("photon_orbit_radius", C.c_double, [C.c_double, C.c_int])
        f("circular_omega", C.c_double, [C.c_double, C.c_double, C.c_int])
        f("launch_from_zamo", None, [C.c_double] * 4 + [_dp, C.c_double, C.POINTER(Constants), C.POINTER(State)])
        f("zamo_four_velocity", None, [C.c_double] * 3 + [_dp])
        f("observer_frame", None, [C.c_double] * 3 + [_dp, C.POINTER(Frame)])
        f("photon_from_frame", None, [C.c_double] * 4 + [C.POINTER(Frame), _dp, C.POINTER(Constants),
                                                         C.POINTER(State)])
        f("cartesian_velocity", None, [C.c_double] * 7 + [_dp])
        f("critical_curve", C.c_int, [C.c_double, C.c_double, C.c_int, _dp, _dp, C.c_int])
        f("critical_radius", C.c_double, [_dp, _dp, C.c_int, C.c_double])
        f("trace_ray", None, [C.POINTER(Scene), C.c_double, C.c_double, C.POINTER(Ray)])
        f("trace_frame", None, [C.POINTER(Scene), C.c_int, C.c_int] + [C.c_double] * 4 + [C.c_int, _ip] + [_dp] * 5
          + [_ip])
        if not reference:
            f("trace_rays", None, [C.POINTER(Scene), C.c_int64] + [_dp] * 5 + [C.c_int, _ip] + [_dp] * 5 + [_ip])
            f("critical_curve_finite", C.c_int, [C.c_double] * 3 + [C.c_int, _dp, _dp, C.c_int])
            f("no_radial_root_below", C.c_int, [C.c_double] * 6)
            f("pinhole_launch", None, [C.POINTER(Scene), C.c_double, C.c_double, C.POINTER(Constants),
                                       C.POINTER(State)])
            f("trace_framed", None, [C.POINTER(Scene), C.POINTER(Frame), _dp, C.POINTER(Ray)])
        else:
            f("eht_captured", C.c_int, [C.c_double] * 4)
            f("bending_angle", C.c_double, [C.c_double, C.c_double])
            f("trajectory_trace", C.c_int, [C.c_double] * 4 + [_dp, C.c_int] + [C.c_double] * 3 + [_dp])
            f("trajectory_trace_framed", C.c_int, [C.c_double] * 4 + [_dp, _dp, C.c_int] + [C.c_double] * 3 + [_dp])
            f("trace_framed", None, [C.POINTER(Scene), _dp, _dp, C.POINTER(Ray)])
        del L

    def _f(self, name, res, args):
        fn = getattr(self.lib, self.p + name)
        fn.restype = res
        fn.argtypes = args
        setattr(self, name + "_raw", fn)

    # -- per-step helpers with Python values ------------------------------------------------
    def derivatives(self, a, c: Constants, s: State) -> Derivs:
        d = Derivs()
        self.derivatives_raw(a, C.byref(c), C.byref(s), C.byref(d))
        return d

    def step_mino(self, a, c: Constants, s: State, h: float) -> State:
        x = State.from_buffer_copy(s)
        self.step_mino_raw(a, C.byref(c), C.byref(x), h)
        return x

    def photon_step_size(self, a, c, s, tol) -> float:
        return self.photon_step_size_raw(a, C.byref(c), C.byref(s), tol)

    def enforce_constraints(self, a, c, s) -> State:
        x = State.from_buffer_copy(s)
        self.enforce_constraints_raw(a, C.byref(c), C.byref(x))
        return x

    def normalize_angles(self, s) -> State:
        x = State.from_buffer_copy(s)
        self.normalize_angles_raw(C.byref(x))
        return x

    def launch_from_zamo(self, a, r, th, ph, v, mu):
        c, s = Constants(), State()
        vv = np.ascontiguousarray(v, dtype=np.float64)
        self.launch_from_zamo_raw(a, r, th, ph, _ptr(vv), mu, C.byref(c), C.byref(s))
        return c, s

    def zamo_frame(self, a, r, th) -> Frame:
        u = np.zeros(4)
        self.zamo_four_velocity_raw(a, r, th, _ptr(u))
        f = Frame()
        self.observer_frame_raw(a, r, th, _ptr(u), C.byref(f))
        return f

    def photon_from_frame(self, a, r, th, ph, f: Frame, look):
        c, s = Constants(), State()
        lk = np.ascontiguousarray(look, dtype=np.float64)
        self.photon_from_frame_raw(a, r, th, ph, C.byref(f), _ptr(lk), C.byref(c), C.byref(s))
        return c, s

    def critical_curve(self, a, incl, samples=400):
        cap = max(samples, 16) * 16 + 64
        al, be = np.zeros(cap), np.zeros(cap)
        n = self.critical_curve_raw(a, incl, samples, _ptr(al), _ptr(be), cap)
        return al[:n].copy(), be[:n].copy()

    def critical_curve_finite(self, a, r_obs, theta_obs, samples=400):
        cap = max(samples, 16) * 16 + 64
        al, be = np.zeros(cap), np.zeros(cap)
        n = self.critical_curve_finite_raw(a, r_obs, theta_obs, samples, _ptr(al), _ptr(be), cap)
        return al[:n].copy(), be[:n].copy()

    def critical_radius(self, al, be, psi):
        al = np.ascontiguousarray(al, dtype=np.float64)
        be = np.ascontiguousarray(be, dtype=np.float64)
        return self.critical_radius_raw(_ptr(al), _ptr(be), len(al), psi)

    def trace_framed(self, sc: Scene, frame, look) -> "Ray":
        """A camera at the scene's (r_obs, theta_obs, phi_obs) with an arbitrary frame (4 x 4 array
        e[k][i] or a Frame)."""
        r = Ray()
        lk = np.ascontiguousarray(look, dtype=np.float64)
        if self.reference:
            fr = np.ascontiguousarray(np.asarray(frame if not isinstance(frame, Frame) else
                                                 np.ctypeslib.as_array(frame.e), dtype=np.float64).reshape(16))
            self.trace_framed_raw(C.byref(sc), _ptr(fr), _ptr(lk), C.byref(r))
        else:
            if not isinstance(frame, Frame):
                f = Frame()
                np.ctypeslib.as_array(f.e)[:] = np.asarray(frame, dtype=np.float64).reshape(4, 4)
                frame = f
            self.trace_framed_raw(C.byref(sc), C.byref(frame), _ptr(lk), C.byref(r))
        return r

    def trace_ray(self, sc: Scene, alpha, beta) -> Ray:
        r = Ray()
        self.trace_ray_raw(C.byref(sc), alpha, beta, C.byref(r))
        return r

    def trace_frame(self, sc: Scene, width, height, alpha_lo, alpha_hi, beta_lo, beta_hi, nthreads=None):
        n = width * height
        nthreads = nthreads or os.cpu_count() or 1
        out = {k: np.zeros(n) for k in ("r_disk", "phi_disk", "g", "theta_inf", "phi_inf")}
        out["outcome"] = np.zeros(n, np.int32)
        out["steps"] = np.zeros(n, np.int32)
        self.trace_frame_raw(C.byref(sc), width, height, alpha_lo, alpha_hi, beta_lo, beta_hi, nthreads,
                             _ptr(out["outcome"], C.c_int32), _ptr(out["r_disk"]), _ptr(out["phi_disk"]),
                             _ptr(out["g"]), _ptr(out["theta_inf"]), _ptr(out["phi_inf"]),
                             _ptr(out["steps"], C.c_int32))
        return out

    def trace_rays(self, sc: Scene, a, r_obs, theta_obs, alpha, beta, nthreads=None):
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (a, r_obs, theta_obs, alpha, beta)]
        n = len(arrs[0])
        nthreads = nthreads or os.cpu_count() or 1
        out = {k: np.zeros(n) for k in ("r_disk", "phi_disk", "g", "theta_inf", "phi_inf")}
        out["outcome"] = np.zeros(n, np.int32)
        out["steps"] = np.zeros(n, np.int32)
        self.trace_rays_raw(C.byref(sc), n, *[_ptr(x) for x in arrs], nthreads, _ptr(out["outcome"], C.c_int32),
                            _ptr(out["r_disk"]), _ptr(out["phi_disk"]), _ptr(out["g"]), _ptr(out["theta_inf"]),
                            _ptr(out["phi_inf"]), _ptr(out["steps"], C.c_int32))
        return out


def pixel_grid(width, height, alpha_lo, alpha_hi, beta_lo, beta_hi):
    """Pixel-centre image-plane coordinates, row-major from the top (beta = beta_hi first)."""
    col = np.arange(width)
    row = np.arange(height)
    alpha = alpha_lo + (col + 0.5) * (alpha_hi - alpha_lo) / width
    beta = beta_hi - (row + 0.5) * (beta_hi - beta_lo) / height
    A, B = np.meshgrid(alpha, beta)
    return A.ravel(), B.ravel()


def band_distance(alpha, beta, curve_alpha, curve_beta):
    """Distance (M, image plane) from each point to the closed polyline (curve_alpha, curve_beta)."""
    px = np.asarray(alpha)[:, None]
    py = np.asarray(beta)[:, None]
    ax, ay = curve_alpha[None, :], curve_beta[None, :]
    bx, by = np.roll(curve_alpha, -1)[None, :], np.roll(curve_beta, -1)[None, :]
    ex, ey = bx - ax, by - ay
    ll = np.maximum(ex * ex + ey * ey, 1e-300)
    t = np.clip(((px - ax) * ex + (py - ay) * ey) / ll, 0.0, 1.0)
    dx, dy = px - (ax + t * ex), py - (ay + t * ey)
    return np.sqrt(dx * dx + dy * dy).min(axis=1)
