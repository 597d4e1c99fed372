"""Python host layer over libbhk's C ABI (include/bhk.h).

Names and argument meanings mirror the reference's kerr:: primitives (src/kerr.h) and its
ray-level drivers (trajectory::traceRay, eht::render): `derivatives`, `step_mino`,
`photon_step_size`, `enforce_constraints`, `normalize_angles`, `observer_frame`,
`photon_from_frame`, `launch_from_zamo`, plus the batch tracer `Context.trace_frames` /
`Context.trace_rays`. Arrays are torch tensors on a CUDA device (torch only supplies device
memory and streams here); every computation runs in libbhk's kernels. There is no CPU
fallback: without the built library or a GPU these raise.

Struct arrays are float64 tensors with a trailing dimension: constants (n, 4) = (E, L, Q, mu),
states (n, 6) = (t, r, theta, phi, vr, vtheta), derivatives (n, 6), frames (n, 4, 4).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import os
from typing import Optional, Sequence

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbhk.so")

OK, EINVAL, ECUDA, EUNFINISHED, ENOMEM = 0, 1, 2, 3, 4
UNFINISHED, CAPTURED, DISK, ESCAPED = 0, 1, 2, 3
# Past |a| = 1 (naked singularity, no horizon): the sky of the r < 0 region, and the ring singularity.
ESCAPED_BEYOND, RING = 4, 5
PREC_FP64, PREC_MIXED = 0, 1


class BhkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"bhk status {status}: {msg}")
        self.status = status


class FrameDescC(C.Structure):
    _fields_ = [("a", C.c_double), ("r_obs", C.c_double), ("theta_obs", C.c_double), ("phi_obs", C.c_double),
                ("width", C.c_int32), ("height", C.c_int32), ("alpha_lo", C.c_double), ("alpha_hi", C.c_double),
                ("beta_lo", C.c_double), ("beta_hi", C.c_double), ("r_disk_in", C.c_double),
                ("r_disk_out", C.c_double)]


class TraceOptsC(C.Structure):
    _fields_ = [("precision", C.c_int32), ("rtol", C.c_double), ("max_steps", C.c_int32), ("r_escape", C.c_double),
                ("capture_eps", C.c_double), ("reproject_every", C.c_int32), ("block", C.c_int32),
                ("chunk", C.c_int32), ("sort_buckets", C.c_int32), ("use_graph", C.c_int32),
                ("reg_budget", C.c_int32), ("pole_step_frac", C.c_double), ("fp64_turning", C.c_int32),
                ("pad", C.c_int32)]


class RaysOutC(C.Structure):
    _fields_ = [("outcome", C.c_void_p), ("r_disk", C.c_void_p), ("phi_disk", C.c_void_p), ("g", C.c_void_p),
                ("theta_inf", C.c_void_p), ("phi_inf", C.c_void_p), ("steps", C.c_void_p),
                ("rejected", C.c_void_p), ("energy", C.c_void_p), ("g_camera", C.c_void_p), ("b", C.c_void_p),
                ("q", C.c_void_p), ("r_min", C.c_void_p), ("delay", C.c_void_p), ("turns", C.c_void_p)]


class StatsC(C.Structure):
    _fields_ = [("rays", C.c_int64), ("accepted_steps", C.c_int64), ("rejected_steps", C.c_int64),
                ("rescued", C.c_int64), ("unfinished", C.c_int64), ("block", C.c_int32), ("chunk", C.c_int32),
                ("sort_buckets", C.c_int32), ("grid", C.c_int32), ("reg_budget", C.c_int32), ("pad", C.c_int32),
                ("kernel_ms", C.c_double), ("fp64_turning_steps", C.c_int64)]


class EhtViewC(C.Structure):
    _fields_ = [("a", C.c_double), ("inclination", C.c_double), ("half_width", C.c_double), ("size", C.c_int32),
                ("pad", C.c_int32), ("frequency", C.c_double), ("mass_solar", C.c_double)]


class EhtFlowC(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("n0", "T0", "beta", "keplerian", "height", "sin_theta_b")]


class PathOutC(C.Structure):
    _fields_ = [("fate", C.c_void_p), ("duration", C.c_void_p), ("r_min", C.c_void_p), ("r_max", C.c_void_p),
                ("periapses", C.c_void_p), ("precession_deg", C.c_void_p), ("points", C.c_void_p),
                ("n_points", C.c_void_p)]


class RenderOptsC(C.Structure):
    _fields_ = [("p_min", C.c_double), ("band", C.c_double), ("fallback", C.c_int32), ("accept", C.c_int32)]


class RenderStatsC(C.Structure):
    _fields_ = [("rays", C.c_int64), ("fallback", C.c_int64), ("infer_ms", C.c_double), ("trace_ms", C.c_double),
                ("accept", C.c_int32), ("grid", C.c_int32)]


@dataclasses.dataclass
class Frame:
    """One ZAMO pinhole camera frame (bhk_frame_desc). Angles in radians."""
    a: float
    r_obs: float
    theta_obs: float
    width: int
    height: int
    alpha_lo: float
    alpha_hi: float
    beta_lo: float
    beta_hi: float
    r_disk_in: float = 0.0
    r_disk_out: float = 20.0
    phi_obs: float = 0.0

    @property
    def rays(self) -> int:
        return self.width * self.height

    def c(self) -> FrameDescC:
        return FrameDescC(self.a, self.r_obs, self.theta_obs, self.phi_obs, self.width, self.height, self.alpha_lo,
                          self.alpha_hi, self.beta_lo, self.beta_hi, self.r_disk_in, self.r_disk_out)


@dataclasses.dataclass
class TraceOpts:
    """bhk_trace_opts; zeros mean the library defaults."""
    precision: str = "fp64"
    rtol: float = 0.0
    max_steps: int = 0
    r_escape: float = 0.0
    capture_eps: float = 0.0
    reproject_every: int = 0
    block: int = 0
    chunk: int = 0
    sort_buckets: int = 0
    use_graph: bool = False
    reg_budget: int = 0
    pole_step_frac: float = 0.0
    fp64_turning: bool = False

    def c(self) -> TraceOptsC:
        prec = {"fp64": PREC_FP64, "mixed": PREC_MIXED}[self.precision]
        return TraceOptsC(prec, self.rtol, self.max_steps, self.r_escape, self.capture_eps, self.reproject_every,
                          self.block, self.chunk, self.sort_buckets, 1 if self.use_graph else 0, self.reg_budget,
                          self.pole_step_frac, 1 if self.fp64_turning else 0, 0)


_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Loads libbhk.so (built by black_simulation_gb300.build). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with black_simulation_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    vp, i64, d = C.c_void_p, C.c_int64, C.c_double
    sig = {
        "bhk_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
        "bhk_destroy": (C.c_int, [vp]),
        "bhk_last_error": (C.c_char_p, []),
        "bhk_version": (C.c_char_p, []),
        "bhk_flops_per_step": (d, []),
        "bhk_flops_per_rejected_step": (d, []),
        "bhk_derivatives": (C.c_int, [d, vp, vp, vp, i64, vp]),
        "bhk_step_mino": (C.c_int, [d, vp, vp, vp, i64, vp]),
        "bhk_photon_step_size": (C.c_int, [d, vp, vp, d, vp, i64, vp]),
        "bhk_enforce_constraints": (C.c_int, [d, vp, vp, i64, vp]),
        "bhk_normalize_angles": (C.c_int, [vp, i64, vp]),
        "bhk_potentials": (C.c_int, [d, vp, vp, vp, vp, i64, vp]),
        "bhk_observer_frame": (C.c_int, [d, vp, vp, vp, vp, i64, vp]),
        "bhk_photon_from_frame": (C.c_int, [d, d, d, d, vp, vp, vp, vp, i64, vp]),
        "bhk_launch_from_zamo": (C.c_int, [d, d, d, d, vp, d, vp, vp, i64, vp]),
        "bhk_cartesian_velocity": (C.c_int, [d, vp, vp, vp, i64, vp]),
        "bhk_trace_frames": (C.c_int, [vp, C.POINTER(FrameDescC), C.c_int32, C.POINTER(TraceOptsC),
                                       C.POINTER(RaysOutC), vp]),
        "bhk_trace_frames_host": (C.c_int, [vp, C.POINTER(FrameDescC), C.c_int32, C.POINTER(TraceOptsC),
                                            C.POINTER(RaysOutC)]),
        "bhk_trace_rays": (C.c_int, [vp, i64, vp, vp, vp, vp, vp, d, d, C.POINTER(TraceOptsC),
                                     C.POINTER(RaysOutC), vp]),
        "bhk_get_stats": (C.c_int, [vp, C.POINTER(StatsC)]),
        "bhk_autotune": (C.c_int, [vp, C.POINTER(FrameDescC), C.c_int32, C.POINTER(TraceOptsC),
                                   C.POINTER(StatsC)]),
        "bhk_critical_curve": (C.c_int, [d, d, d, C.c_int32, vp, vp, C.c_int32, C.POINTER(C.c_int32)]),
        "bhk_fp32_fma_peak": (C.c_int, [C.c_int, C.POINTER(d)]),
        "bhk_tc_gemm": (C.c_int, [vp, vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp]),
        "bhk_trace_frames_static": (C.c_int, [C.POINTER(FrameDescC), C.c_int32, C.POINTER(TraceOptsC),
                                              C.POINTER(RaysOutC), vp]),
        "bhk_surrogate_num_params": (i64, []),
        "bhk_surrogate_create": (C.c_int, [C.c_int, C.c_uint64, C.c_int32, C.POINTER(vp)]),
        "bhk_surrogate_create_width": (C.c_int, [C.c_int, C.c_uint64, C.c_int32, C.c_int32, C.POINTER(vp)]),
        "bhk_surrogate_width": (C.c_int32, [vp]),
        "bhk_surrogate_param_count": (i64, [vp]),
        "bhk_surrogate_destroy": (C.c_int, [vp]),
        "bhk_surrogate_params": (C.c_int, [vp, vp, C.c_int32]),
        "bhk_surrogate_fourier": (C.c_int, [vp, vp, C.c_int32]),
        "bhk_surrogate_loss_weights": (C.c_int, [vp, vp]),
        "bhk_surrogate_adam_state": (C.c_int, [vp, vp, vp, C.POINTER(i64), C.c_int32]),
        "bhk_surrogate_gradients": (C.c_int, [vp, vp, vp, vp, C.c_int32, vp, vp]),
        "bhk_surrogate_train": (C.c_int, [vp, vp, vp, vp, i64, C.c_int32, i64, C.c_float, vp, vp]),
        "bhk_surrogate_predict": (C.c_int, [vp, vp, i64, vp, vp]),
        "bhk_surrogate_render": (C.c_int, [vp, vp, C.POINTER(FrameDescC), C.c_int32, C.POINTER(TraceOptsC),
                                           C.POINTER(RenderOptsC), C.POINTER(RaysOutC), C.POINTER(RenderStatsC), vp]),
        "bhk_surrogate_fallback_list": (C.c_int, [vp, vp, i64, C.POINTER(i64)]),
        "bhk_surrogate_dataset": (C.c_int, [vp, i64, C.c_uint64, d, C.POINTER(TraceOptsC), vp, vp, vp, vp, vp]),
        "bhk_trace_pixels": (C.c_int, [vp, C.POINTER(FrameDescC), C.c_int32, vp, i64, C.POINTER(TraceOptsC),
                                       C.POINTER(RaysOutC), vp]),
        "bhk_trace_rays_framed": (C.c_int, [vp, i64, vp, vp, vp, vp, vp, vp, d, d, C.POINTER(TraceOptsC),
                                            C.POINTER(RaysOutC), vp]),
        "bhk_eht_render": (C.c_int, [C.POINTER(EhtViewC), C.POINTER(EhtFlowC), C.c_int32, vp, vp, vp, vp]),
        "bhk_predict": (C.c_int, [d, vp, vp, i64, d, d, C.c_int32, d, d, vp, C.POINTER(PathOutC), vp]),
        "bhk_eht_flux": (d, [vp, C.c_int32, d, d]),
        "bhk_eht_calibrate": (C.c_int, [C.POINTER(EhtViewC), C.POINTER(EhtFlowC), d, d, C.POINTER(d)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int, allow_unfinished: bool = False) -> int:
    if status == OK or (allow_unfinished and status == EUNFINISHED):
        return status
    raise BhkError(status, lib().bhk_last_error().decode())


def exported_symbols() -> list[str]:
    """Symbols include/bhk.h declares (for the load/export test)."""
    hdr = os.path.join(os.path.dirname(PKG), "include", "bhk.h")
    import re
    text = open(hdr).read()
    return sorted(set(re.findall(r"\b(bhk_[a-z_0-9]+)\s*\(", text)))


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    import torch
    if isinstance(t, torch.Tensor):
        if not t.is_cuda:
            raise ValueError("libbhk arrays must be CUDA tensors")
        if not t.is_contiguous():
            raise ValueError("libbhk arrays must be contiguous")
        return t.data_ptr()
    return int(t)


CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy: the legacy default stream, which torch's handle 0 denotes


def _stream(stream) -> Optional[int]:
    """The cudaStream_t to pass: torch's current stream unless given. Handle 0 (torch's default
    stream) goes over as cudaStreamLegacy, since NULL means the context's own stream to libbhk."""
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    h = int(getattr(stream, "cuda_stream", stream))
    return h if h != 0 else CUDA_STREAM_LEGACY


def _n(t, width) -> int:
    if t.dtype.itemsize != 8:
        raise ValueError("expected float64")
    if t.dim() != 2 or t.shape[1] != width:
        raise ValueError(f"expected shape (n, {width})")
    return t.shape[0]


# --------------------------------------------------------------------------- per-step mirrors ----

def derivatives(a: float, c, s, stream=None):
    """kerr::derivatives for each row: returns (n, 6) float64 (dt, dr, dtheta, dphi, dvr, dvtheta)."""
    import torch
    n = _n(s, 6)
    d = torch.empty((n, 6), dtype=torch.float64, device=s.device)
    check(lib().bhk_derivatives(a, _ptr(c), _ptr(s), _ptr(d), n, _stream(stream)))
    return d


def step_mino(a: float, c, s, h, stream=None):
    """kerr::stepMino in place on each row of s with step h[i]."""
    check(lib().bhk_step_mino(a, _ptr(c), _ptr(s), _ptr(h), _n(s, 6), _stream(stream)))
    return s


def photon_step_size(a: float, c, s, tolerance: float, stream=None):
    import torch
    n = _n(s, 6)
    h = torch.empty(n, dtype=torch.float64, device=s.device)
    check(lib().bhk_photon_step_size(a, _ptr(c), _ptr(s), tolerance, _ptr(h), n, _stream(stream)))
    return h


def enforce_constraints(a: float, c, s, stream=None):
    check(lib().bhk_enforce_constraints(a, _ptr(c), _ptr(s), _n(s, 6), _stream(stream)))
    return s


def normalize_angles(s, stream=None):
    check(lib().bhk_normalize_angles(_ptr(s), _n(s, 6), _stream(stream)))
    return s


def potentials(a: float, c, s, stream=None):
    import torch
    n = _n(s, 6)
    R = torch.empty(n, dtype=torch.float64, device=s.device)
    Th = torch.empty(n, dtype=torch.float64, device=s.device)
    check(lib().bhk_potentials(a, _ptr(c), _ptr(s), _ptr(R), _ptr(Th), n, _stream(stream)))
    return R, Th


def observer_frame(a: float, r, theta, u=None, stream=None):
    """kerr::observerFrame at each (r[i], theta[i]); u None = the ZAMO. Returns (n, 4, 4)."""
    import torch
    n = r.shape[0]
    f = torch.empty((n, 4, 4), dtype=torch.float64, device=r.device)
    check(lib().bhk_observer_frame(a, _ptr(r), _ptr(theta), _ptr(u), _ptr(f), n, _stream(stream)))
    return f


def photon_from_frame(a: float, r: float, theta: float, phi: float, frame, look, stream=None):
    """kerr::photonFromFrame for one camera frame (4, 4) and n look directions (n, 3)."""
    import torch
    n = _n(look, 3)
    c = torch.empty((n, 4), dtype=torch.float64, device=look.device)
    s = torch.empty((n, 6), dtype=torch.float64, device=look.device)
    check(lib().bhk_photon_from_frame(a, r, theta, phi, _ptr(frame.contiguous()), _ptr(look), _ptr(c), _ptr(s), n,
                                      _stream(stream)))
    return c, s


def launch_from_zamo(a: float, r: float, theta: float, phi: float, v, mu: float = 0.0, stream=None):
    import torch
    n = _n(v, 3)
    c = torch.empty((n, 4), dtype=torch.float64, device=v.device)
    s = torch.empty((n, 6), dtype=torch.float64, device=v.device)
    check(lib().bhk_launch_from_zamo(a, r, theta, phi, _ptr(v), mu, _ptr(c), _ptr(s), n, _stream(stream)))
    return c, s


def cartesian_velocity(a: float, c, s, stream=None):
    import torch
    n = _n(s, 6)
    out = torch.empty((n, 3), dtype=torch.float64, device=s.device)
    check(lib().bhk_cartesian_velocity(a, _ptr(c), _ptr(s), _ptr(out), n, _stream(stream)))
    return out


def critical_curve(a: float, r_obs: float, theta_obs: float, samples: int = 400):
    cap = max(samples, 16) * 16 + 64
    al = np.zeros(cap)
    be = np.zeros(cap)
    n = C.c_int32(0)
    check(lib().bhk_critical_curve(a, r_obs, theta_obs, samples, al.ctypes.data, be.ctypes.data, cap, C.byref(n)))
    return al[:n.value].copy(), be[:n.value].copy()


def pixel_alpha_beta(frame: "Frame", local):
    """Image-plane (alpha, beta) of the frame's pixels with row-major indices `local` (numpy), as the
    tracer places them: pixel centres, rows from beta_hi down."""
    local = np.asarray(local, dtype=np.int64)
    row, col = np.divmod(local, frame.width)
    alpha = frame.alpha_lo + (col + 0.5) * (frame.alpha_hi - frame.alpha_lo) / frame.width
    beta = frame.beta_hi - (row + 0.5) * (frame.beta_hi - frame.beta_lo) / frame.height
    return alpha, beta


def _segment_distance(px, py, ax, ay, bx, by):
    ex, ey = bx - ax, by - ay
    ll = np.maximum(ex * ex + ey * ey, 1e-300)
    t = np.clip(((px - ax) * ex + (py - ay) * ey) / ll, 0.0, 1.0)
    dx, dy = px - (ax + t * ex), py - (ay + t * ey)
    return np.sqrt(dx * dx + dy * dy)


def curve_distance(alpha, beta, curve_alpha, curve_beta, spacing: float = 1e-3, near: float = 0.2):
    """Image-plane distance (M) from each point (alpha, beta) to the closed polyline through
    (curve_alpha, curve_beta): the analytic critical curve critical_curve() returns, symmetric about
    beta = 0 and star-shaped about its centre. Every point gets the polar estimate |rho - rho_c(psi)|
    rho_c / sqrt(rho_c^2 + rho_c'^2) about the centre; points it puts within `near` get the exact
    distance (the polyline resampled to vertices at most `spacing` apart, the nearest vertex by k-d tree,
    the distance taken to the two segments beside it)."""
    alpha, beta = np.asarray(alpha, dtype=np.float64), np.asarray(beta, dtype=np.float64)
    ax, ay = np.asarray(curve_alpha, dtype=np.float64), np.asarray(curve_beta, dtype=np.float64)
    ac = 0.5 * (ax.min() + ax.max())
    up = ay >= 0.0
    psi_c = np.arctan2(ay[up], ax[up] - ac)
    rho_c = np.hypot(ay[up], ax[up] - ac)
    o = np.argsort(psi_c)
    psi_c, rho_c = psi_c[o], rho_c[o]
    drho = np.gradient(rho_c, psi_c) if psi_c.size > 2 else np.zeros_like(rho_c)
    psi = np.arctan2(np.abs(beta), alpha - ac)
    rho = np.hypot(beta, alpha - ac)
    rc = np.interp(psi, psi_c, rho_c)
    kn = rc / np.sqrt(rc * rc + np.interp(psi, psi_c, drho) ** 2)
    out = np.abs(rho - rc) * kn
    close = np.nonzero(out < near)[0]
    if close.size == 0:
        return out
    bx, by = np.roll(ax, -1), np.roll(ay, -1)
    seg = np.hypot(bx - ax, by - ay)
    pieces = np.maximum(1, np.ceil(seg / spacing).astype(np.int64))
    start = np.repeat(np.arange(ax.size), pieces)
    frac = (np.arange(pieces.sum()) - np.repeat(np.cumsum(pieces) - pieces, pieces)) / np.repeat(pieces, pieces)
    vx = ax[start] + frac * (bx - ax)[start]
    vy = ay[start] + frac * (by - ay)[start]
    from scipy.spatial import cKDTree
    d, j = cKDTree(np.stack([vx, vy], 1)).query(np.stack([alpha[close], beta[close]], 1),
                                               distance_upper_bound=2.0 * near)
    ok = np.isfinite(d)
    c, j = close[ok], j[ok]
    nv = vx.size
    prev, nxt = (j - 1) % nv, (j + 1) % nv
    out[c] = np.minimum(_segment_distance(alpha[c], beta[c], vx[prev], vy[prev], vx[j], vy[j]),
                        _segment_distance(alpha[c], beta[c], vx[j], vy[j], vx[nxt], vy[nxt]))
    return out


FATES = ("bound", "circular", "plunges", "escapes", "hits_surface")  # trajectory::Fate


def predict(a: float, c, s, max_time: float, min_spacing: float = 0.5, max_points: int = 4000,
            surface: float = 0.0, escape_radius: float = 2000.0, points: bool = True, stream=None) -> dict:
    """trajectory::predict for n massive particles at once: constants (n, 4) and states (n, 6) float64
    CUDA tensors -> dict of per-particle fate, duration, r_min, r_max, periapses, precession_deg,
    n_points, points ((n, max_points + 1, 3), if asked) and the final states."""
    import torch
    n = _n(c, 4)
    if _n(s, 6) != n:
        raise ValueError("constants and states differ in length")
    dev = c.device
    out = {"fate": torch.empty(n, dtype=torch.int32, device=dev), "periapses": torch.empty(n, dtype=torch.int32, device=dev),
           "n_points": torch.empty(n, dtype=torch.int32, device=dev), "state": torch.empty((n, 6), dtype=torch.float64, device=dev)}
    for k in ("duration", "r_min", "r_max", "precession_deg"):
        out[k] = torch.empty(n, dtype=torch.float64, device=dev)
    if points:
        out["points"] = torch.empty((n, max_points + 1, 3), dtype=torch.float64, device=dev)
    po = PathOutC(*[_ptr(out.get(k)) for k in ("fate", "duration", "r_min", "r_max", "periapses", "precession_deg",
                                                 "points", "n_points")])
    check(lib().bhk_predict(a, _ptr(c.contiguous()), _ptr(s.contiguous()), n, max_time, min_spacing, max_points, surface,
                            escape_radius, _ptr(out["state"]), C.byref(po), _stream(stream)))
    return out


def flops_per_step() -> float:
    return float(lib().bhk_flops_per_step())


def flops_per_rejected_step() -> float:
    return float(lib().bhk_flops_per_rejected_step())


def tc_gemm(A, B, splits: int = 1, stream=None):
    """C = A @ B.T on the tcgen05 GEMM kernel (A: M x K, B: N x K, BF16 CUDA tensors) -> FP32 M x N."""
    import torch
    M, K = A.shape
    N = B.shape[0]
    Cm = torch.zeros((M, N), dtype=torch.float32, device=A.device)
    check(lib().bhk_tc_gemm(_ptr(A.contiguous()), _ptr(B.contiguous()), _ptr(Cm), M, N, K, splits, _stream(stream)))
    return Cm


def fp32_fma_peak_tflops(device: int = 0) -> float:
    """Measured FP32 FMA throughput of the device (TFLOP/s)."""
    x = C.c_double(0.0)
    check(lib().bhk_fp32_fma_peak(device, C.byref(x)))
    return x.value


# ----------------------------------------------------------------------------- batch tracer ----

FIELDS = ("outcome", "r_disk", "phi_disk", "g", "theta_inf", "phi_inf", "steps", "rejected")
# The rest of trajectory::RayReport, allocated on request (56 more bytes per ray).
EXTRA_FIELDS = ("energy", "g_camera", "b", "q", "r_min", "delay", "turns")


def alloc_outputs(n: int, device="cuda", extras: bool = False):
    import torch
    out = {k: torch.empty(n, dtype=torch.float64, device=device) for k in FIELDS[1:6]}
    out["outcome"] = torch.empty(n, dtype=torch.uint8, device=device)
    out["steps"] = torch.empty(n, dtype=torch.int32, device=device)
    out["rejected"] = torch.empty(n, dtype=torch.int32, device=device)
    if extras:
        out.update({k: torch.empty(n, dtype=torch.float64, device=device) for k in EXTRA_FIELDS})
    return out


def _out_c(out: dict) -> RaysOutC:
    return RaysOutC(*[_ptr(out.get(k)) for k in FIELDS + EXTRA_FIELDS])


class Context:
    """A bhk_context: stream, scratch, autotuned launch shape, cached CUDA graph."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().bhk_create(device, C.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            lib().bhk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def _frames(frames: Sequence[Frame]):
        arr = (FrameDescC * len(frames))(*[f.c() for f in frames])
        return arr, len(frames)

    def trace_frames(self, frames: Sequence[Frame], opts: TraceOpts = TraceOpts(), out: Optional[dict] = None,
                     stream=None) -> dict:
        """Traces all pixels of `frames` into device tensors (allocated if out is None)."""
        arr, nf = self._frames(frames)
        n = sum(f.rays for f in frames)
        if out is None:
            out = alloc_outputs(n, f"cuda:{self.device}")
        oc = opts.c()
        outc = _out_c(out)
        check(lib().bhk_trace_frames(self.h, arr, nf, C.byref(oc), C.byref(outc), _stream(stream)))
        return out

    def trace_frames_host(self, frames: Sequence[Frame], opts: TraceOpts = TraceOpts(),
                          out: Optional[dict] = None) -> tuple[dict, int]:
        """Host-buffer call: numpy outputs (pinned or pageable), synchronous. Returns (out, status)."""
        n = sum(f.rays for f in frames)
        if out is None:
            out = {k: np.empty(n) for k in FIELDS[1:6]}
            out["outcome"] = np.empty(n, np.uint8)
            out["steps"] = np.empty(n, np.int32)
            out["rejected"] = np.empty(n, np.int32)
        arr, nf = self._frames(frames)
        oc = opts.c()
        ptrs = []
        for k in FIELDS + EXTRA_FIELDS:
            v = out.get(k)
            ptrs.append(None if v is None else (v.data_ptr() if hasattr(v, "data_ptr") else v.ctypes.data))
        outc = RaysOutC(*ptrs)
        st = check(lib().bhk_trace_frames_host(self.h, arr, nf, C.byref(oc), C.byref(outc)), allow_unfinished=True)
        return out, st

    def trace_rays(self, a, r_obs, theta_obs, alpha, beta, r_disk_in: float = 0.0, r_disk_out: float = 20.0,
                   opts: TraceOpts = TraceOpts(), out: Optional[dict] = None, stream=None) -> dict:
        n = a.shape[0]
        if out is None:
            out = alloc_outputs(n, a.device)
        oc = opts.c()
        outc = _out_c(out)
        check(lib().bhk_trace_rays(self.h, n, _ptr(a), _ptr(r_obs), _ptr(theta_obs), _ptr(alpha), _ptr(beta),
                                   r_disk_in, r_disk_out, C.byref(oc), C.byref(outc), _stream(stream)))
        return out

    def trace_pixels(self, frames: Sequence[Frame], pixels, opts: TraceOpts = TraceOpts(), out: Optional[dict] = None,
                     stream=None) -> dict:
        """Traces the listed global pixel indices (int32 CUDA tensor) of `frames`; compact outputs."""
        if pixels.dtype.itemsize != 4:
            raise ValueError("pixels must be int32")
        arr, nf = self._frames(frames)
        n = pixels.shape[0]
        if out is None:
            out = alloc_outputs(n, f"cuda:{self.device}")
        oc = opts.c()
        outc = _out_c(out)
        check(lib().bhk_trace_pixels(self.h, arr, nf, _ptr(pixels), n, C.byref(oc), C.byref(outc), _stream(stream)))
        return out

    def trace_rays_framed(self, a, r, theta, phi, frames, look, r_disk_in: float = 0.0, r_disk_out: float = 20.0,
                          opts: TraceOpts = TraceOpts(), out: Optional[dict] = None, stream=None) -> dict:
        """trajectory::traceRay's call shape, batched: per-ray camera position (float64 (n,) each), frame
        (float64 (n, 4, 4), e[k][mu]) and unit look direction on the frame's (r, theta, phi) axes ((n, 3))."""
        n = a.shape[0]
        if tuple(frames.shape) != (n, 4, 4) or tuple(look.shape) != (n, 3):
            raise ValueError("frames must be (n, 4, 4) and look (n, 3)")
        if out is None:
            out = alloc_outputs(n, a.device)
        oc = opts.c()
        outc = _out_c(out)
        check(lib().bhk_trace_rays_framed(self.h, n, _ptr(a), _ptr(r), _ptr(theta), _ptr(phi), _ptr(frames),
                                          _ptr(look), r_disk_in, r_disk_out, C.byref(oc), C.byref(outc),
                                          _stream(stream)))
        return out

    def stats(self) -> dict:
        s = StatsC()
        check(lib().bhk_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in StatsC._fields_}

    def autotune(self, frames: Sequence[Frame], opts: TraceOpts = TraceOpts()) -> dict:
        arr, nf = self._frames(frames)
        oc = opts.c()
        s = StatsC()
        check(lib().bhk_autotune(self.h, arr, nf, C.byref(oc), C.byref(s)))
        return {k: getattr(s, k) for k, _ in StatsC._fields_}


# ------------------------------------------------------------------------------ eht::render ----

EHT_FLOW_DEFAULTS = dict(n0=1e5, T0=4e11, beta=10.0, keplerian=0.9, height=1.0, sin_theta_b=0.8165)


def eht_view(a=0.9, inclination=0.3, half_width=16.0, size=128, frequency=230e9, mass_solar=6.5e9) -> EhtViewC:
    """eht::View (defaults as the reference's, src/eht.h)."""
    return EhtViewC(a, inclination, half_width, size, 0, frequency, mass_solar)


def eht_flow(**kw) -> EhtFlowC:
    """eht::Flow (defaults as the reference's, src/eht.h)."""
    v = dict(EHT_FLOW_DEFAULTS)
    v.update(kw)
    return EhtFlowC(*[v[k] for k in ("n0", "T0", "beta", "keplerian", "height", "sin_theta_b")])


def eht_render(view: EhtViewC, flow: EhtFlowC, with_light: bool = True, device="cuda", stream=None):
    """eht::render on the GPU: (intensity float64 (size, size), shadow uint8 (size, size), steps int32)
    CUDA tensors, row-major from beta = +half_width."""
    import torch
    n = view.size * view.size
    inten = torch.empty(n, dtype=torch.float64, device=device)
    shadow = torch.empty(n, dtype=torch.uint8, device=device)
    steps = torch.empty(n, dtype=torch.int32, device=device)
    check(lib().bhk_eht_render(C.byref(view), C.byref(flow), 1 if with_light else 0, _ptr(inten), _ptr(shadow),
                               _ptr(steps), _stream(stream)))
    sh = (view.size, view.size)
    return inten.view(sh), shadow.view(sh), steps.view(sh)


def eht_flux(intensity, half_width: float, theta_g_uas: float) -> float:
    """eht::flux (Jy) of an intensity image (host array or tensor)."""
    arr = np.ascontiguousarray(intensity.cpu().numpy() if hasattr(intensity, "cpu") else intensity, dtype=np.float64)
    return float(lib().bhk_eht_flux(arr.ctypes.data, arr.shape[0], half_width, theta_g_uas))


def eht_calibrate(view: EhtViewC, flow: EhtFlowC, target_jy: float, theta_g_uas: float) -> float:
    """eht::calibrate: the density n0 that gives target_jy."""
    n0 = C.c_double(0.0)
    check(lib().bhk_eht_calibrate(C.byref(view), C.byref(flow), target_jy, theta_g_uas, C.byref(n0)))
    return n0.value


# ------------------------------------------------------------------------ standard workloads ----

def isco_prograde(a: float) -> float:
    """Bardeen-Press-Teukolsky prograde ISCO (host helper for workload set-up and tests)."""
    z1 = 1 + (1 - a * a) ** (1 / 3) * ((1 + a) ** (1 / 3) + (1 - a) ** (1 / 3))
    z2 = math.sqrt(3 * a * a + z1 * z1)
    return 3 + z2 - math.sqrt(max(0.0, (3 - z1) * (3 + z1 + 2 * z2)))


def frame_c1(width: int = 128, height: int = 128) -> Frame:
    """a=0.9, r_obs=50, theta=80 deg, alpha,beta in [-15, 15], disk ISCO..20 (the FP64 parity frame)."""
    return Frame(0.9, 50.0, math.radians(80.0), width, height, -15.0, 15.0, -15.0, 15.0, 0.0, 20.0)


def frame_c2(width: int = 1920, height: int = 1080) -> Frame:
    """a=0.998, r_obs=1000, theta=60 deg, alpha in +-20 with square pixels, disk ISCO..30 (1080p)."""
    half_b = 20.0 * height / width
    return Frame(0.998, 1000.0, math.radians(60.0), width, height, -20.0, 20.0, -half_b, half_b, 0.0, 30.0)
