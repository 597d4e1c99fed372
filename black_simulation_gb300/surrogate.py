"""Host layer over libbhk's surrogate C ABI (include/bhk.h, bhk_surrogate_*).

The surrogate is the tracer's learned stand-in: a BF16 MLP from (a, theta_obs, log10 r_obs, alpha,
beta) to 3 outcome logits (captured, disk, escaped), r_disk / 30, ln g and the unit escape direction.
It has no counterpart in the reference (Black_simulation has no learned model); its labels come from
the tracer (`bhk.Context.trace_rays`). Training, gradients and inference run in libbhk's tcgen05
kernels; torch tensors only carry device memory here, and there is no CPU fallback.

Array conventions: inputs x are float32 (n, 5) CUDA tensors, classes uint8 (n,) with the
bhk outcome codes (1 captured, 2 disk, 3 escaped; 0 = unfinished, ignored by the loss), targets
float32 (n, 8) in the output convention (entries a class does not use are ignored).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import bhk

N_IN, N_OUT = 5, 8
WIDTHS = (64, 256)  # hidden widths the kernels are built for (bhk_surrogate_create_width)


def layers(width: int = 256):
    """(fan_out, fan_in) of the five layers for a hidden width; the head is padded to 16 outputs."""
    return ((width, 64), (width, width), (width, width), (width, width), (16, width))


LAYERS = layers(256)
R_DISK_SCALE = 30.0
ACCEPT = {"all": 0, "captured": 1}  # bhk_render_opts.accept (BHK_ACCEPT_ALL, BHK_ACCEPT_CAPTURED)


def layer_offsets(width: int = 256):
    """[(w_offset, b_offset, fan_out, fan_in)] into the flat FP32 parameter vector."""
    o, res = 0, []
    for fo, fi in layers(width):
        res.append((o, o + fo * fi, fo, fi))
        o += fo * fi + fo
    return res


def unpack(p: np.ndarray, width: int = 256):
    """Views (W, b) per layer of a flat parameter vector."""
    return [(p[w:w + fo * fi].reshape(fo, fi), p[b:b + fo]) for w, b, fo, fi in layer_offsets(width)]


def targets_from_rays(out: dict):
    """Training labels from tracer outputs (a dict of CUDA tensors as bhk.alloc_outputs gives):
    classes (uint8) and targets (float32, n x 8): r_disk / 30 and ln g for disk rays, the unit escape
    vector (sin th cos ph, sin th sin ph, cos th) of (theta_inf, phi_inf) for escaped rays."""
    import torch
    cls = out["outcome"].clone()
    n = cls.shape[0]
    t = torch.zeros((n, N_OUT), dtype=torch.float32, device=cls.device)
    disk = cls == bhk.DISK
    esc = cls == bhk.ESCAPED
    t[:, 3] = torch.where(disk, out["r_disk"] / R_DISK_SCALE, torch.zeros_like(out["r_disk"])).float()
    g = torch.where(disk, out["g"], torch.ones_like(out["g"]))
    t[:, 4] = torch.log(g.clamp_min(1e-30)).float()
    th, ph = out["theta_inf"], out["phi_inf"]
    st = torch.sin(th)
    for k, v in enumerate((st * torch.cos(ph), st * torch.sin(ph), torch.cos(th))):
        t[:, 5 + k] = torch.where(esc, v, torch.zeros_like(v)).float()
    return cls, t


class Surrogate:
    """A bhk_surrogate: FP32 master parameters, Adam state and BF16 weight copies on one device."""

    def __init__(self, device: int = 0, seed: int = 1, max_batch: int = 65536, width: int = 256):
        if width not in WIDTHS:
            raise ValueError(f"hidden width must be one of {WIDTHS}")
        self._h = C.c_void_p()
        bhk.check(bhk.lib().bhk_surrogate_create_width(device, seed, max_batch, width, C.byref(self._h)))
        self.device = device
        self.max_batch = max_batch
        self.width = width

    def close(self):
        if self._h:
            bhk.lib().bhk_surrogate_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_params(self) -> int:
        return int(bhk.lib().bhk_surrogate_param_count(self._h))

    def params(self) -> np.ndarray:
        p = np.empty(self.num_params(), dtype=np.float32)
        bhk.check(bhk.lib().bhk_surrogate_params(self._h, p.ctypes.data, 0))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params():
            raise ValueError("parameter vector has the wrong length")
        bhk.check(bhk.lib().bhk_surrogate_params(self._h, p.ctypes.data, 1))

    def fourier(self) -> np.ndarray:
        b = np.empty((32, N_IN), dtype=np.float32)
        bhk.check(bhk.lib().bhk_surrogate_fourier(self._h, b.ctypes.data, 0))
        return b

    def set_fourier(self, b: np.ndarray):
        b = np.ascontiguousarray(b, dtype=np.float32)
        if b.shape != (32, N_IN):
            raise ValueError("the Fourier matrix is 32 x 5")
        bhk.check(bhk.lib().bhk_surrogate_fourier(self._h, b.ctypes.data, 1))

    def set_loss_weights(self, ce: float = 1.0, r_disk: float = 10.0, log_g: float = 10.0, direction: float = 10.0):
        w = np.array([ce, r_disk, log_g, direction], dtype=np.float32)
        bhk.check(bhk.lib().bhk_surrogate_loss_weights(self._h, w.ctypes.data))

    def adam_state(self):
        """(m, v, step) of the optimiser."""
        m = np.empty(self.num_params(), np.float32)
        v = np.empty(self.num_params(), np.float32)
        st = C.c_int64(0)
        bhk.check(bhk.lib().bhk_surrogate_adam_state(self._h, m.ctypes.data, v.ctypes.data, C.byref(st), 0))
        return m, v, st.value

    def set_adam_state(self, m: np.ndarray, v: np.ndarray, step: int):
        m = np.ascontiguousarray(m, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        if m.size != self.num_params() or v.size != self.num_params():
            raise ValueError("moment vectors have the wrong length")
        st = C.c_int64(step)
        bhk.check(bhk.lib().bhk_surrogate_adam_state(self._h, m.ctypes.data, v.ctypes.data, C.byref(st), 1))

    def save(self, path: str):
        """Checkpoint: parameters, Fourier matrix and Adam state (numpy .npz)."""
        m, v, step = self.adam_state()
        np.savez(path, params=self.params(), fourier=self.fourier(), m=m, v=v, step=np.int64(step))

    def load(self, path: str):
        z = np.load(path)
        self.set_params(z["params"])
        self.set_fourier(z["fourier"])
        self.set_adam_state(z["m"], z["v"], int(z["step"]))

    @staticmethod
    def _check_batch(x, cls, tgt):
        if x.dtype != _torch().float32 or x.dim() != 2 or x.shape[1] != N_IN:
            raise ValueError("x must be float32 (n, 5)")
        if cls.dtype != _torch().uint8 or cls.shape[0] != x.shape[0]:
            raise ValueError("classes must be uint8 (n,)")
        if tgt.dtype != _torch().float32 or tuple(tgt.shape) != (x.shape[0], N_OUT):
            raise ValueError("targets must be float32 (n, 8)")

    def gradients(self, x, cls, tgt):
        """(gradient of the summed loss terms as a flat FP32 vector, loss terms[4]) for one batch."""
        self._check_batch(x, cls, tgt)
        g = np.empty(self.num_params(), dtype=np.float32)
        loss = np.empty(4, dtype=np.float32)
        bhk.check(bhk.lib().bhk_surrogate_gradients(self._h, bhk._ptr(x), bhk._ptr(cls), bhk._ptr(tgt), x.shape[0],
                                                    g.ctypes.data, loss.ctypes.data))
        return g, loss

    def train(self, x, cls, tgt, batch: int = 65536, steps: int = 100, lr: float = 1e-3, stream=None):
        """`steps` Adam steps (cosine learning rate from lr) over consecutive batches; returns the
        per-step loss terms (steps x 4: cross-entropy, r_disk MSE, ln g MSE, direction MSE)."""
        self._check_batch(x, cls, tgt)
        hist = np.empty((steps, 4), dtype=np.float32)
        bhk.check(bhk.lib().bhk_surrogate_train(self._h, bhk._ptr(x), bhk._ptr(cls), bhk._ptr(tgt), x.shape[0],
                                                batch, steps, lr, hist.ctypes.data, bhk._stream(stream)))
        return hist

    def predict(self, x, stream=None):
        """Network outputs (n x 8 float32 CUDA tensor) for inputs x (n x 5)."""
        torch = _torch()
        if x.dtype != torch.float32 or x.dim() != 2 or x.shape[1] != N_IN:
            raise ValueError("x must be float32 (n, 5)")
        y = torch.empty((x.shape[0], N_OUT), dtype=torch.float32, device=x.device)
        bhk.check(bhk.lib().bhk_surrogate_predict(self._h, bhk._ptr(x), x.shape[0], bhk._ptr(y), bhk._stream(stream)))
        return y


    def render(self, ctx, frames, opts=None, p_min: float = 0.99, band: float = 0.05, fallback: bool = True,
               out: Optional[dict] = None, stream=None, accept: str = "all"):
        """Surrogate + integrator-fallback render of `frames` (bhk.Frame list) through the fused
        inference kernel; returns (outputs as bhk.alloc_outputs gives, stats dict). accept="captured"
        keeps only the network's captured answers and traces every other ray."""
        n = sum(f.rays for f in frames)
        if out is None:
            out = bhk.alloc_outputs(n, f"cuda:{self.device}")
        arr = (bhk.FrameDescC * len(frames))(*[f.c() for f in frames])
        oc = (opts or bhk.TraceOpts("mixed")).c()
        if accept not in ACCEPT:
            raise ValueError(f"accept must be one of {sorted(ACCEPT)}")
        ro = bhk.RenderOptsC(p_min, band, 1 if fallback else 0, ACCEPT[accept])
        st = bhk.RenderStatsC()
        outc = bhk._out_c(out)
        bhk.check(bhk.lib().bhk_surrogate_render(self._h, ctx.h, arr, len(frames), C.byref(oc), C.byref(ro),
                                                 C.byref(outc), C.byref(st), bhk._stream(stream)))
        return out, {k: getattr(st, k) for k, _ in bhk.RenderStatsC._fields_}

    def fallback_list(self):
        """The last render's fallback pixels (int32 CUDA tensor, unordered)."""
        import torch
        n = C.c_int64()
        bhk.check(bhk.lib().bhk_surrogate_fallback_list(self._h, None, 0, C.byref(n)))
        t = torch.empty(n.value, dtype=torch.int32, device=f"cuda:{self.device}")
        if n.value:
            bhk.check(bhk.lib().bhk_surrogate_fallback_list(self._h, t.data_ptr(), n.value, C.byref(n)))
        return t


def make_dataset(ctx, n: int, seed: int = 1, r_disk_out: float = 30.0, opts=None, keep_rays: bool = False,
                 stream=None):
    """The surrogate's training set, generated on the device by bhk_surrogate_dataset: (x, classes,
    targets) CUDA tensors, plus the rays (5 x n float64: a, r_obs, theta_obs, alpha, beta) if asked."""
    import torch
    dev = f"cuda:{ctx.device}"
    x = torch.empty((n, N_IN), dtype=torch.float32, device=dev)
    cls = torch.empty(n, dtype=torch.uint8, device=dev)
    tgt = torch.empty((n, N_OUT), dtype=torch.float32, device=dev)
    rays = torch.empty((5, n), dtype=torch.float64, device=dev) if keep_rays else None
    oc = (opts or bhk.TraceOpts("mixed")).c()
    bhk.check(bhk.lib().bhk_surrogate_dataset(ctx.h, n, seed, r_disk_out, C.byref(oc), bhk._ptr(x), bhk._ptr(cls),
                                              bhk._ptr(tgt), bhk._ptr(rays), bhk._stream(stream)))
    return (x, cls, tgt, rays) if keep_rays else (x, cls, tgt)


def _torch():
    import torch
    return torch


def inputs_from_rays(a, r_obs, theta_obs, alpha, beta):
    """Network inputs (n x 5 float32) from per-ray float64 tensors."""
    import torch
    return torch.stack([a, theta_obs, torch.log10(r_obs), alpha, beta], dim=1).float().contiguous()


def sample_rays(n: int, seed: int, device="cuda", shadow_radius=None):
    """Training rays as the surrogate's training set draws them: a in [0, 0.998], theta_obs in
    [5, 89] deg, log10 r_obs uniform over [log10 20, 3], (alpha, beta) uniform in a disk of radius 1.5 x
    the shadow radius (a callable of (a, r_obs, theta_obs) arrays; default: the Schwarzschild value
    sqrt(27) M). Seeded numpy draws; float64 CUDA tensors (a, r_obs, theta_obs, alpha, beta)."""
    import torch
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.0, 0.998, n)
    th = np.deg2rad(rng.uniform(5.0, 89.0, n))
    r = 10.0 ** rng.uniform(np.log10(20.0), 3.0, n)
    R = np.full(n, np.sqrt(27.0)) if shadow_radius is None else np.asarray(shadow_radius(a, r, th))
    rad = 1.5 * R * np.sqrt(rng.uniform(0.0, 1.0, n))
    ang = rng.uniform(0.0, 2.0 * np.pi, n)
    al, be = rad * np.cos(ang), rad * np.sin(ang)
    return tuple(torch.from_numpy(np.ascontiguousarray(v)).to(device) for v in (a, r, th, al, be))


def shadow_radius(a: float, r_obs: float, theta_obs: float) -> float:
    """Largest distance of the analytic critical curve from the image centre (M, pinhole units)."""
    al, be = bhk.critical_curve(a, r_obs, theta_obs)
    return float(np.max(np.hypot(al, be)))


def orbit_frames(poses: int = 60, width: int = 3840, height: int = 2160, a: float = 0.998, r_obs: float = 30.0,
                 theta_from: float = 85.0, theta_to: float = 45.0, half_width_factor: float = 1.2,
                 r_disk_out: float = 30.0):
    """Camera poses along a circular orbit at r_obs with the inclination moving linearly from
    theta_from to theta_to (degrees), phi advancing 2 pi / poses per frame; image half-width
    half_width_factor x the frame's shadow radius, square pixels, disk from the ISCO to r_disk_out."""
    frames = []
    for k in range(poses):
        th = np.deg2rad(theta_from + (theta_to - theta_from) * (k / max(poses - 1, 1)))
        hw = half_width_factor * shadow_radius(a, r_obs, th)
        hh = hw * height / width
        f = bhk.Frame(a, r_obs, float(th), width, height, -hw, hw, -hh, hh, 0.0, r_disk_out)
        f.phi_obs = 2 * np.pi * k / poses
        frames.append(f)
    return frames


def pixel_inputs(frame, pixels=None):
    """Network inputs (float32 numpy, n x 5) of a frame's pixels (all, or the given local indices),
    computed as the fused inference kernel does."""
    n = frame.width * frame.height
    idx = np.arange(n) if pixels is None else np.asarray(pixels)
    row, col = idx // frame.width, idx % frame.width
    px = (frame.alpha_hi - frame.alpha_lo) / frame.width
    py = (frame.beta_hi - frame.beta_lo) / frame.height
    x = np.empty((idx.size, N_IN), np.float32)
    x[:, 0] = np.float32(frame.a)
    x[:, 1] = np.float32(frame.theta_obs)
    x[:, 2] = np.float32(np.log10(frame.r_obs))
    x[:, 3] = (frame.alpha_lo + (col + 0.5) * px).astype(np.float32)
    x[:, 4] = (frame.beta_hi - (row + 0.5) * py).astype(np.float32)
    return x
