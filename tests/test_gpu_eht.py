"""eht::render on the GPU (bhk_eht_render): the synchrotron image and shadow of the reference's hot
flow, against images rendered by the reference itself (tests/golden/eht_ref.npz), and the
reference's own EHT checks (tests/test_kerr.cpp:2322-2355) re-run on the GPU image."""
import math

import numpy as np
import pytest
import torch

from black_simulation_gb300 import bhk

pytestmark = pytest.mark.gpu


def _view(g, i):
    a, inc, hw, size = g["views"][i]
    return bhk.eht_view(a=a, inclination=math.radians(inc), half_width=hw, size=int(size), mass_solar=float(g["mass"]))


def _flow(g, i):
    f = g["flow"].copy()
    if i == 0:
        f[0] = g["n0_calibrated"]
    return bhk.eht_flow(n0=f[0], T0=f[1], beta=f[2], keplerian=f[3], height=f[4], sin_theta_b=f[5])


def _edge(shadow):
    """Pixels next to a change of the shadow mask (their rays skim the photon ring)."""
    s = shadow.astype(bool)
    e = np.zeros_like(s)
    e[:-1] |= s[:-1] != s[1:]
    e[1:] |= s[:-1] != s[1:]
    e[:, :-1] |= s[:, :-1] != s[:, 1:]
    e[:, 1:] |= s[:, :-1] != s[:, 1:]
    return e


@pytest.mark.parametrize("i", [0, 1, 2])
def test_image_matches_reference_render(cuda, golden, i):
    g = golden("eht_ref.npz")
    v = _view(g, i)
    inten, shadow, steps = bhk.eht_render(v, _flow(g, i))
    torch.cuda.synchronize()
    inten, shadow = inten.cpu().numpy(), shadow.cpu().numpy()
    want_i = g[f"intensity_{i}"].reshape(v.size, v.size)
    want_s = g[f"shadow_{i}"].reshape(v.size, v.size)
    assert (shadow != want_s).sum() <= 1
    keep = ~_edge(want_s) & (shadow == want_s)
    scale = want_i.max()
    assert np.abs(inten - want_i)[keep].max() <= 1e-6 * scale
    flux = bhk.eht_flux(inten, v.half_width, float(g["theta_g"]))
    assert abs(flux / g[f"flux_{i}"] - 1.0) < 1e-4
    assert int(steps.min()) > 0


def test_reference_calibration_checks_on_the_gpu(cuda, golden, oracle):
    """The reference's image test: calibrated to M87*'s 0.5 Jy, the approaching side brighter, the
    shadow with the critical curve's area."""
    g = golden("eht_ref.npz")
    theta_g = float(g["theta_g"])
    v = bhk.eht_view(a=0.9, inclination=math.radians(60.0), size=40, mass_solar=float(g["mass"]))
    n0 = bhk.eht_calibrate(v, bhk.eht_flow(), float(g["target_jy"]), theta_g)
    assert abs(n0 / float(g["n0_calibrated"]) - 1.0) < 1e-3
    v.size = 48
    inten, shadow, _ = bhk.eht_render(v, bhk.eht_flow(n0=n0))
    inten, shadow = inten.cpu().numpy(), shadow.cpu().numpy()
    assert abs(bhk.eht_flux(inten, v.half_width, theta_g) / 0.5 - 1.0) < 0.08
    left, right = inten[:, :24].sum(), inten[:, 24:].sum()
    assert left > 1.5 * right  # Bardeen's alpha: gas coming toward us is on the left
    pix = 2.0 * v.half_width / v.size
    ca, cb = oracle.critical_curve(0.9, math.radians(60.0), 400)
    area = abs(0.5 * np.sum(ca * np.roll(cb, -1) - np.roll(ca, -1) * cb))
    assert abs(shadow.sum() * pix * pix / area - 1.0) < 0.05


def test_shadow_only_mode_and_bad_views(cuda):
    v = bhk.eht_view(a=0.0, inclination=math.radians(40.0), half_width=8.0, size=64)
    inten, shadow, _ = bhk.eht_render(v, bhk.eht_flow(), with_light=False)
    assert float(inten.abs().max()) == 0.0
    # a = 0: the shadow is the disk of radius sqrt(27) M
    pix = 2.0 * 8.0 / 64
    assert abs(float(shadow.sum()) * pix * pix / (math.pi * 27.0) - 1.0) < 0.03
    with pytest.raises(bhk.BhkError):
        bhk.eht_render(bhk.eht_view(a=1.0), bhk.eht_flow())  # extremal spin (|a| > 1 is a naked singularity)
    with pytest.raises(bhk.BhkError):
        bhk.eht_render(bhk.eht_view(size=0), bhk.eht_flow())
