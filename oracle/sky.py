"""Test infrastructure only (the oracle): float64 restatement of the reference's Hosek-Wilkie sky.

Imported by tests/ only. Follows:
* the Hosek-Wilkie 2013 model's radiance (ArHosekSkyModel_GetRadianceInternal and
  arhosekskymodel_radiance, restated in renderer/gpu_kernels/analytic_sky_kernels.cu:16-66):
  per-band model state = 11 x 9 configuration values, 11 radiances, 11 sky emission correction
  factors; the radiance at a wavelength interpolates the two neighbouring 40 nm channels;
* the solar disc (arhosekskymodel_sr_internal and _solar_radiance_internal2, restated in
  analytic_sky_kernels.cu:69-191): the model's piecewise-cubic direct solar radiance at the
  texel's elevation with limb darkening, from the model's coefficient tables;
* the sky texture (analytic_sky_kernels.cu:220-276, the solar disc optional): texel (x, y) ->
  polar angles (y from the zenith), the lower hemisphere mirrored, 16 bands weighted by the CIE
  1931 CMF integrals into XYZ, XYZ -> linear sRGB (common/basic_types.h:3000-3010), the HSV
  saturation push towards blue (:257-266 with basic_types.h:3114-3160), and the lower hemisphere
  blended into the "sea" colour (:268-274).
"""
from __future__ import annotations

import math

import numpy as np

BANDS = 16


class Angles:
    """View angles of a batch of texels with the trigonometric terms the radiance formula reuses."""

    def __init__(self, theta, gamma):
        self.theta = np.asarray(theta, dtype=np.float64)
        self.gamma = np.asarray(gamma, dtype=np.float64)
        self.cos_t = np.cos(self.theta)
        self.cos_g = np.cos(self.gamma)
        self.cos_g2 = self.cos_g ** 2
        self.zenith = np.sqrt(self.cos_t)
        self.inv_ct = 1.0 / (self.cos_t + 0.01)


def radiance_internal(cfg, theta, gamma, ang: "Angles | None" = None):
    """ArHosekSkyModel_GetRadianceInternal for one configuration (9 values)."""
    a = ang if ang is not None else Angles(theta, gamma)
    exp_m = np.exp(cfg[4] * a.gamma)
    ray_m = a.cos_g2
    mie_m = (1.0 + a.cos_g2) / (1.0 + cfg[8] ** 2 - 2.0 * cfg[8] * a.cos_g) ** 1.5
    return (1.0 + cfg[0] * np.exp(cfg[1] * a.inv_ct)) * (
        cfg[2] + cfg[3] * exp_m + cfg[5] * ray_m + cfg[6] * mie_m + cfg[7] * a.zenith)


def unpack_state(state: np.ndarray) -> dict:
    """One band's 122 floats: configs[11][9], radiances[11], emission correction[11], solar radius."""
    s = np.asarray(state, dtype=np.float64)
    return {"configs": s[:99].reshape(11, 9), "radiances": s[99:110], "ecf": s[110:121], "solar_radius": s[121]}


def sky_radiance(state: dict, theta, gamma, wavelength: float, ang: "Angles | None" = None):
    """arhosekskymodel_radiance: the sky (no solar disc) at one wavelength in nm."""
    low = int((wavelength - 320.0) / 40.0)
    if low < 0 or low >= 11:
        return np.zeros_like(np.asarray(theta, dtype=np.float64))
    a = ang if ang is not None else Angles(theta, gamma)
    interp = math.fmod((wavelength - 320.0) / 40.0, 1.0)
    val_low = radiance_internal(state["configs"][low], theta, gamma, a) * state["radiances"][low] * state["ecf"][low]
    if interp < 1e-6:
        return val_low
    result = (1.0 - interp) * val_low
    if low + 1 < 11:
        result = result + interp * radiance_internal(state["configs"][low + 1], theta, gamma, a) * \
            state["radiances"][low + 1] * state["ecf"][low + 1]
    return result


def sr_internal(solar: np.ndarray, turbidity_index: int, channel: int, elevation):
    """arhosekskymodel_sr_internal (analytic_sky_kernels.cu:69-97): the direct solar radiance of one
    channel and integer turbidity, a cubic in the elevation on 45 pieces spaced cubically in
    elevation. `solar` = the model's solar tables (11 x 1800)."""
    pieces, order = 45, 4
    e = np.asarray(elevation, dtype=np.float64)
    pos = np.minimum(np.floor(np.power(2.0 * e / math.pi, 1.0 / 3.0) * pieces).astype(np.int64), 44)
    break_x = np.power(pos / pieces, 3.0) * (math.pi * 0.5)
    x = e - break_x
    base = order * pieces * turbidity_index + order * (pos + 1) - 1
    res = np.zeros_like(e)
    x_exp = np.ones_like(e)
    for i in range(order):
        res = res + x_exp * solar[channel][base - i]
        x_exp = x_exp * x
    return res


def solar_direct(tables: dict, turbidity: float, wavelength: float, elevation, gamma, solar_radius: float):
    """arhosekskymodel_solar_radiance_internal2 (analytic_sky_kernels.cu:99-184): the solar
    radiance interpolated between turbidities and channels, times the limb-darkening polynomial."""
    turb_low = int(turbidity) - 1
    turb_frac = turbidity - (turb_low + 1)
    if turb_low == 9:
        turb_low, turb_frac = 8, 1.0
    wl_low = int((wavelength - 320.0) / 40.0)
    wl_frac = math.fmod(wavelength, 40.0) / 40.0
    if wl_low == 10:
        wl_low, wl_frac = 9, 1.0
    sol = tables["solar"]
    direct = (1.0 - turb_frac) * ((1.0 - wl_frac) * sr_internal(sol, turb_low, wl_low, elevation) +
                                  wl_frac * sr_internal(sol, turb_low, wl_low + 1, elevation)) + \
        turb_frac * ((1.0 - wl_frac) * sr_internal(sol, turb_low + 1, wl_low, elevation) +
                     wl_frac * sr_internal(sol, turb_low + 1, wl_low + 1, elevation))
    ld = (1.0 - wl_frac) * tables["limb"][wl_low] + wl_frac * tables["limb"][wl_low + 1]
    sol_rad_sin = math.sin(solar_radius)
    ar2 = 1.0 / (sol_rad_sin * sol_rad_sin)
    sc2 = np.maximum(1.0 - ar2 * np.sin(gamma) ** 2, 0.0)
    c = np.sqrt(sc2)
    darkening = ld[0] + ld[1] * c + ld[2] * c ** 2 + ld[3] * c ** 3 + ld[4] * c ** 4 + ld[5] * c ** 5
    return direct * darkening


def _rgb_to_hsv(r, g, b):
    mn = np.minimum(np.minimum(r, g), b)
    mx = np.maximum(np.maximum(r, g), b)
    delta = mx - mn
    grey = (delta < 1e-5) | (mx == 0.0)
    safe = np.where(grey, 1.0, delta)
    h = np.where(r >= mx, (g - b) / safe, np.where(g >= mx, 2.0 + (b - r) / safe, 4.0 + (r - g) / safe))
    h = np.fmod(h / 6.0 + 1.0, 1.0)
    s = np.where(grey, 0.0, delta / np.where(mx == 0.0, 1.0, mx))
    return np.where(grey, 0.0, h), s, mx


def _hsv_to_rgb(h, s, v):
    h = h - np.floor(h)
    hi = np.floor(h * 6).astype(np.int64)
    f = h * 6 - hi
    m, n, k = v * (1 - s), v * (1 - s * f), v * (1 - s * (1 - f))
    table = [(v, k, m), (n, v, m), (m, v, k), (m, n, v), (k, m, v), (v, m, n)]
    out = [np.zeros_like(h) for _ in range(3)]
    for i, (a, b, c) in enumerate(table):
        sel = hi == i
        for ch, val in enumerate((a, b, c)):
            out[ch] = np.where(sel, val, out[ch])
    grey = s == 0
    return [np.where(grey, v, o) for o in out]


def sky_texture(width: int, height: int, states: np.ndarray, cmf: np.ndarray, sun_dir, disc: dict | None = None,
                window: tuple | None = None, cos_gamma_ulps: int | None = None) -> np.ndarray:
    """The sky texture: (height, width, 3) float64, without the solar disc unless `disc` =
    {"tables": the model's tables, "turbidity": t} is given (texels within the solar radius of the
    sun in the upper hemisphere then add the limb-darkened direct radiance, :238-239). `window` =
    (y0, y1, x0, x1) evaluates only those rows and columns of the texture. With `cos_gamma_ulps`
    = k the cosine of the view-sun angle is rounded to float32 and moved by k float32 steps before
    the arccos: the renderer takes that angle as acos of a float32 dot product
    (analytic_sky_kernels.cu:237), and within the disc (1 - cos < 1e-5) a float32 cosine takes
    only a few dozen values, so its rounding moves the limb-darkened radiance by percents; a test
    brackets the float32 result between evaluations at neighbouring cosines."""
    bands = [unpack_state(states[b]) for b in range(BANDS)]
    cmf = np.asarray(cmf, dtype=np.float64)
    xs, ys, zs, centers, integral = cmf[:16], cmf[16:32], cmf[32:48], cmf[48:64], cmf[64]
    y0, y1, x0, x1 = window if window is not None else (0, height, 0, width)
    yy, xx = np.meshgrid(np.arange(y0, y1), np.arange(x0, x1), indexing="ij")
    theta = math.pi * (yy + 0.5) / height
    phi = 2 * math.pi * (xx + 0.5) / width
    lower = theta >= 0.5 * math.pi
    m_theta = np.where(lower, math.pi - theta, theta)
    view = np.stack([-np.sin(phi) * np.sin(m_theta), np.cos(m_theta), np.cos(phi) * np.sin(m_theta)], axis=-1)
    sd = np.asarray(sun_dir, dtype=np.float64)
    cos_gamma = view @ sd
    if cos_gamma_ulps is not None:
        c32 = np.clip(cos_gamma, -1.0, 1.0).astype(np.float32)
        step = np.float32(np.inf) if cos_gamma_ulps > 0 else np.float32(-np.inf)
        for _ in range(abs(int(cos_gamma_ulps))):
            c32 = np.nextafter(c32, step)
        cos_gamma = c32.astype(np.float64)
    gamma = np.arccos(np.clip(cos_gamma, -1.0, 1.0))
    X = np.zeros_like(theta)
    Y = np.zeros_like(theta)
    Z = np.zeros_like(theta)
    ang = Angles(m_theta, gamma)
    for b in range(BANDS):
        wl = min(max(float(centers[b]), 320.0), 720.0)
        v = sky_radiance(bands[b], m_theta, gamma, wl, ang)
        if disc is not None:
            in_disc = (gamma < bands[b]["solar_radius"]) & ~lower
            if in_disc.any():
                v = v.copy()
                v[in_disc] += solar_direct(disc["tables"], disc["turbidity"], wl, 0.5 * math.pi - m_theta[in_disc],
                                           gamma[in_disc], float(bands[b]["solar_radius"]))
        X += xs[b] * v
        Y += ys[b] * v
        Z += zs[b] * v
    X, Y, Z = X / integral, Y / integral, Z / integral
    r = 3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z
    g = -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z
    bl = 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z
    max_v = np.maximum(r, np.maximum(g, bl))
    h, s, _ = _rgb_to_hsv(r / max_v, g / max_v, bl / max_v)
    diff_angle = 2 * math.pi * np.fmod(h - 2.0 / 3 + 1.0, 1.0)
    t_s = s * (0.5 * (1 + np.cos(diff_angle)))
    s = (1 - t_s) * s + t_s
    r, g, bl = (max_v * c for c in _hsv_to_rgb(h, s, np.ones_like(h)))
    sea_b = (1 - sd[1]) * 0.01 + sd[1] * 0.1
    sea = 0.5 * np.array([0.01, 0.01, sea_b])
    t = np.where(lower, np.cos(m_theta) ** (1 / 5.0), 0.0)
    out = np.stack([r, g, bl], axis=-1)
    return np.where(lower[..., None], (1 - t)[..., None] * out + t[..., None] * sea, out)
