"""Seeded synthetic observations with the shapes of the benchmark workloads.

No public dataset is involved: a 27-antenna Y array (three arms at 0, 120 and
240 degrees, nine antennas per arm with radii 40 m * (R / 40 m)^(k/8)),
Earth-rotation uvw at declination +40 degrees seen from latitude 34.0784
degrees, and visibilities of seeded point sources (and Gaussians) with the
reference's sign convention V = sum S exp(-2 pi i (u l + v m + w (n - 1)))
(point_source_visibilities_with_mode, lib.rs:86969-87020: l grows with x,
m falls with y), plus complex Gaussian noise.  Rows are time-major
(all baselines of a dump, then the next dump), as a MeasurementSet stores
them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

C_LIGHT = 299_792_458.0
SIDEREAL_DAY_S = 86_164.0905
LATITUDE_DEG = 34.0784


def antenna_enu(max_radius_m: float) -> np.ndarray:
    k = np.arange(9)
    radii = 40.0 * (max_radius_m / 40.0) ** (k / 8.0)
    out = []
    for az in (0.0, 120.0, 240.0):
        a = math.radians(az)
        out += [(r * math.sin(a), r * math.cos(a), 0.0) for r in radii]
    return np.array(out)


def baselines_xyz(max_radius_m: float, latitude_deg: float = LATITUDE_DEG) -> np.ndarray:
    e, n, u = antenna_enu(max_radius_m).T
    lat = math.radians(latitude_deg)
    xyz = np.stack([-n * math.sin(lat) + u * math.cos(lat), e, n * math.cos(lat) + u * math.sin(lat)], 1)
    i, j = np.triu_indices(len(xyz), 1)
    return xyz[j] - xyz[i]


def uvw_metres(max_radius_m: float, hours: float, dump_s: float, dec_deg: float = 40.0):
    """(u, v, w) in metres, shape [dumps * baselines], time-major."""
    B = baselines_xyz(max_radius_m)
    nd = int(round(hours * 3600.0 / dump_s))
    H = (-hours / 2.0 * 3600.0 + (np.arange(nd) + 0.5) * dump_s) * (2.0 * math.pi / SIDEREAL_DAY_S)
    d = math.radians(dec_deg)
    sH, cH = np.sin(H)[:, None], np.cos(H)[:, None]
    bx, by, bz = B[:, 0][None], B[:, 1][None], B[:, 2][None]
    u = sH * bx + cH * by
    v = -math.sin(d) * cH * bx + math.sin(d) * sH * by + math.cos(d) * bz
    w = math.cos(d) * cH * bx - math.cos(d) * sH * by + math.sin(d) * bz
    return u.ravel(), v.ravel(), w.ravel()


@dataclass
class Sky:
    x_pix: np.ndarray
    y_pix: np.ndarray
    flux: np.ndarray
    fwhm_pix: np.ndarray = field(default_factory=lambda: np.zeros(0))

    def lmn(self, nx: int, ny: int, cell: float):
        l = (self.x_pix - nx / 2.0) * cell
        m = (ny / 2.0 - self.y_pix) * cell
        return l, m, np.sqrt(1.0 - l * l - m * m) - 1.0


def point_sky(rng, n: int, nx: int, ny: int, fmin: float, fmax: float) -> Sky:
    """Fluxes log-uniform in [fmin, fmax]; positions uniform in the inner half."""
    x = rng.uniform(nx * 0.25, nx * 0.75, n)
    y = rng.uniform(ny * 0.25, ny * 0.75, n)
    flux = np.exp(rng.uniform(math.log(fmin), math.log(fmax), n))
    return Sky(x, y, flux)


def model_image(sky: Sky, nx: int, ny: int) -> np.ndarray:
    img = np.zeros((nx, ny), np.float32)
    xi = np.clip(np.round(sky.x_pix).astype(int), 0, nx - 1)
    yi = np.clip(np.round(sky.y_pix).astype(int), 0, ny - 1)
    np.add.at(img, (xi, yi), sky.flux.astype(np.float32))
    return img


def visibilities(u, v, w, sky: Sky, nx: int, ny: int, cell: float, noise_sigma: float,
                 rng, w_term: bool = True, chunk: int = 1 << 20) -> np.ndarray:
    """Direct DFT of the sky (FP64 phase), complex64, plus complex noise."""
    l, m, nm1 = sky.lmn(nx, ny, cell)
    if not w_term:
        nm1 = np.zeros_like(nm1)
    out = np.empty(len(u), np.complex64)
    for s in range(0, len(u), chunk):
        e = min(len(u), s + chunk)
        ph = -2.0 * math.pi * (np.outer(u[s:e], l) + np.outer(v[s:e], m) + np.outer(w[s:e], nm1))
        out[s:e] = (np.cos(ph) @ sky.flux + 1j * (np.sin(ph) @ sky.flux)).astype(np.complex64)
    if noise_sigma > 0:
        out += (rng.normal(0, noise_sigma, len(u)) + 1j * rng.normal(0, noise_sigma, len(u))).astype(np.complex64)
    return out


def visibilities_torch(u, v, w, sky: Sky, nx: int, ny: int, cell: float, noise_sigma: float,
                       seed: int, device="cuda", chunk: int = 1 << 19):
    """The same DFT on the GPU with torch (float64 phase), for large observations."""
    import torch
    l, m, nm1 = sky.lmn(nx, ny, cell)
    L = torch.tensor(np.stack([l, m, nm1], 0), dtype=torch.float64, device=device)
    F = torch.tensor(sky.flux, dtype=torch.float64, device=device)
    U = torch.stack([torch.as_tensor(u, device=device), torch.as_tensor(v, device=device),
                     torch.as_tensor(w, device=device)], 1).to(torch.float64)
    out = torch.empty(len(u), dtype=torch.complex64, device=device)
    for s in range(0, len(u), chunk):
        ph = (-2.0 * math.pi) * (U[s:s + chunk] @ L)
        re = torch.cos(ph) @ F
        im = torch.sin(ph) @ F
        out[s:s + chunk] = torch.complex(re, im).to(torch.complex64)
    if noise_sigma > 0:
        g = torch.Generator(device=device)
        g.manual_seed(seed)
        nr = torch.randn(len(u), generator=g, device=device, dtype=torch.float32) * noise_sigma
        ni = torch.randn(len(u), generator=g, device=device, dtype=torch.float32) * noise_sigma
        out += torch.complex(nr, ni)
    return out


@dataclass
class Observation:
    name: str
    nx: int
    ny: int
    cell: float
    freq_hz: float
    u: np.ndarray   # wavelengths
    v: np.ndarray
    w: np.ndarray
    sky: Sky
    seed: int
    vis: object = None

    @property
    def rows(self):
        return len(self.u)


def observation(max_radius_m: float, hours: float, dump_s: float, freq_hz: float, image: int,
                n_sources: int, fmin: float, fmax: float, seed: int, name: str) -> Observation:
    """uvw in wavelengths, cell = 1/3 of the synthesised beam (lambda / B_max)."""
    rng = np.random.default_rng(seed)
    um, vm, wm = uvw_metres(max_radius_m, hours, dump_s)
    lam = C_LIGHT / freq_hz
    u, v, w = um / lam, vm / lam, wm / lam
    cell = 1.0 / (3.0 * float(np.sqrt(u * u + v * v).max()))
    sky = point_sky(rng, n_sources, image, image, fmin, fmax)
    return Observation(name, image, image, cell, freq_hz, u, v, w, sky, seed)


def pswf_512_observation(seed: int = 1) -> Observation:
    """27 antennas out to 1 km, 1 h of 10 s dumps at 1.4 GHz (126,360 rows),
    512 x 512 image, 20 points 0.01-1 Jy, noise 0.01 Jy."""
    obs = observation(1000.0, 1.0, 10.0, 1.4e9, 512, 20, 0.01, 1.0, seed, "pswf_512")
    rng = np.random.default_rng(seed + 1000)
    obs.vis = visibilities(obs.u, obs.v, np.zeros_like(obs.w), obs.sky, 512, 512, obs.cell,
                           0.01, rng, w_term=False)
    return obs


def wproj_4096_observation(seed: int = 2) -> Observation:
    """27 antennas out to 21 km, 8 h of 2 s dumps at 1.4 GHz (5,054,400 rows),
    4096 x 4096 image, 200 points 1 mJy-1 Jy; visibilities not yet made."""
    return observation(21000.0, 8.0, 2.0, 1.4e9, 4096, 200, 1e-3, 1.0, seed, "wproj_4096")


# ----------------------------------------------------------------------------
# spectral cube
# ----------------------------------------------------------------------------
@dataclass
class CubeObservation:
    nx: int
    cell: float
    freqs_hz: np.ndarray      # [C]
    u_m: np.ndarray           # [R] metres, time-major rows
    v_m: np.ndarray
    sky: Sky
    flag_fraction: np.ndarray  # [C]
    seed: int

    @property
    def channels(self):
        return len(self.freqs_hz)

    @property
    def rows(self):
        return len(self.u_m)

    @property
    def lambda_scale(self):
        return self.freqs_hz / C_LIGHT


def cube_observation(channels: int = 256, nx: int = 1024, hours: float = 10.0,
                     dump_s: float = 10.0, max_radius_m: float = 1000.0, f_lo: float = 1.0e9,
                     f_hi: float = 2.0e9, n_sources: int = 20, max_flag: float = 0.6,
                     seed: int = 4) -> CubeObservation:
    """Channels linear in [f_lo, f_hi]; cell = 1/3 of the synthesised beam at
    f_hi; per-channel flag fraction uniform in [0, max_flag]."""
    um, vm, _ = uvw_metres(max_radius_m, hours, dump_s)
    freqs = np.linspace(f_lo, f_hi, channels)
    ls_hi = f_hi / C_LIGHT
    cell = 1.0 / (3.0 * float(np.sqrt(um * um + vm * vm).max()) * ls_hi)
    rng = np.random.default_rng(seed)
    frac = rng.uniform(0.0, max_flag, channels)
    sky = point_sky(rng, n_sources, nx, nx, 0.01, 1.0)
    return CubeObservation(nx, cell, freqs, um, vm, sky, frac, seed)


def cube_flags(obs: CubeObservation):
    """[C][R] bool, per-sample Bernoulli with the channel's flag fraction."""
    rng = np.random.default_rng(obs.seed + 7)
    return rng.random((obs.channels, obs.rows)) < obs.flag_fraction[:, None]


def cube_visibilities(obs: CubeObservation) -> np.ndarray:
    """[C][R] complex64 point-source visibilities (FP64 DFT, no w-term)."""
    l, m, _ = obs.sky.lmn(obs.nx, obs.nx, obs.cell)
    out = np.empty((obs.channels, obs.rows), np.complex64)
    for c, ls in enumerate(obs.lambda_scale):
        ph = -2.0 * math.pi * (np.outer(obs.u_m * ls, l) + np.outer(obs.v_m * ls, m))
        out[c] = (np.cos(ph) @ obs.sky.flux + 1j * (np.sin(ph) @ obs.sky.flux))
    return out


def cube_device_inputs(obs: CubeObservation, device="cuda"):
    """Flags and visibilities generated on the GPU for the full-size cube
    (float32 phases: the benchmark only needs their shape and spread)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(obs.seed + 7)
    frac = torch.as_tensor(obs.flag_fraction, dtype=torch.float32, device=device)
    flags = torch.empty((obs.channels, obs.rows), dtype=torch.uint8, device=device)
    vis = torch.empty((obs.channels, obs.rows), dtype=torch.complex64, device=device)
    l, m, _ = obs.sky.lmn(obs.nx, obs.nx, obs.cell)
    L = torch.tensor(np.stack([l, m], 0), dtype=torch.float32, device=device)
    Fx = torch.tensor(obs.sky.flux, dtype=torch.float32, device=device)
    U = torch.stack([torch.as_tensor(obs.u_m, device=device),
                     torch.as_tensor(obs.v_m, device=device)], 1).to(torch.float32)
    for c in range(obs.channels):
        flags[c] = (torch.rand(obs.rows, generator=g, device=device) < frac[c]).to(torch.uint8)
        ph = (-2.0 * math.pi * float(obs.lambda_scale[c])) * (U @ L)
        vis[c] = torch.complex(torch.cos(ph) @ Fx, torch.sin(ph) @ Fx)
    return flags, vis


def gaussian_model(rng, n: int, nx: int, ny: int, fmin: float, fmax: float,
                   fwhm_min: float = 1.0, fwhm_max: float = 5.0) -> np.ndarray:
    """float32 [nx][ny] image of n circular Gaussians (integrated flux
    log-uniform in [fmin, fmax], FWHM uniform in [fwhm_min, fwhm_max] pixels,
    centres uniform in the inner half of the field)."""
    img = np.zeros((nx, ny), np.float64)
    flux = np.exp(rng.uniform(np.log(fmin), np.log(fmax), n))
    fwhm = rng.uniform(fwhm_min, fwhm_max, n)
    cx = rng.uniform(nx / 4, 3 * nx / 4, n)
    cy = rng.uniform(ny / 4, 3 * ny / 4, n)
    for s, f, x0, y0 in zip(flux, fwhm, cx, cy):
        sig = f / (2.0 * math.sqrt(2.0 * math.log(2.0)))
        h = int(math.ceil(5 * sig)) + 1
        xs = np.arange(max(int(x0) - h, 0), min(int(x0) + h + 1, nx))
        ys = np.arange(max(int(y0) - h, 0), min(int(y0) + h + 1, ny))
        g = np.exp(-((xs[:, None] - x0) ** 2 + (ys[None, :] - y0) ** 2) / (2 * sig * sig))
        img[np.ix_(xs, ys)] += s * g / g.sum()
    return img.astype(np.float32)


def pair_2048_observation(seed: int = 3) -> Observation:
    """Differentiable-imaging workload: 27 antennas to 5 km, 8 h of 5 s dumps
    at 1.4 GHz (2,021,760 rows), 2048 x 2048 image; the sky is a Gaussian
    model image (gaussian_model, 50 components 0.01-1 Jy, FWHM 1-5 px)."""
    return observation(5000.0, 8.0, 5.0, 1.4e9, 2048, 0, 0.01, 1.0, seed, "pair_2048")


def major_minor_2048_observation(seed: int = 5):
    """Major/minor-loop workload: 27 antennas to 21 km, 8 h of 4 s dumps
    (2,527,200 rows) at 4 channels over 1.3-1.5 GHz gridded together (MFS:
    10,108,800 visibilities), 2048 x 2048 image with the cell 1/3 of the beam
    at 1.5 GHz, sky of 300 points (1 mJy-1 Jy, on pixel centres) and 5
    Gaussians (0.1-0.5 Jy, FWHM 3-10 px).  Returns (observation with u, v, w
    in wavelengths for all channels, model image)."""
    um, vm, wm = uvw_metres(21000.0, 8.0, 4.0)
    freqs = np.linspace(1.3e9, 1.5e9, 4)
    ls = freqs / C_LIGHT
    u = np.concatenate([um * s for s in ls])
    v = np.concatenate([vm * s for s in ls])
    w = np.concatenate([wm * s for s in ls])
    nx = 2048
    cell = 1.0 / (3.0 * float(np.sqrt(um * um + vm * vm).max()) * ls[-1])
    rng = np.random.default_rng(seed)
    sky = point_sky(rng, 300, nx, nx, 1e-3, 1.0)
    sky.x_pix, sky.y_pix = np.round(sky.x_pix), np.round(sky.y_pix)
    model = model_image(sky, nx, nx) + gaussian_model(rng, 5, nx, nx, 0.1, 0.5, 3.0, 10.0)
    obs = Observation("major_minor_2048", nx, nx, cell, float(freqs.mean()), u, v, w, sky, seed)
    return obs, model
