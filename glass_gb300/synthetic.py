"""Seeded synthetic light stacks with the shapes and noise model of the
benchmark configurations (uint16 raw lights + bias/dark/flat frames, with the
truth registration matrices).

The reference's own generator (src/glass/synthetic/generator.py) writes a
different model (float32, integer shifts only); these stacks follow the
benchmark descriptions instead: Gaussian/Moffat stars with log-uniform peak
flux, per-frame sky, Poisson shot noise plus Gaussian read noise, a pedestal,
quadratic vignetting flats, hot pixels, cosmic-ray streaks, satellite trails
and thin-cloud frames, under seeded random similarity transforms.

Truth convention: a star at reference-frame position r appears in frame i at
m = A_i r + t_i.  `truth_matrices[i]` maps frame-i (moving) pixel coordinates
to reference coordinates, i.e. the matrix registration should recover.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class StackConfig:
    frames: int
    height: int
    width: int
    stars: int
    fwhm: tuple[float, float] = (2.5, 2.5)
    moffat_fraction: float = 0.0
    peak_flux: tuple[float, float] = (500.0, 20000.0)
    sky: tuple[float, float] = (1000.0, 1000.0)
    sky_gradient: float = 0.05
    read_noise: float = 5.0
    pedestal: float = 500.0
    dark_current: float = 0.02  # ADU / s
    exposure_s: float = 300.0
    hot_pixel_fraction: float = 0.0
    cosmic_ray_density: float = 0.0
    satellite_fraction: float = 0.0
    cloud_frames: int = 0
    max_shift: float = 5.0
    max_rotation_deg: float = 0.0
    integer_shifts: bool = False
    calibration_frames: int = 4
    flat_level: float = 30000.0
    vignetting: tuple[float, float] = (0.9, 1.0)
    seed: int = 0


CONFIGS = {
    # 8 uint16 lights 128x128, ~30 stars FWHM 2.5, sky 1000, pedestal 500,
    # integer shifts within +/-5 px, 4 calibration frames of each kind.
    "c1": StackConfig(frames=8, height=128, width=128, stars=30, sky=(1000.0, 1000.0), max_shift=5.0,
                      integer_shifts=True, calibration_frames=4, seed=1),
    # 32 uint16 lights 2048x2048, ~2000 stars FWHM 2-4 (Gaussian/Moffat),
    # sky 800-1200, hot pixels 0.01 %, cosmic rays 1e-4, satellite in 10 %,
    # +/-20 px and +/-0.5 deg, 10 calibration frames of each kind.
    "c2": StackConfig(frames=32, height=2048, width=2048, stars=2000, fwhm=(2.0, 4.0), moffat_fraction=0.5,
                      sky=(800.0, 1200.0), hot_pixel_fraction=1e-4, cosmic_ray_density=1e-4,
                      satellite_fraction=0.1, max_shift=20.0, max_rotation_deg=0.5, calibration_frames=10, seed=2),
    # 200 uint16 lights 9600x6422 (W x H), ~20000 stars FWHM 2-5, sky drift
    # +/-15 %, 7 thin-cloud frames, cosmic rays 1e-4, +/-40 px and +/-0.3 deg,
    # 20 calibration frames of each kind.
    "c5": StackConfig(frames=200, height=6422, width=9600, stars=20000, fwhm=(2.0, 5.0), moffat_fraction=0.5,
                      sky=(850.0, 1150.0), hot_pixel_fraction=1e-4, cosmic_ray_density=1e-4, cloud_frames=7,
                      max_shift=40.0, max_rotation_deg=0.3, calibration_frames=20, seed=5),
}


@dataclass
class SyntheticStack:
    config: StackConfig
    lights: np.ndarray  # (N, H, W) uint16
    bias_frames: np.ndarray  # (C, H, W) uint16
    dark_frames: np.ndarray
    flat_frames: np.ndarray
    truth_matrices: np.ndarray  # (N, 3, 3) float64, moving -> reference
    star_xy: np.ndarray  # (S, 2) reference-frame positions
    star_peak: np.ndarray  # (S,)
    cloud: np.ndarray  # (N,) bool
    meta: dict = field(default_factory=dict)


def _similarity(theta: float, dx: float, dy: float) -> np.ndarray:
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c, -s, dx], [s, c, dy], [0.0, 0.0, 1.0]], dtype=np.float64)


def _render_stars(image: np.ndarray, xs: np.ndarray, ys: np.ndarray, peaks: np.ndarray, sigmas: np.ndarray,
                  moffat: np.ndarray, radius: int) -> None:
    """Adds PSFs to `image` in place (vectorised over stars, window radius)."""
    h, w = image.shape
    offs = np.arange(-radius, radius + 1)
    inside = (xs > -radius) & (xs < w + radius) & (ys > -radius) & (ys < h + radius)
    xs, ys, peaks, sigmas, moffat = xs[inside], ys[inside], peaks[inside], sigmas[inside], moffat[inside]
    if xs.size == 0:
        return
    cx = np.floor(xs).astype(np.int64)
    cy = np.floor(ys).astype(np.int64)
    px = cx[:, None] + offs[None, :]  # (S, K)
    py = cy[:, None] + offs[None, :]
    dx = px - xs[:, None]
    dy = py - ys[:, None]
    r2 = dx[:, None, :] ** 2 + dy[:, :, None] ** 2  # (S, K, K) [y, x]
    s2 = (sigmas**2)[:, None, None]
    gauss = np.exp(-0.5 * r2 / s2)
    beta = 3.0
    alpha2 = (s2 * 2.0 * np.sqrt(2.0)) ** 1  # moffat core ~ same FWHM scale
    moff = (1.0 + r2 / alpha2) ** (-beta)
    prof = np.where(moffat[:, None, None], moff, gauss) * peaks[:, None, None]
    yy = np.broadcast_to(py[:, :, None], prof.shape)
    xx = np.broadcast_to(px[:, None, :], prof.shape)
    ok = (yy >= 0) & (yy < h) & (xx >= 0) & (xx < w)
    np.add.at(image, (yy[ok], xx[ok]), prof[ok])


def generate(config: StackConfig | str, frames: int | None = None) -> SyntheticStack:
    """Generates one synthetic stack (deterministic for a given config)."""
    cfg = CONFIGS[config] if isinstance(config, str) else config
    n = int(frames or cfg.frames)
    rng = np.random.default_rng(cfg.seed)
    h, w = cfg.height, cfg.width
    margin = cfg.max_shift + np.deg2rad(cfg.max_rotation_deg) * max(h, w) + 8
    star_xy = np.column_stack([
        rng.uniform(-margin, w + margin, cfg.stars),
        rng.uniform(-margin, h + margin, cfg.stars),
    ])
    lo, hi = cfg.peak_flux
    star_peak = np.exp(rng.uniform(np.log(lo), np.log(hi), cfg.stars))
    fwhm = rng.uniform(cfg.fwhm[0], cfg.fwhm[1], cfg.stars)
    sigma = fwhm / 2.3548200450309493
    moffat = rng.random(cfg.stars) < cfg.moffat_fraction
    radius = int(np.ceil(4.0 * sigma.max())) + 1

    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    rr = ((xx - w / 2) / (w / 2)) ** 2 + ((yy - h / 2) / (h / 2)) ** 2
    vmin, vmax = cfg.vignetting
    vignette = (vmax - (vmax - vmin) * np.clip(rr / 2.0, 0.0, 1.0)).astype(np.float32)
    dark_rate = np.full((h, w), cfg.dark_current, dtype=np.float32)
    n_hot = int(round(cfg.hot_pixel_fraction * h * w))
    if n_hot:
        hot = rng.choice(h * w, size=n_hot, replace=False)
        dark_rate.reshape(-1)[hot] = rng.uniform(5.0, 50.0, n_hot).astype(np.float32)

    def noisy(signal: np.ndarray) -> np.ndarray:
        out = rng.poisson(np.maximum(signal, 0.0)).astype(np.float32)
        out += cfg.pedestal + cfg.read_noise * rng.standard_normal((h, w)).astype(np.float32)
        return np.clip(np.rint(out), 0, 65535).astype(np.uint16)

    cal = cfg.calibration_frames
    bias_frames = np.stack([noisy(np.zeros((h, w), np.float32)) for _ in range(cal)])
    dark_frames = np.stack([noisy(dark_rate * cfg.exposure_s) for _ in range(cal)])
    flat_frames = np.stack([noisy(vignette * cfg.flat_level) for _ in range(cal)])

    cloud = np.zeros(n, dtype=bool)
    if cfg.cloud_frames and n > 1:
        # frame 0 is the registration reference: never a thin-cloud frame
        cloud[1 + rng.choice(n - 1, size=min(cfg.cloud_frames, n - 1), replace=False)] = True
    lights = np.empty((n, h, w), dtype=np.uint16)
    truth = np.empty((n, 3, 3), dtype=np.float64)
    for i in range(n):
        if i == 0:
            theta, dx, dy = 0.0, 0.0, 0.0
        elif cfg.integer_shifts:
            theta = 0.0
            dx, dy = (float(v) for v in rng.integers(-int(cfg.max_shift), int(cfg.max_shift) + 1, 2))
        else:
            theta = np.deg2rad(rng.uniform(-cfg.max_rotation_deg, cfg.max_rotation_deg))
            dx, dy = (float(v) for v in rng.uniform(-cfg.max_shift, cfg.max_shift, 2))
        forward = _similarity(theta, dx, dy)  # reference -> frame
        truth[i] = np.linalg.inv(forward)
        pos = star_xy @ forward[:2, :2].T + forward[:2, 2]
        sky = rng.uniform(*cfg.sky)
        flux_scale = 0.5 if cloud[i] else 1.0
        if cloud[i]:
            sky *= 2.0
        signal = np.full((h, w), sky, dtype=np.float32)
        if cfg.sky_gradient:
            gx, gy = rng.uniform(-1, 1, 2) * cfg.sky_gradient * sky
            signal += (gx * (xx / w - 0.5) + gy * (yy / h - 0.5)).astype(np.float32)
        _render_stars(signal, pos[:, 0], pos[:, 1], star_peak * flux_scale, sigma, moffat, radius)
        signal *= vignette
        signal += dark_rate * cfg.exposure_s
        frame = rng.poisson(np.maximum(signal, 0.0)).astype(np.float32)
        frame += cfg.pedestal + cfg.read_noise * rng.standard_normal((h, w)).astype(np.float32)
        if cfg.cosmic_ray_density:
            hits = rng.poisson(cfg.cosmic_ray_density * h * w)
            cy = rng.integers(0, h, hits)
            cx = rng.integers(0, w, hits)
            length = rng.integers(2, 7, hits)
            ang = rng.uniform(0, np.pi, hits)
            # 5k-60k ADU per hit pixel: as bright as the brightest stars, so
            # a brightness-ranked catalog needs a shape filter
            energy = rng.uniform(5000.0, 60000.0, hits).astype(np.float32)
            for step in range(6):
                on = step < length
                sy = np.clip(np.rint(cy + step * np.sin(ang)).astype(np.int64), 0, h - 1)
                sx = np.clip(np.rint(cx + step * np.cos(ang)).astype(np.int64), 0, w - 1)
                frame[sy[on], sx[on]] += energy[on]
        if cfg.satellite_fraction and rng.random() < cfg.satellite_fraction:
            y0, y1 = rng.uniform(0, h, 2)
            xs = np.arange(w)
            ys = np.rint(y0 + (y1 - y0) * xs / max(w - 1, 1)).astype(np.int64)
            for t in (-1, 0, 1):
                yt = np.clip(ys + t, 0, h - 1)
                frame[yt, xs] += 3000.0 if t == 0 else 1200.0
        lights[i] = np.clip(np.rint(frame), 0, 65535).astype(np.uint16)
    return SyntheticStack(cfg, lights, bias_frames, dark_frames, flat_frames, truth, star_xy, star_peak, cloud,
                          {"vignette_min": vmin, "vignette_max": vmax})


@dataclass
class DeviceStack:
    """A synthetic stack rendered on the GPU (the same model as generate()):
    `lights` is a (N, H, W) int16 CUDA tensor holding the uint16 raw frames
    bit for bit; the calibration frames are host uint16 arrays."""

    config: StackConfig
    lights: "object"  # torch.Tensor (N, H, W) int16 on the device
    bias_frames: np.ndarray
    dark_frames: np.ndarray
    flat_frames: np.ndarray
    truth_matrices: np.ndarray
    cloud: np.ndarray


def _u16_as_i16(torch, values):
    """Rounded float32 ADU -> int16 tensor with the uint16 bit pattern."""
    v = torch.clamp(torch.round(values), 0.0, 65535.0).to(torch.int32)
    return torch.where(v > 32767, v - 65536, v).to(torch.int16)


def generate_device(config: StackConfig | str, frames: int | None = None, cloud_slots: list[int] | None = None,
                    device: str = "cuda") -> DeviceStack:
    """Renders a stack of `config`'s model directly in device memory, one
    frame at a time (a 200 x 9600 x 6422 stack in seconds; the NumPy
    generator would take most of an hour).  Star positions, fluxes, PSFs,
    transforms and sky levels come from NumPy's seeded generator; the shot,
    read and cosmic-ray noise from a seeded torch CUDA generator.  Thin-cloud
    frames (50 % star flux, 2x sky) are exactly `cloud_slots` when given
    (frame 0, the registration reference, is never one), else
    `config.cloud_frames` frames drawn from 1..N-1."""
    import torch

    cfg = CONFIGS[config] if isinstance(config, str) else config
    n = int(frames or cfg.frames)
    rng = np.random.default_rng(cfg.seed)
    gen = torch.Generator(device=device)
    gen.manual_seed(cfg.seed)
    h, w = cfg.height, cfg.width
    margin = cfg.max_shift + np.deg2rad(cfg.max_rotation_deg) * max(h, w) + 8
    star_xy = np.column_stack([rng.uniform(-margin, w + margin, cfg.stars), rng.uniform(-margin, h + margin, cfg.stars)])
    lo, hi = cfg.peak_flux
    star_peak = np.exp(rng.uniform(np.log(lo), np.log(hi), cfg.stars))
    sigma = rng.uniform(cfg.fwhm[0], cfg.fwhm[1], cfg.stars) / 2.3548200450309493
    moffat = rng.random(cfg.stars) < cfg.moffat_fraction
    radius = int(np.ceil(4.0 * sigma.max())) + 1
    offs = torch.arange(-radius, radius + 1, device=device, dtype=torch.float32)
    t_sigma = torch.as_tensor(sigma, device=device, dtype=torch.float32)
    t_moffat = torch.as_tensor(moffat, device=device)

    yy = torch.arange(h, device=device, dtype=torch.float32)[:, None]
    xx = torch.arange(w, device=device, dtype=torch.float32)[None, :]
    rr = ((xx - w / 2) / (w / 2)) ** 2 + ((yy - h / 2) / (h / 2)) ** 2
    vmin, vmax = cfg.vignetting
    vignette = vmax - (vmax - vmin) * torch.clamp(rr / 2.0, 0.0, 1.0)
    del rr
    dark_rate = torch.full((h, w), cfg.dark_current, device=device, dtype=torch.float32)
    n_hot = int(round(cfg.hot_pixel_fraction * h * w))
    if n_hot:
        hot = rng.choice(h * w, size=n_hot, replace=False)
        dark_rate.view(-1)[torch.as_tensor(hot, device=device)] = torch.as_tensor(
            rng.uniform(5.0, 50.0, n_hot), device=device, dtype=torch.float32)

    def noisy(signal):
        out = torch.poisson(torch.clamp(signal, min=0.0), generator=gen)
        out += cfg.pedestal + cfg.read_noise * torch.randn((h, w), device=device, generator=gen)
        return _u16_as_i16(torch, out)

    def host_u16(t):
        return t.cpu().numpy().view(np.uint16)

    cal = cfg.calibration_frames
    zeros = torch.zeros((h, w), device=device)
    bias_frames = np.stack([host_u16(noisy(zeros)) for _ in range(cal)])
    dark_frames = np.stack([host_u16(noisy(dark_rate * cfg.exposure_s)) for _ in range(cal)])
    flat_frames = np.stack([host_u16(noisy(vignette * cfg.flat_level)) for _ in range(cal)])
    del zeros

    cloud = np.zeros(n, dtype=bool)
    if cloud_slots is not None:
        cloud[np.asarray(cloud_slots, dtype=np.int64)] = True
    elif cfg.cloud_frames and n > 1:
        cloud[1 + rng.choice(n - 1, size=min(cfg.cloud_frames, n - 1), replace=False)] = True
    if cloud[0]:
        raise ValueError("frame 0 is the registration reference and cannot be a thin-cloud frame")
    lights = torch.empty((n, h, w), device=device, dtype=torch.int16)
    truth = np.empty((n, 3, 3), dtype=np.float64)
    beta = 3.0
    for i in range(n):
        if i == 0:
            theta, dx, dy = 0.0, 0.0, 0.0
        elif cfg.integer_shifts:
            theta = 0.0
            dx, dy = (float(v) for v in rng.integers(-int(cfg.max_shift), int(cfg.max_shift) + 1, 2))
        else:
            theta = np.deg2rad(rng.uniform(-cfg.max_rotation_deg, cfg.max_rotation_deg))
            dx, dy = (float(v) for v in rng.uniform(-cfg.max_shift, cfg.max_shift, 2))
        forward = _similarity(theta, dx, dy)
        truth[i] = np.linalg.inv(forward)
        pos = star_xy @ forward[:2, :2].T + forward[:2, 2]
        sky = rng.uniform(*cfg.sky) * (2.0 if cloud[i] else 1.0)
        flux = star_peak * (0.5 if cloud[i] else 1.0)
        gx, gy = rng.uniform(-1, 1, 2) * cfg.sky_gradient * sky
        signal = sky + gx * (xx / w - 0.5) + gy * (yy / h - 0.5)
        # stars: one (2r+1)^2 stamp per star, accumulated into the frame
        px_c = torch.as_tensor(pos[:, 0], device=device)
        py_c = torch.as_tensor(pos[:, 1], device=device)
        inside = (px_c > -radius) & (px_c < w + radius) & (py_c > -radius) & (py_c < h + radius)
        cx = torch.floor(px_c).to(torch.int64)
        cy = torch.floor(py_c).to(torch.int64)
        gxs = cx[:, None] + offs.to(torch.int64)[None, :]
        gys = cy[:, None] + offs.to(torch.int64)[None, :]
        ddx = (gxs.to(torch.float64) - px_c[:, None]).to(torch.float32)
        ddy = (gys.to(torch.float64) - py_c[:, None]).to(torch.float32)
        r2 = ddx[:, None, :] ** 2 + ddy[:, :, None] ** 2
        s2 = (t_sigma**2)[:, None, None]
        prof = torch.where(t_moffat[:, None, None], (1.0 + r2 / (s2 * 2.0 * np.sqrt(2.0))) ** (-beta),
                           torch.exp(-0.5 * r2 / s2))
        prof = prof * torch.as_tensor(flux, device=device, dtype=torch.float32)[:, None, None]
        ys_b = gys[:, :, None].expand_as(prof)
        xs_b = gxs[:, None, :].expand_as(prof)
        ok = inside[:, None, None] & (ys_b >= 0) & (ys_b < h) & (xs_b >= 0) & (xs_b < w)
        signal.view(-1).index_put_((ys_b[ok] * w + xs_b[ok],), prof[ok], accumulate=True)
        del prof, ys_b, xs_b, ok, r2, ddx, ddy
        signal = signal * vignette + dark_rate * cfg.exposure_s
        frame = torch.poisson(torch.clamp(signal, min=0.0), generator=gen)
        frame += cfg.pedestal + cfg.read_noise * torch.randn((h, w), device=device, generator=gen)
        del signal
        if cfg.cosmic_ray_density:
            hits = int(rng.poisson(cfg.cosmic_ray_density * h * w))
            crx = rng.integers(0, w, hits)
            cry = rng.integers(0, h, hits)
            length = rng.integers(2, 7, hits)
            ang = rng.uniform(0, np.pi, hits)
            energy = rng.uniform(5000.0, 60000.0, hits)
            flat_idx, vals = [], []
            for step in range(6):
                on = step < length
                sy = np.clip(np.rint(cry + step * np.sin(ang)).astype(np.int64), 0, h - 1)
                sx = np.clip(np.rint(crx + step * np.cos(ang)).astype(np.int64), 0, w - 1)
                flat_idx.append(sy[on] * w + sx[on])
                vals.append(energy[on])
            frame.view(-1).index_put_((torch.as_tensor(np.concatenate(flat_idx), device=device),),
                                      torch.as_tensor(np.concatenate(vals), device=device, dtype=torch.float32),
                                      accumulate=True)
        if cfg.satellite_fraction and rng.random() < cfg.satellite_fraction:
            y0, y1 = rng.uniform(0, h, 2)
            xs = np.arange(w)
            ys = np.rint(y0 + (y1 - y0) * xs / max(w - 1, 1)).astype(np.int64)
            for t in (-1, 0, 1):
                yt = np.clip(ys + t, 0, h - 1)
                frame.view(-1).index_put_((torch.as_tensor(yt * w + xs, device=device),),
                                          torch.full((w,), 3000.0 if t == 0 else 1200.0, device=device),
                                          accumulate=True)
        lights[i] = _u16_as_i16(torch, frame)
        del frame
    return DeviceStack(cfg, lights, bias_frames, dark_frames, flat_frames, truth, cloud)


def render_affine_device(frames: int, height: int, width: int, stars_per_128: float = 30.0, linear_sigma: float = 1e-3,
                         max_shift: float = 0.5, fwhm: float = 2.5, sky: float = 1000.0, read_noise: float = 5.0,
                         seed: int = 3, device: str = "cuda"):
    """Calibrated float32 frames of one star field under random affine maps
    (the differentiable-registration workload): ~`stars_per_128` Gaussian
    stars per 128 x 128 pixels (FWHM `fwhm`, peak log-uniform 500-20000 ADU),
    sky `sky`, Poisson shot noise plus Gaussian read noise; frame i shows the
    field under forward = I + N(0, linear_sigma) on the linear terms and a
    uniform +-max_shift translation (frame 0: identity).  Returns a (N, H, W)
    float32 CUDA tensor and the (N, 3, 3) moving -> reference truth
    matrices."""
    import torch

    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    n_stars = int(round(stars_per_128 * height * width / 128.0 ** 2))
    margin = max_shift + 4.0 * linear_sigma * max(height, width) + 8
    xy = np.column_stack([rng.uniform(-margin, width + margin, n_stars), rng.uniform(-margin, height + margin, n_stars)])
    peak = torch.as_tensor(np.exp(rng.uniform(np.log(500.0), np.log(20000.0), n_stars)), device=device,
                           dtype=torch.float32)
    sigma = fwhm / 2.3548200450309493
    radius = int(np.ceil(4.0 * sigma)) + 1
    offs = torch.arange(-radius, radius + 1, device=device, dtype=torch.int64)
    out = torch.empty((frames, height, width), device=device, dtype=torch.float32)
    truth = np.empty((frames, 3, 3))
    for i in range(frames):
        fwd = np.eye(3)
        if i:
            fwd[:2, :2] += rng.normal(0.0, linear_sigma, (2, 2))
            fwd[:2, 2] = rng.uniform(-max_shift, max_shift, 2)
        truth[i] = np.linalg.inv(fwd)
        pos = torch.as_tensor(xy @ fwd[:2, :2].T + fwd[:2, 2], device=device)
        cx = torch.floor(pos[:, 0]).to(torch.int64)
        cy = torch.floor(pos[:, 1]).to(torch.int64)
        gx = cx[:, None] + offs[None, :]
        gy = cy[:, None] + offs[None, :]
        dx = (gx.to(torch.float64) - pos[:, 0:1]).to(torch.float32)
        dy = (gy.to(torch.float64) - pos[:, 1:2]).to(torch.float32)
        prof = torch.exp(-0.5 * (dx[:, None, :] ** 2 + dy[:, :, None] ** 2) / (sigma * sigma)) * peak[:, None, None]
        ys = gy[:, :, None].expand_as(prof)
        xs = gx[:, None, :].expand_as(prof)
        ok = (ys >= 0) & (ys < height) & (xs >= 0) & (xs < width)
        signal = torch.full((height * width,), sky, device=device, dtype=torch.float32)
        signal.index_put_((ys[ok] * width + xs[ok],), prof[ok], accumulate=True)
        frame = torch.poisson(signal, generator=gen)
        frame += read_noise * torch.randn(frame.shape, device=device, generator=gen)
        out[i] = frame.view(height, width)
    return out, truth
