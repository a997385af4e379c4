"""Seeded synthetic instruments for the response benchmarks (numpy, float64).

No public dataset exists for this path; these generators follow the stated
recipes of the five benchmark configurations:

1. 256^2 sky, 1 module x 1 energy, 8x8 patches of stride 32, margin 16 (P=96);
   elliptical Gaussian PSFs (sigma 1 -> 3 px with distance from the centre,
   axis ratio 0.8); exposure 1e3 (1 - 0.05 r^2 / r_max^2).
2. 1024^2 sky, 7 modules x 3 energies, 16x16 patches of stride 64, margin 32
   (P=192); Moffat(beta=2.5) PSFs, FWHM 2 -> 8 px radially, module k rotated by
   k*51.4 deg (axis ratio 0.8 so that the rotation matters), FWHM scaled by
   (1 + 0.1 e) per energy; per-module exposure 1e3 + 1e3 k/6 with 1 % of the
   pixels masked (seed 2, the same pixels for every energy).
3. config-1 PSF recipe on a 1024^2 x 3 sky with the config-2 grid; the sky is
   exp of a correlated field with power-law slope -4 (xi ~ N(0,1), seed 3).
4. 2048^2 x 3 sky of GRF diffuse plus 0.1 % point sources (flux log-uniform
   1e1..1e5), 32x32 patches of stride 64, margin 32 (P=192); Gaussian core
   sigma 0.5 -> 6 px plus a 5 % r^-3 wing out to 30 px.
5. uneven batch of 64 independent problems (sizes log-uniform 128^2..1024^2,
   FFT sides 32/64/128, 1..3 energies, Gaussian PSFs sigma 0.8 -> 0.8..4 px).

Skies are exp(s) of a Gaussian random field with P(k) ~ (1 + (k/0.05)^2)^-2
(k in cycles/pixel), rescaled to std 1.5 and the stated mean.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


@dataclass
class Instrument:
    name: str
    n_modules: int
    n_energies: int
    shape: tuple
    n_patches: int
    margin: int
    sky: np.ndarray            # (E, nx, ny)
    psf: np.ndarray            # (M, n^2, E, K, K) pre-cut, unit sum ((M, n^2, K, K): all E)
    exposure: np.ndarray       # (M, E, nx, ny)
    readmask: np.ndarray       # (M, E, nx, ny) bool, True = read out
    pixel_area: float = 1.0
    extra: dict = field(default_factory=dict)

    @property
    def dx(self):
        return self.shape[0] // self.n_patches

    @property
    def K(self):
        return 2 * self.dx

    @property
    def P(self):
        return self.K + 2 * self.margin

    @property
    def mpix(self):
        return self.n_modules * self.n_energies * self.shape[0] * self.shape[1] / 1e6


def grf(shape, rng, mean=2.0, std=1.5, k0=0.05):
    """Gaussian random field with P(k) ~ (1 + (k/k0)^2)^-2, rescaled."""
    kx = np.fft.fftfreq(shape[0])
    ky = np.fft.fftfreq(shape[1])
    k = np.sqrt(kx[:, None] ** 2 + ky[None, :] ** 2)
    pk = (1.0 + (k / k0) ** 2) ** -2
    noise = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    s = np.fft.ifft2(noise * np.sqrt(pk)).real
    s = (s - s.mean()) / s.std()
    return s * std + mean


def powerlaw_field(shape, rng, slope=-4.0, mean=1.0, std=1.0):
    """Correlated field with power spectrum ~ k^slope (k >= 1/N), xi ~ N(0,1)."""
    kx = np.fft.fftfreq(shape[0])
    ky = np.fft.fftfreq(shape[1])
    k = np.sqrt(kx[:, None] ** 2 + ky[None, :] ** 2)
    k[0, 0] = 1.0 / max(shape)
    pk = k ** slope
    xi = rng.normal(size=shape)
    s = np.fft.ifft2(np.fft.fft2(xi) * np.sqrt(pk)).real
    s = (s - s.mean()) / s.std()
    return s * std + mean


def patch_centres(nx, n):
    """(n^2, 2) patch centres (row, col) in slice_patches order (k%n, k//n)."""
    dx = nx // n
    k = np.arange(n * n)
    return np.stack([(k % n) * dx + dx // 2, (k // n) * dx + dx // 2], axis=1).astype(float)


def _window(K):
    """Offsets (u, v) of the pre-cut window: origin at local index dx = K/2."""
    off = np.arange(K) - K // 2
    return np.meshgrid(off, off, indexing="ij")


def _rot(u, v, theta):
    c, s = np.cos(theta), np.sin(theta)
    return c * u + s * v, -s * u + c * v


def gaussian_psfs(nx, n, K, sig_min, sig_max, ratio=0.8, wing=0.0, wing_rmax=30.0):
    """Elliptical Gaussian (plus optional r^-3 wing) per patch, unit sum."""
    cen = patch_centres(nx, n)
    c0 = nx / 2.0
    r = np.hypot(cen[:, 0] - c0, cen[:, 1] - c0)
    rmax = max(r.max(), 1e-9)
    u, v = _window(K)
    out = np.empty((n * n, K, K))
    for k in range(n * n):
        sig = sig_min + (sig_max - sig_min) * r[k] / rmax
        theta = np.arctan2(cen[k, 1] - c0, cen[k, 0] - c0)
        a, b = _rot(u, v, theta)
        core = np.exp(-0.5 * ((a / sig) ** 2 + (b / (ratio * sig)) ** 2))
        core /= core.sum()
        if wing > 0:
            rr = np.hypot(u, v)
            w = np.where(rr <= wing_rmax, (1.0 + rr) ** -3.0, 0.0)
            w /= w.sum()
            core = (1 - wing) * core + wing * w
        out[k] = core / core.sum()
    return out


def moffat_psfs(nx, n, K, fwhm_min, fwhm_max, beta=2.5, rot=0.0, ratio=0.8):
    cen = patch_centres(nx, n)
    c0 = nx / 2.0
    r = np.hypot(cen[:, 0] - c0, cen[:, 1] - c0)
    rmax = max(r.max(), 1e-9)
    u, v = _window(K)
    out = np.empty((n * n, K, K))
    for k in range(n * n):
        fwhm = fwhm_min + (fwhm_max - fwhm_min) * r[k] / rmax
        alpha = fwhm / (2.0 * np.sqrt(2.0 ** (1.0 / beta) - 1.0))
        a, b = _rot(u, v, rot)
        q = (a / alpha) ** 2 + (b / (ratio * alpha)) ** 2
        p = (1.0 + q) ** -beta
        out[k] = p / p.sum()
    return out


def config1(nx=256, n=8, margin=16, seed=0) -> Instrument:
    rng = np.random.default_rng(seed)
    sky = np.exp(grf((nx, nx), rng, mean=2.0))[None]
    K = 2 * (nx // n)
    psf = gaussian_psfs(nx, n, K, 1.0, 3.0)[None, :, None]
    yy, xx = np.meshgrid(np.arange(nx), np.arange(nx), indexing="ij")
    r2 = (yy - nx / 2 + 0.5) ** 2 + (xx - nx / 2 + 0.5) ** 2
    exposure = (1e3 * (1.0 - 0.05 * r2 / r2.max()))[None, None]
    readmask = np.ones_like(exposure, dtype=bool)
    return Instrument("config1", 1, 1, (nx, nx), n, margin, sky, psf, exposure, readmask)


def config2(nx=1024, dx=64, margin=32, n_modules=7, n_energies=3, seed=0,
            dtype=np.float64) -> Instrument:
    """Headline workload (full size by default; smaller ``nx`` keeps P = 192)."""
    rng = np.random.default_rng(seed)
    n = nx // dx
    means = [1.0, 1.5, 2.0, 2.5, 3.0][:n_energies]
    sky = np.stack([np.exp(grf((nx, nx), rng, mean=mu)) for mu in means]).astype(dtype)
    K = 2 * dx
    psf = np.empty((n_modules, n * n, n_energies, K, K), dtype=dtype)
    for m in range(n_modules):
        for e in range(n_energies):
            s = 1.0 + 0.1 * e
            psf[m, :, e] = moffat_psfs(nx, n, K, 2.0 * s, 8.0 * s, beta=2.5,
                                       rot=np.deg2rad(51.4 * m))
    mrng = np.random.default_rng(2)
    bad = mrng.random((n_modules, 1, nx, nx)) < 0.01
    readmask = np.broadcast_to(~bad, (n_modules, n_energies, nx, nx)).copy()
    level = 1e3 + 1e3 * np.arange(n_modules) / 6.0
    exposure = (level[:, None, None, None] * readmask).astype(dtype)
    return Instrument("config2", n_modules, n_energies, (nx, nx), n, margin, sky, psf, exposure,
                      readmask)


def config3(nx=1024, dx=64, margin=32, n_energies=3, seed=3) -> Instrument:
    rng = np.random.default_rng(seed)
    n = nx // dx
    sky = np.stack([np.exp(powerlaw_field((nx, nx), rng, mean=1.0 + 0.5 * e))
                    for e in range(n_energies)])
    K = 2 * dx
    psf = np.repeat(gaussian_psfs(nx, n, K, 1.0, 3.0)[None, :, None], n_energies, axis=2)
    yy, xx = np.meshgrid(np.arange(nx), np.arange(nx), indexing="ij")
    r2 = (yy - nx / 2 + 0.5) ** 2 + (xx - nx / 2 + 0.5) ** 2
    exposure = np.broadcast_to((1e3 * (1.0 - 0.05 * r2 / r2.max()))[None, None],
                               (1, n_energies, nx, nx)).copy()
    readmask = np.ones_like(exposure, dtype=bool)
    return Instrument("config3", 1, n_energies, (nx, nx), n, margin, sky, psf, exposure,
                      readmask)


def config4(nx=2048, dx=64, margin=32, n_energies=3, seed=0) -> Instrument:
    rng = np.random.default_rng(seed)
    n = nx // dx
    sky = np.stack([np.exp(grf((nx, nx), rng, mean=1.0 + 0.5 * e))
                    for e in range(n_energies)])
    npts = max(1, int(round(1e-3 * nx * nx)))
    pos = rng.integers(0, nx, size=(npts, 2))
    flux = 10.0 ** rng.uniform(1.0, 5.0, size=npts)
    for e in range(n_energies):
        np.add.at(sky[e], (pos[:, 0], pos[:, 1]), flux)
    K = 2 * dx
    psf = np.repeat(gaussian_psfs(nx, n, K, 0.5, 6.0, wing=0.05)[None, :, None], n_energies,
                    axis=2)
    exposure = np.full((1, n_energies, nx, nx), 1e3)
    readmask = np.ones_like(exposure, dtype=bool)
    return Instrument("config4", 1, n_energies, (nx, nx), n, margin, sky, psf, exposure,
                      readmask)


def config5_geometry(count=64, seed=4, min_side=128, max_side=1024) -> List[dict]:
    """Geometry of the uneven batch, one dict per problem.

    The side is drawn log-uniform in [min_side, max_side], the number of
    energies in 1..3 and the widest PSF sigma in 0.8..4 px.  The margin covers
    3 sigma of the widest PSF (at least 4 px); the FFT side P is 32, 64 or 128
    and the stride dx = P/2 - margin (made even); (n, P) with n in 4..16 is
    the pair whose field side n * dx is closest to the draw, where each
    doubling of P counts as a 4 % miss (smaller FFTs are preferred).  With P <= 128 and n <= 16 the largest reachable side is 16 * 60 =
    960: larger draws take the largest side their margin allows."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        side = float(np.exp(rng.uniform(np.log(min_side), np.log(max_side))))
        n_e = int(rng.integers(1, 4))
        sig_max = float(rng.uniform(0.8, 4.0))
        m0 = max(4, int(np.ceil(3.0 * sig_max)))
        best = None
        for P in (32, 64, 128):
            dx = P // 2 - m0
            dx -= dx % 2
            if dx < 2:
                continue
            for n in range(4, 17):
                # closest side; each doubling of P costs as much as a 4 % miss
                cost = abs(np.log(n * dx / side)) + 0.04 * np.log2(P / 32)
                if best is None or cost < best[0] - 1e-12:
                    best = (cost, P, n, dx)
        _, P, n, dx = best
        out.append(dict(nx=n * dx, n=n, dx=dx, margin=P // 2 - dx, P=P, E=n_e,
                        sigma=(0.8, sig_max), seed=1000 + i))
    return out


def config5(count=64, seed=4, min_side=128, max_side=1024) -> List[Instrument]:
    """The uneven batch: independent one-module problems of the geometry of
    :func:`config5_geometry`.  Sky: GRF recipe with mean 1 + 0.5 e; PSFs:
    Gaussians of sigma 0.8 px at the field centre growing linearly to the
    problem's widest sigma, one set for all energies (psf shape (1, n^2, K, K),
    broadcast over energies); exposure 1e3 everywhere, nothing masked."""
    out = []
    for i, g in enumerate(config5_geometry(count, seed, min_side, max_side)):
        rng = np.random.default_rng(g["seed"])
        nx, n, n_e = g["nx"], g["n"], g["E"]
        sky = np.stack([np.exp(grf((nx, nx), rng, mean=1.0 + 0.5 * e)) for e in range(n_e)])
        psf = gaussian_psfs(nx, n, 2 * g["dx"], g["sigma"][0], g["sigma"][1])[None]
        exposure = np.full((1, n_e, nx, nx), 1e3)
        readmask = np.ones_like(exposure, dtype=bool)
        out.append(Instrument(f"uneven{i}", 1, n_e, (nx, nx), n, g["margin"], sky, psf,
                              exposure, readmask, extra=dict(P=g["P"])))
    return out


def poisson_data(lam_readout: np.ndarray, seed: int = 1) -> np.ndarray:
    """Poisson counts (int32) of expected counts in readout order."""
    rng = np.random.default_rng(seed)
    return rng.poisson(np.maximum(np.asarray(lam_readout, np.float64), 0.0)).astype(np.int32)


def erosita_like_psf_infos(n_energies=2, n_radii=5, grid=64, field=(256, 256),
                           distances=(1.0, 1.0), seed=0) -> List[dict]:
    """Gridded PSFs at a few off-axis radii in the layout of
    ``eROSITA_PSF._get_psf_infos`` (one dict per energy): elongated Gaussians
    whose width grows with the radius and with the energy, sampled on a
    ``grid`` x ``grid`` PSF grid of half the sky pixel, centre indices near
    the grid centre, radii given out of order, pointing at the field centre."""
    rng = np.random.default_rng(seed)
    infos = []
    for e in range(n_energies):
        rs = np.linspace(0.0, 0.6 * field[0] * distances[0], n_radii)
        order = rng.permutation(n_radii)
        delta = (0.5 * distances[0], 0.5 * distances[1])
        cids = np.stack([np.full(n_radii, grid / 2) + rng.integers(-2, 3, n_radii),
                         np.full(n_radii, grid / 2) + rng.integers(-2, 3, n_radii)], -1)
        psfs = []
        for j in range(n_radii):
            sig = (1.0 + 0.08 * rs[j] / distances[0]) * (1.0 + 0.2 * e)
            u = (np.arange(grid) - cids[j, 0]) * delta[0]
            v = (np.arange(grid) - cids[j, 1]) * delta[1]
            uu, vv = np.meshgrid(u, v, indexing="ij")
            p = np.exp(-0.5 * ((uu / (1.6 * sig)) ** 2 + (vv / sig) ** 2))
            psfs.append(p / p.sum())
        infos.append({"psfs": np.array(psfs)[order], "rs": rs[order],
                      "patch_center_ids": cids[order], "patch_deltas": delta,
                      "pointing_center": (field[0] / 2 * distances[0],
                                          field[1] / 2 * distances[1])})
    return infos
