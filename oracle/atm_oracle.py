"""CPU oracle for the reference's infinite-phase-screen atmosphere.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker, never by the
``oopao_gb300`` package.  A float64 restatement of ``OOPAO/Atmosphere.py``
(layers built by ``buildLayer`` :275-366, covariance matrices
``get_covariance_matrices`` :707-777 with the ``r0`` setter's Cholesky factor
:1017-1035, screens regenerated by ``generateNewPhaseScreen(0)`` :779-808,
frozen flow ``updateLayer`` / ``add_row`` :410-531, OPD assembly
``fill_OPD_support`` :589-622) and of the screen generators of
``OOPAO/phaseStats.py`` (``ft_phase_screen`` :153-199, ``ft_sh_phase_screen``
:201-271, ``makeCovarianceMatrix`` :72-132), for on-axis sources, ``mode=2``,
no boiling, geometric propagation.

The sub-pixel shift of the reference is scikit-image's ``warp(image,
SimilarityTransform(translation).inverse, order=3)`` (``OOPAO/tools/tools.py:
202-209``).  scikit-image is not installed where these fixtures are made; the
shift is restated as the bicubic convolution (Keys, a = -0.5) of
scikit-image's fast warp path, constant-zero outside the image, followed by
the clip to the input's range that ``warp`` applies by default.  Parity of
this step is pinned to that restatement only.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.special
from numpy.random import RandomState

R0_DEF = 0.15          # Atmosphere.r0_def, OOPAO/Atmosphere.py:185
N_EXTRA = 2            # Atmosphere.n_extra_pixel, :195


def ft_phase_screen(r0, L0, N, delta, seed, l0=1e-10):
    """``phaseStats.ft_phase_screen`` (:153-199), radians at 500 nm."""
    delta = float(delta)
    rs = RandomState(seed)
    del_f = 1. / (N * delta)
    fx = np.arange(-N / 2., N / 2.) * del_f
    fx, fy = np.meshgrid(fx, fx)
    f = np.sqrt(fx ** 2 + fy ** 2)
    fm = 5.92 / l0 / (2 * np.pi)
    f0 = 1. / L0
    psd = 0.023 * r0 ** (-5. / 3.) * np.exp(-1 * ((f / fm) ** 2)) / (((f ** 2) + (f0 ** 2)) ** (11. / 6))
    psd[int(N / 2), int(N / 2)] = 0
    cn = (rs.normal(size=(N, N)) + 1j * rs.normal(size=(N, N))) * np.sqrt(psd) * del_f
    return np.fft.fftshift(np.fft.fft2(np.fft.fftshift(cn))).real


def ft_sh_phase_screen(r0, L0, resolution, pixel_size, seed, l0=1e-10):
    """``phaseStats.ft_sh_phase_screen`` (:201-271): FFT screen plus three
    levels of 3x3 sub-harmonics."""
    pixel_size = float(pixel_size)
    rs = RandomState(seed)
    D = resolution * pixel_size
    phs_hi = ft_phase_screen(r0, L0, resolution, pixel_size, seed=seed, l0=l0)
    coords = np.arange(-resolution / 2, resolution / 2) * pixel_size
    x, y = np.meshgrid(coords, coords)
    phs_lo = np.zeros(phs_hi.shape)
    for p in range(1, 4):
        del_f = 1 / (3 ** p * D)
        fx = np.arange(-1, 2) * del_f
        fx, fy = np.meshgrid(fx, fx)
        f = np.sqrt(fx ** 2 + fy ** 2)
        fm = 5.92 / l0 / (2 * np.pi)
        f0 = 1. / L0
        psd = 0.023 * r0 ** (-5. / 3) * np.exp(-1 * (f / fm) ** 2) / ((f ** 2 + f0 ** 2) ** (11. / 6))
        psd[1, 1] = 0
        cn = (rs.normal(size=(3, 3)) + 1j * rs.normal(size=(3, 3))) * np.sqrt(psd) * del_f
        sh = np.zeros((resolution, resolution), dtype=complex)
        for i in range(0, 2):
            for j in range(0, 2):
                sh += cn[i, j] * np.exp(1j * 2 * np.pi * (fx[i, j] * x + fy[i, j] * y))
        phs_lo = phs_lo + sh
    phs_lo = phs_lo.real - phs_lo.real.mean()
    return phs_lo + phs_hi


def covariance_matrix(rho1, rho2, L0, r0_def=R0_DEF):
    """``phaseStats.makeCovarianceMatrix`` (:72-132) for complex coordinates."""
    rho = np.abs(rho1[:, None] - rho2[None, :])
    g = math.gamma
    ratio = (L0 / r0_def) ** (5. / 3)
    cst = (24. * g(6. / 5) / 5) ** (5. / 6) * (g(11. / 6) / ((2. ** (5. / 6)) * np.pi ** (8. / 3))) * ratio
    out = np.ones(rho.shape) * ((24. * g(6. / 5) / 5) ** (5. / 6)) * (g(11. / 6) * g(5. / 6) / (2 * np.pi ** (8. / 3))) \
        * ratio
    idx = np.where(rho != 0)
    u = 2 * np.pi * rho[idx] / L0
    out[idx] = cst * u ** (5. / 6) * scipy.special.kv(5. / 6, u)
    return out


def cubic_shift(image, tx, ty):
    """warp(image, translation(tx, ty).inverse, order=3) with clip: output
    pixel (r, c) = bicubic convolution of `image` at (r - ty, c - tx), zero
    outside the image, clipped to [min(image), max(image)]."""
    R, C = image.shape
    rr, cc = np.meshgrid(np.arange(R, dtype=np.float64) - ty, np.arange(C, dtype=np.float64) - tx, indexing='ij')
    r0 = np.floor(rr).astype(int)
    c0 = np.floor(cc).astype(int)
    xr, xc = rr - r0, cc - c0

    def pix(r, c):
        ok = (r >= 0) & (r < R) & (c >= 0) & (c < C)
        return np.where(ok, image[np.clip(r, 0, R - 1), np.clip(c, 0, C - 1)], 0.0)

    def cubic(x, f0, f1, f2, f3):
        return f1 + 0.5 * x * (f2 - f0 + x * (2.0 * f0 - 5.0 * f1 + 4.0 * f2 - f3 + x * (3.0 * (f1 - f2) + f3 - f0)))

    rows = [cubic(xc, *[pix(r0 + pr - 1, c0 + pc - 1) for pc in range(4)]) for pr in range(4)]
    out = cubic(xr, *rows)
    return np.clip(out, image.min(), image.max())


class OracleLayer:
    pass


class OracleAtmosphere:
    """Reference atmosphere for an on-axis source (telescope fov 0)."""

    def __init__(self, res, diameter, sampling_time, r0, L0, fractional_r0, wind_speed, wind_direction,
                 altitude, wavelength=500e-9, t_boiling=None):
        self.res, self.D, self.dt = res, diameter, sampling_time
        n_layers = len(fractional_r0)
        self.t_boiling = list(t_boiling) if t_boiling is not None else [None] * n_layers
        self.r0, self.L0 = r0, L0
        self.fractional_r0 = list(fractional_r0)
        self.wavelength = wavelength
        self.layers = []
        cov = None
        for i in range(len(self.fractional_r0)):
            L = OracleLayer()
            L.vY = wind_speed[i] * np.cos(np.deg2rad(wind_direction[i]))
            L.vX = wind_speed[i] * np.sin(np.deg2rad(wind_direction[i]))
            L.altitude = altitude[i]
            L.resolution = int(np.ceil((res / diameter) * diameter)) + 4
            L.D = L.resolution * diameter / res
            L.pixel_size = L.D / L.resolution
            n = L.resolution + N_EXTRA
            L.outer = np.ones((n, n))
            L.outer[1:-1, 1:-1] = 0
            L.inner = np.ones((n, n)) - L.outer
            L.inner[1 + N_EXTRA:-1 - N_EXTRA, 1 + N_EXTRA:-1 - N_EXTRA] = 0
            x = np.linspace(0, L.resolution + 1, L.resolution + 2) * L.D / (L.resolution - 1)
            u, v = np.meshgrid(x, x)
            inner_z = u[L.inner != 0] + 1j * v[L.inner != 0]
            outer_z = u[L.outer != 0] + 1j * v[L.outer != 0]
            if cov is None:      # SCAO: the matrices are computed once (:711-724)
                zz = covariance_matrix(inner_z, inner_z, L0)
                zz_inv = np.linalg.pinv(zz)
                zx = covariance_matrix(inner_z, outer_z, L0)
                xx = covariance_matrix(outer_z, outer_z, L0)
                s = (R0_DEF / r0) ** (5 / 3)
                A = (zx * s).T @ (zz_inv / s)
                B = np.linalg.cholesky(xx * s - A @ (zx * s))
                cov = (A, B)
            L.A, L.B = cov
            self.layers.append(L)
        self.generate_new_phase_screen(0)

    def generate_new_phase_screen(self, seed):
        """``generateNewPhaseScreen`` (:779-808)."""
        for i, L in enumerate(self.layers):
            L.opd = ft_sh_phase_screen(self.r0, self.L0, L.resolution, L.D / L.resolution, seed=seed + i)
            L.rs = RandomState(seed + i * 1000)
            n = L.resolution + N_EXTRA
            L.map = np.zeros((n, n))
            z = L.opd[L.inner[1:-1, 1:-1] != 0]
            L.map[L.outer != 0] = L.A @ z + L.B @ L.rs.normal(size=L.B.shape[1])
            L.map[L.outer == 0] = L.opd.reshape(-1)
            L.not_done_once = True
            L.boiling_seed = 100000 + seed + i * 100000

    def _boil(self, i, L):
        """``apply_boiling`` (:387-408): AR(1) decorrelation of the map,
        map = alpha map + beta phi with alpha = exp(-dt / t_boiling) and phi a
        fresh screen of the map's size; returns whether the layer boiled."""
        t_b = self.t_boiling[i]
        if t_b is None or not np.isfinite(t_b) or t_b <= 0:
            return False
        alpha = float(np.exp(-self.dt / t_b))
        if alpha >= 1.0 - 1e-6:
            return False
        beta = float(np.sqrt(max(0.0, 1.0 - alpha ** 2)))
        L.boiling_seed += 1
        phi = ft_sh_phase_screen(self.r0, self.L0, L.map.shape[0], L.D / L.resolution, seed=L.boiling_seed)
        L.map = alpha * L.map + beta * phi
        return True

    def _add_row(self, L, step):
        """``add_row`` (:410-419): one-pixel shift, ring extrusion."""
        tmp = cubic_shift(L.map, step[0], step[1])
        shifted = tmp[1:-1, 1:-1]
        z = shifted[L.inner[1:-1, 1:-1] != 0]
        L.map[L.outer != 0] = L.A @ z + L.B @ L.rs.normal(size=L.B.shape[1])
        L.map[L.outer == 0] = shifted.reshape(-1)
        return shifted

    def update(self):
        """``updateLayer`` for every layer (:447-514): boiling first, then the
        frozen-flow moves; a still layer that boiled shows its map's interior."""
        for i, L in enumerate(self.layers):
            boiled = self._boil(i, L)
            if L.vX == 0 and L.vY == 0:
                if boiled:
                    L.opd = L.map[L.outer == 0].reshape(L.resolution, L.resolution)
                continue
            if L.not_done_once:
                L.not_done_once = False
                L.ratio = np.array([L.vX * self.dt / L.pixel_size, L.vY * self.dt / L.pixel_size])
                L.buff = np.zeros(2)
            ratio = L.ratio
            tmp = np.abs(ratio)
            tmp[np.isinf(tmp)] = 0
            n_scr = tmp.astype('int')
            step = np.zeros(2)
            for _ in range(n_scr.min()):
                step[0] = 1
                step[1] = 1
                step = step * np.sign(ratio)
                L.opd = self._add_row(L, step)
            for _ in range(n_scr.max() - n_scr.min()):
                step[0] = 1
                step[1] = 1
                step = step * np.sign(ratio)
                step[np.where(n_scr == n_scr.min())] = 0
                L.opd = self._add_row(L, step)
            sub = np.zeros(2)
            sub[0] = (np.abs(ratio[0]) % 1) * np.sign(ratio[0])
            sub[1] = (np.abs(ratio[1]) % 1) * np.sign(ratio[1])
            L.buff += sub
            if np.abs(L.buff[0]) >= 1 or np.abs(L.buff[1]) >= 1:
                step[0] = 1 * np.sign(L.buff[0])
                step[1] = 1 * np.sign(L.buff[1])
                step[np.where(np.abs(L.buff) < 1)] = 0
                L.opd = self._add_row(L, step)
            L.buff[0] = (np.abs(L.buff[0]) % 1) * np.sign(L.buff[0])
            L.buff[1] = (np.abs(L.buff[1]) % 1) * np.sign(L.buff[1])
            L.opd = cubic_shift(L.map, L.buff[0], L.buff[1])[1:-1, 1:-1]

    @property
    def opd(self):
        """``fill_OPD_support`` for an on-axis source: centred res x res crop of
        every layer, radians -> metres, times sqrt(fractionalR0), summed."""
        out = np.zeros((self.res, self.res))
        for i, L in enumerate(self.layers):
            c = L.resolution // 2
            crop = L.opd[c - self.res // 2:c + self.res // 2, c - self.res // 2:c + self.res // 2]
            out += crop * self.wavelength / 2 / np.pi * np.sqrt(self.fractional_r0[i])
        return out
