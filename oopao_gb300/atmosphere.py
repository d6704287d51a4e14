"""Infinite-phase-screen atmosphere: drop-in for the reference ``Atmosphere``
(``OOPAO/Atmosphere.py``) for an on-axis source, geometric propagation.

Set-up follows the reference step by step:

* layers of (res + 4) pixels plus a 1-pixel ring (``buildLayer`` :275-366);
* screens from ``ft_sh_phase_screen`` (FFT method plus sub-harmonics,
  ``OOPAO/phaseStats.py:201-271``), seeded by ``generateNewPhaseScreen(0)``
  (:779-808) as the reference's ``initializeAtmosphere`` does;
* the extrusion matrices from the von Karman covariance of the ring pixels
  (``makeCovarianceMatrix`` :72-132, ``get_covariance_matrices`` :707-777):
  A = ZX^T pinv(ZZ), B = chol(XX - A ZX).  The covariances are evaluated on
  the host in float64; the pseudo-inverse and the Cholesky factor are
  computed in float64 on the GPU.

Every ``update()`` (and every step of a captured closed loop) runs
``oopao_atm_update``: the one-pixel moves of each layer with their ring
extrusion X = A Z + B w, then the bicubic sub-pixel shift and the OPD sum.
The moves, sub-pixel offsets and extrusion normals of each step are planned
on the host ahead of time with the reference's arithmetic (``updateLayer``
:450-514) and each layer's ``RandomState(seed + 1000 i)``.

Boiling layers (``t_boiling``, ``apply_boiling`` :387-408) decorrelate
before each step's moves: map = alpha map + beta phi, phi a new screen drawn
on the host with the layer's seed counter (``oopao_atm_boil`` on the GPU).
A captured closed loop draws the screens of its whole horizon up front
(``boiling_horizon``).

The sub-pixel shift is the reference's scikit-image ``warp(order=3)``: the
bicubic convolution kernel (Keys, a = -0.5) with zeros outside the map and
the output clipped to the map's range.
"""
import math
import time

import numpy as np
import torch
from numpy.random import RandomState

from . import _native as N
from .runtime import device
from .tools import OopaoError, warning

R0_DEF = 0.15
N_EXTRA = 2


def ft_phase_screen(r0, L0, n, delta, seed, l0=1e-10):
    """FFT-method von Karman phase screen in radians (OOPAO/phaseStats.py:153-199)."""
    rs = RandomState(seed)
    del_f = 1. / (n * float(delta))
    f1 = np.arange(-n / 2., n / 2.) * del_f
    fx, fy = np.meshgrid(f1, f1)
    f = np.sqrt(fx ** 2 + fy ** 2)
    fm = 5.92 / l0 / (2 * np.pi)
    psd = 0.023 * r0 ** (-5. / 3.) * np.exp(-((f / fm) ** 2)) / ((f ** 2 + (1. / L0) ** 2) ** (11. / 6))
    psd[n // 2, n // 2] = 0
    cn = (rs.normal(size=(n, n)) + 1j * rs.normal(size=(n, n))) * np.sqrt(psd) * del_f
    return np.fft.fftshift(np.fft.fft2(np.fft.fftshift(cn))).real


def ft_sh_phase_screen(r0, L0, n, delta, seed, l0=1e-10):
    """FFT screen plus three 3x3 sub-harmonic levels (OOPAO/phaseStats.py:201-271)."""
    rs = RandomState(seed)
    size = n * float(delta)
    hi = ft_phase_screen(r0, L0, n, delta, seed, l0)
    c = np.arange(-n / 2, n / 2) * float(delta)
    x, y = np.meshgrid(c, c)
    lo = np.zeros(hi.shape)
    fm = 5.92 / l0 / (2 * np.pi)
    for p in range(1, 4):
        df = 1 / (3 ** p * size)
        fx, fy = np.meshgrid(np.arange(-1, 2) * df, np.arange(-1, 2) * df)
        f = np.sqrt(fx ** 2 + fy ** 2)
        psd = 0.023 * r0 ** (-5. / 3) * np.exp(-(f / fm) ** 2) / ((f ** 2 + (1. / L0) ** 2) ** (11. / 6))
        psd[1, 1] = 0
        cn = (rs.normal(size=(3, 3)) + 1j * rs.normal(size=(3, 3))) * np.sqrt(psd) * df
        sh = np.zeros((n, n), dtype=complex)
        for i in range(2):
            for j in range(2):
                sh += cn[i, j] * np.exp(1j * 2 * np.pi * (fx[i, j] * x + fy[i, j] * y))
        lo = lo + sh
    return (lo.real - lo.real.mean()) + hi


def phase_covariance(rho1, rho2, L0, r0=R0_DEF):
    """Von Karman phase covariance between two sets of points given as complex
    coordinates (OOPAO/phaseStats.py:72-132), radians^2 at r0."""
    from scipy.special import kv
    g = math.gamma
    rho = np.abs(rho1[:, None] - rho2[None, :])
    ratio = (L0 / r0) ** (5. / 3)
    k = (24. * g(6. / 5) / 5) ** (5. / 6)
    out = np.full(rho.shape, k * (g(11. / 6) * g(5. / 6) / (2 * np.pi ** (8. / 3))) * ratio)
    nz = rho != 0
    u = 2 * np.pi * rho[nz] / L0
    out[nz] = k * (g(11. / 6) / ((2. ** (5. / 6)) * np.pi ** (8. / 3))) * ratio * u ** (5. / 6) * kv(5. / 6, u)
    return out


class _Layer:
    pass


class Atmosphere:
    def __init__(self, telescope, r0: float, L0: float, windSpeed: list, fractionalR0: list, windDirection: list,
                 altitude: list, src=None, param=None, elevation: float = 90.0, mode: float = 2,
                 angular_spectrum_propagation: bool = False, geometric_phase_backup: bool = False,
                 unwrap_diffractive_phase=False, rytov_var: float = None, rytov_wvl: float = 500e-9,
                 t_boiling=None):
        if angular_spectrum_propagation or geometric_phase_backup or unwrap_diffractive_phase:
            raise OopaoError('oopao_gb300 Atmosphere propagates geometrically only')
        if elevation != 90.0:
            raise OopaoError('oopao_gb300 Atmosphere supports zenith pointing (elevation=90) only')
        if mode == 1:
            raise DeprecationWarning('The dependency to the aotools package has been deprecated.')
        n = len(fractionalR0)
        if not (len(windSpeed) == len(windDirection) == len(altitude) == n):
            raise OopaoError('windSpeed, windDirection, altitude and fractionalR0 must have one value per layer')
        self.hasNotBeenInitialized = True
        self.telescope = telescope
        self.wavelength = 500e-9
        self.r0_def = R0_DEF
        self._r0 = r0
        self._L0 = L0
        self.fractionalR0 = list(fractionalR0)
        self.nLayer = n
        self._t_boiling = self.get_t_boiling(t_boiling)
        self._windSpeed = list(windSpeed)
        self._windDirection = list(windDirection)
        self.altitude = list(altitude)
        self.elevation = elevation
        self.mode = mode
        self.n_extra_pixel = N_EXTRA
        self.param = param
        self.tag = 'atmosphere'
        self.rad2arcsec = (180. / np.pi) * 3600
        self.seeingArcsec = self.rad2arcsec * (self.wavelength / r0)
        self.cn2 = (r0 ** (-5. / 3) / (0.423 * (2 * np.pi / self.wavelength) ** 2)) / np.max([1, np.max(altitude)])
        self.V0 = (np.sum(np.asarray(self.fractionalR0) * np.asarray(self._windSpeed) ** (5 / 3))) ** (3 / 5)
        self.tau0 = 0.31 * r0 / self.V0
        if src is None and getattr(telescope, 'src', None) is None:
            raise OopaoError('The Atmosphere object requires a Source. Either provide a Source directly as an '
                             'attribute, or propagate the Source through the Telescope before creating the '
                             'Atmosphere.')
        self.src = src if src is not None else telescope.src
        self.user_defined_opd = None

    # ------------------------------------------------------------------ set-up
    def initializeAtmosphere(self, telescope=None, compute_covariance=True):
        """Build the layers and their extrusion matrices (OOPAO/Atmosphere.py:227-273)."""
        if telescope is not None:
            self.telescope = telescope
        tel = self.telescope
        if getattr(tel, 'fov', 0) not in (0, None):
            raise OopaoError('oopao_gb300 Atmosphere supports an on-axis source only (telescope fov 0)')
        self.compute_covariance = compute_covariance
        self._dev = device()
        d = self._dev
        res, D = tel.resolution, tel.D
        self.layers = []
        for i in range(self.nLayer):
            L = _Layer()
            L.resolution = int(np.ceil((res / D) * D)) + 4
            L.D = L.resolution * D / res
            L.pixel_size = L.D / L.resolution
            L.altitude = self.altitude[i]
            self.layers.append(L)
        L = self.layers[0]
        n = L.resolution + N_EXTRA
        self._n = n
        outer = np.ones((n, n))
        outer[1:-1, 1:-1] = 0
        inner = np.ones((n, n)) - outer
        inner[1 + N_EXTRA:-1 - N_EXTRA, 1 + N_EXTRA:-1 - N_EXTRA] = 0
        self.outerMask, self.innerMask = outer, inner
        self._inner_idx = np.flatnonzero(inner.reshape(-1) != 0).astype(np.int32)
        self._outer_idx = np.flatnonzero(outer.reshape(-1) != 0).astype(np.int32)
        if compute_covariance:
            x = np.linspace(0, L.resolution + 1, L.resolution + 2) * L.D / (L.resolution - 1)
            u, v = np.meshgrid(x, x)
            zi = u[inner != 0] + 1j * v[inner != 0]
            zo = u[outer != 0] + 1j * v[outer != 0]
            zz = torch.as_tensor(phase_covariance(zi, zi, self._L0), device=d)
            self._zx = torch.as_tensor(phase_covariance(zi, zo, self._L0), device=d)
            self._xx = torch.as_tensor(phase_covariance(zo, zo, self._L0), device=d)
            # numpy's pinv cut-off (1e-15 of the largest singular value)
            self._zz_inv = torch.linalg.pinv(zz, rtol=1e-15)
            self._set_matrices()
        self._idx_dev = (torch.as_tensor(self._inner_idx, device=d), torch.as_tensor(self._outer_idx, device=d))
        self._scale_dev = self._scale()
        self._frozen = False
        self._step_dev = torch.zeros(1, dtype=torch.int32, device=d)
        self._err = torch.zeros(1, dtype=torch.int32, device=d)
        self._range = torch.zeros((self.nLayer, 32, 2), dtype=torch.float64, device=d)
        self._mirror = torch.zeros((self.nLayer, n, n), dtype=torch.float32, device=d)
        self._opd_dev = torch.zeros((res, res), dtype=torch.float32, device=d)
        self.hasNotBeenInitialized = False
        self.generateNewPhaseScreen(0)
        print(self)

    def _set_matrices(self):
        s = (self.r0_def / self._r0) ** (5 / 3)
        A = (self._zx * s).T @ (self._zz_inv / s)
        B = torch.linalg.cholesky(self._xx * s - A @ (self._zx * s))
        self._A, self._B = A.contiguous(), B.contiguous()

    def generateNewPhaseScreen(self, seed=None):
        """New screens and extrusion random streams (OOPAO/Atmosphere.py:779-808)."""
        if seed is None:
            t = time.localtime()
            seed = t.tm_hour * 3600 + t.tm_min * 60 + t.tm_sec
        d, n, res = self._dev, self._n, self.telescope.resolution
        maps = torch.zeros((2, self.nLayer, n, n), dtype=torch.float64, device=d)
        inner_idx = torch.as_tensor(self._inner_idx.astype(np.int64), device=d)
        outer_idx = torch.as_tensor(self._outer_idx.astype(np.int64), device=d)
        for i, L in enumerate(self.layers):
            gen = ft_sh_phase_screen if self.mode == 2 else ft_phase_screen
            scr = gen(self._r0, self._L0, L.resolution, L.D / L.resolution, seed=seed + i)
            L.rs = RandomState(seed + i * 1000)
            m = maps[0, i].view(-1)
            m.view(n, n)[1:-1, 1:-1] = torch.as_tensor(scr, device=d)
            L.boiling_seed = 100000 + seed + i * 100000
            if self.compute_covariance:
                w = torch.as_tensor(L.rs.normal(size=self._B.shape[1]), device=d)
                m[outer_idx] = self._A @ m[inner_idx] + self._B @ w
            L.not_done_once = True
        self._maps = maps
        self._maps0 = maps[0].clone()
        self._seed = seed
        self._reset_plan()
        self._step = 0
        self._step_dev.zero_()
        self._launch(advance=False, moved=False)

    # ------------------------------------------------------------------ plan
    def _ratio(self, L, i):
        vy = self._windSpeed[i] * np.cos(np.deg2rad(self._windDirection[i]))
        vx = self._windSpeed[i] * np.sin(np.deg2rad(self._windDirection[i]))
        return vx, vy, np.array([vx * self.telescope.samplingTime / L.pixel_size,
                                 vy * self.telescope.samplingTime / L.pixel_size])

    def _reset_plan(self):
        self._plan_moves = []   # per step: per layer: list of (dx, dy, normal row)
        self._plan_buff = []    # per step: per layer: (bx, by)
        self._normals = []
        for i, L in enumerate(self.layers):
            L.plan_done_once = False
            L.plan_buff = np.zeros(2)
        self._slots = None
        self._dev_plan_len = -1

    def _plan_one(self):
        moves, buffs = [], []
        for i, L in enumerate(self.layers):
            mv = []
            vx, vy, ratio_now = self._ratio(L, i)
            if vx == 0 and vy == 0:
                moves.append(mv)
                buffs.append((0.0, 0.0))
                continue
            if not L.plan_done_once:   # updateLayer computes the ratio at its first call only
                L.plan_done_once = True
                L.plan_ratio = ratio_now
                L.plan_buff = np.zeros(2)
            ratio = L.plan_ratio
            tmp = np.abs(ratio)
            tmp[np.isinf(tmp)] = 0
            n_scr = tmp.astype('int')
            step = np.zeros(2)

            def add(s):
                mv.append((int(s[0]), int(s[1]), len(self._normals)))
                self._normals.append(L.rs.normal(size=self._B.shape[1]))

            for _ in range(n_scr.min()):
                step[0] = 1
                step[1] = 1
                step = step * np.sign(ratio)
                add(step)
            for _ in range(n_scr.max() - n_scr.min()):
                step[0] = 1
                step[1] = 1
                step = step * np.sign(ratio)
                step[np.where(n_scr == n_scr.min())] = 0
                add(step)
            sub = np.array([(np.abs(ratio[0]) % 1) * np.sign(ratio[0]), (np.abs(ratio[1]) % 1) * np.sign(ratio[1])])
            L.plan_buff = L.plan_buff + sub
            if np.abs(L.plan_buff[0]) >= 1 or np.abs(L.plan_buff[1]) >= 1:
                step[0] = 1 * np.sign(L.plan_buff[0])
                step[1] = 1 * np.sign(L.plan_buff[1])
                step[np.where(np.abs(L.plan_buff) < 1)] = 0
                add(step)
            L.plan_buff = np.array([(np.abs(L.plan_buff[0]) % 1) * np.sign(L.plan_buff[0]),
                                    (np.abs(L.plan_buff[1]) % 1) * np.sign(L.plan_buff[1])])
            moves.append(mv)
            buffs.append((float(L.plan_buff[0]), float(L.plan_buff[1])))
        self._plan_moves.append(moves)
        self._plan_buff.append(buffs)

    def _slot_count(self):
        s = 0
        for i, L in enumerate(self.layers):
            vx, vy, ratio = self._ratio(L, i)
            if vx == 0 and vy == 0:
                continue
            if getattr(L, 'plan_done_once', False):
                ratio = L.plan_ratio
            s = max(s, int(np.abs(ratio).max()) + 1)
        return s + (s % 2)

    def prepare(self, n_steps):
        """Plan the moves of the steps [0, n_steps) and put the plan on the GPU
        (a captured closed loop needs its whole horizon planned first)."""
        if self.hasNotBeenInitialized:
            raise OopaoError('The Atmosphere object needs to be initialised using the initialiseAtmosphere()')
        if not self.compute_covariance and self._slot_count() > 0:
            raise OopaoError('The computation of the covariance matrices was set to False in the atmosphere '
                             'initialisation. Set it to True to provide moving layers.')
        if self._slots is None:
            self._slots = self._slot_count()
        while len(self._plan_moves) < n_steps:
            self._plan_one()
        if self._dev_plan_len >= n_steps:
            return
        if self._frozen:
            raise OopaoError('the atmosphere plan is captured in a CUDA graph; plan the whole horizon before the '
                             'capture (ClosedLoop(max_steps=...))')
        T, Ln, S = len(self._plan_moves), self.nLayer, max(self._slots, 2)
        sched = np.zeros((T, Ln, S, 4), dtype=np.int32)
        buff = np.zeros((T, Ln, 2), dtype=np.float64)
        for t, (mv, bf) in enumerate(zip(self._plan_moves, self._plan_buff)):
            for l in range(Ln):
                if len(mv[l]) > self._slots:
                    raise OopaoError('more one-pixel moves in a step than planned slots')
                for s, (dx, dy, r) in enumerate(mv[l]):
                    sched[t, l, s] = (1, dx, dy, r)
                buff[t, l] = bf[l]
        d = self._dev
        self._sched_dev = torch.as_tensor(sched, device=d)
        self._buff_dev = torch.as_tensor(buff, device=d)
        nrm = np.array(self._normals) if self._normals else np.zeros((1, max(1, len(self._outer_idx))))
        self._normals_dev = torch.as_tensor(nrm, dtype=torch.float64, device=d)
        self._dev_plan_len = T

    # ------------------------------------------------------------------ device step
    def _scale(self):
        return torch.as_tensor([self.wavelength / 2 / np.pi * np.sqrt(f) for f in self.fractionalR0],
                               dtype=torch.float64, device=self._dev)

    def _launch(self, advance=True, moved=True, stream=None, boil=None):
        st = N.stream_handle(stream)
        res = self.telescope.resolution
        if boil is not None and moved:
            N.call('oopao_atm_boil', self._maps, self.nLayer, self._n, boil['phi'], len(boil['layers']),
                   boil['layers'], boil['alpha'], boil['beta'], self._step_dev if boil['by_step'] else None,
                   boil['steps'], self._err, st)
        if not moved:
            N.call('oopao_atm_update', self._maps, self._mirror, self.nLayer, self._n, 0, None, None, 0, None, None,
                   None, None, 0, 0, None, self._range, self._scale_dev, res, self._opd_dev, self._step_dev, 0,
                   self._err, st)
            return
        slots = self._slots if self._slots else 0
        if slots:
            slots = max(slots, 2)
        inner, outer = self._idx_dev
        N.call('oopao_atm_update', self._maps, self._mirror, self.nLayer, self._n, slots, self._sched_dev,
               self._buff_dev, self._dev_plan_len, self._A if slots else None, self._B if slots else None, inner, outer,
               len(self._inner_idx), len(self._outer_idx), self._normals_dev, self._range, self._scale_dev, res,
               self._opd_dev, self._step_dev, 1 if advance else 0, self._err, st)

    # ------------------------------------------------------------------ boiling
    def get_t_boiling(self, val):
        """One boiling time per layer, None for frozen flow (OOPAO/Atmosphere.py:376-385)."""
        if val is None:
            return [None] * self.nLayer
        if np.isscalar(val):
            return [val] * self.nLayer
        val = list(val)
        if len(val) != self.nLayer:
            raise OopaoError('Wrong value for t_boiling! Provide either a scalar '
                             '(applied to each layer) or a list with a value per layer.')
        return val

    def _boil_coefs(self):
        """(layer, alpha, beta) of the layers that boil at this sampling time:
        alpha = exp(-dt / t_boiling), beta = sqrt(1 - alpha^2); layers with
        no, a non-finite or a non-positive t_boiling, or with alpha >= 1 - 1e-6,
        stay frozen (``apply_boiling`` :387-398)."""
        out = []
        dt = self.telescope.samplingTime
        for i, t_b in enumerate(self._t_boiling):
            if t_b is None or not np.isfinite(t_b) or t_b <= 0:
                continue
            alpha = float(np.exp(-dt / t_b))
            if alpha >= 1.0 - 1e-6:
                continue
            out.append((i, alpha, float(np.sqrt(max(0.0, 1.0 - alpha ** 2)))))
        return out

    def _boil_screen(self, i, seed):
        gen = ft_sh_phase_screen if self.mode == 2 else ft_phase_screen
        L = self.layers[i]
        return gen(self._r0, self._L0, self._n, L.D / L.resolution, seed=seed)

    def _boil_table(self, coefs, phi, by_step):
        """by_step: phi holds the screens of the steps [0, n) picked by the
        device step counter; otherwise the one step of an eager update."""
        return dict(phi=phi, steps=phi.shape[0], by_step=by_step, layers=N.host([c[0] for c in coefs], np.int32),
                    alpha=N.host([c[1] for c in coefs], np.float64), beta=N.host([c[2] for c in coefs], np.float64))

    def _boil_now(self):
        """The boiling of one eager update: each boiling layer's seed counter
        moves on and a new screen of the map's size is drawn with it on the
        host, as the reference does, then blended on the GPU."""
        coefs = self._boil_coefs()
        if not coefs:
            return None
        phi = np.empty((1, len(coefs), self._n, self._n))
        for k, (i, _, _) in enumerate(coefs):
            self.layers[i].boiling_seed += 1
            phi[0, k] = self._boil_screen(i, self.layers[i].boiling_seed)
        return self._boil_table(coefs, torch.as_tensor(phi, device=self._dev), False)

    def boiling_horizon(self, n_steps):
        """The boiling screens of the steps [0, n_steps) after the last
        generateNewPhaseScreen, on the GPU ([n_steps][boiling layers][n][n]
        float64), for a captured closed loop whose device step counter picks
        the step's screens: step t of layer i uses the seed
        100000 + seed + 100000 i + t + 1, as t + 1 eager updates would.  None
        when no layer boils."""
        coefs = self._boil_coefs()
        if not coefs:
            return None
        nbytes = n_steps * len(coefs) * self._n * self._n * 8
        free = torch.cuda.mem_get_info(self._dev)[0]
        if nbytes > 0.5 * free:
            raise OopaoError('the boiling screens of %d steps need %.1f GB on the GPU (%.1f GB free); plan fewer '
                             'steps' % (n_steps, nbytes / 1e9, free / 1e9))
        phi = torch.empty((n_steps, len(coefs), self._n, self._n), dtype=torch.float64, device=self._dev)
        for k, (i, _, _) in enumerate(coefs):
            base = 100000 + self._seed + i * 100000
            host = np.empty((n_steps, self._n, self._n))
            for t in range(n_steps):
                host[t] = self._boil_screen(i, base + t + 1)
            phi[:, k].copy_(torch.as_tensor(host))
        return self._boil_table(coefs, phi, True)

    def reset_state(self):
        """Back to the screens of the last generateNewPhaseScreen (same plan)."""
        self._maps[0].copy_(self._maps0)
        for i, L in enumerate(self.layers):
            L.boiling_seed = 100000 + self._seed + i * 100000
        self._step_dev.zero_()
        self._step = 0
        self._err.zero_()
        self._launch(advance=False, moved=False)

    def status(self):
        """0, or 1 when a step outside the planned horizon was requested."""
        return int(self._err.item())

    def update(self, OPD=None):
        """One step of frozen flow for every layer (OOPAO/Atmosphere.py:516-531)."""
        if self.hasNotBeenInitialized:
            raise OopaoError('The Atmosphere object needs to be initialised using the initialiseAtmosphere()')
        if OPD is not None:
            self.user_defined_opd = np.asarray(OPD)
            return
        self.user_defined_opd = None
        need = self._step + 1
        if self._dev_plan_len < need:
            self.prepare(max(need, 2 * max(self._dev_plan_len, 16)))
        boil = self._boil_now()
        self._launch(advance=True, boil=boil)
        self._step += 1

    # ------------------------------------------------------------------ outputs
    @property
    def OPD(self):
        if self.user_defined_opd is not None:
            return self.user_defined_opd
        return self._opd_dev.double().cpu().numpy()

    @property
    def OPD_no_pupil(self):
        return self.OPD

    def device_opd(self):
        return self._opd_dev

    def relay(self, src):
        if src.tag != 'source':
            raise OopaoError('oopao_gb300 Atmosphere propagates a single on-axis Source')
        if np.asarray(getattr(src, 'coordinates', [0, 0]))[0] != 0:
            raise OopaoError('oopao_gb300 Atmosphere supports an on-axis source only')
        src.optical_path.append([self.tag, self])
        if self.user_defined_opd is not None:
            warning('User-Defined OPD are only propagated once in the Atmosphere class.')
            src.OPD_no_pupil = np.array(self.user_defined_opd)
            self.user_defined_opd = None
            return
        src._set_device_opd(self._opd_dev.clone())

    # ------------------------------------------------------------------ setters
    @property
    def r0(self):
        return self._r0

    @r0.setter
    def r0(self, val):
        """Rescales B to the new r0 (OOPAO/Atmosphere.py:1017-1035); the screens
        keep their statistics until regenerated."""
        self._r0 = val
        self.seeingArcsec = self.rad2arcsec * (self.wavelength / val)
        self.cn2 = (val ** (-5. / 3) / (0.423 * (2 * np.pi / self.wavelength) ** 2)) / np.max([1, np.max(self.altitude)])
        if not self.hasNotBeenInitialized and self.compute_covariance:
            self._set_matrices()

    @property
    def L0(self):
        return self._L0

    @L0.setter
    def L0(self, val):
        self._L0 = val
        if not self.hasNotBeenInitialized:
            self.hasNotBeenInitialized = True
            self.initializeAtmosphere(self.telescope)

    @property
    def windSpeed(self):
        return self._windSpeed

    @windSpeed.setter
    def windSpeed(self, val):
        """As the reference, a layer's velocity in pixels per step is fixed by
        its first update; later changes apply after generateNewPhaseScreen."""
        if len(val) != self.nLayer:
            raise OopaoError('Wrong value for the wind-speed! Make sure that you inpute a wind-speed for each layer')
        self._windSpeed = list(val)

    @property
    def t_boiling(self):
        return self._t_boiling

    @t_boiling.setter
    def t_boiling(self, val):
        """Boiling times, applied from the next update on (OOPAO/Atmosphere.py:1104-1115)."""
        self._t_boiling = self.get_t_boiling(val)

    @property
    def windDirection(self):
        return self._windDirection

    @windDirection.setter
    def windDirection(self, val):
        if len(val) != self.nLayer:
            raise OopaoError('Wrong value for the wind-direction! Make sure that you inpute a wind-direction for '
                             'each layer')
        self._windDirection = list(val)

    def __repr__(self):
        return 'Atmosphere(%d layers, r0=%.3f m, L0=%.1f m, res=%d, %s)' % (
            self.nLayer, self._r0, self._L0, self.telescope.resolution,
            'initialised' if not self.hasNotBeenInitialized else 'not initialised')
