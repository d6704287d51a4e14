"""Closed-loop AO step on the GPU, captured in a CUDA graph.

One step follows ``tutorials/AO_closed_loop_Pyramid_WFS.py:601-639`` and
``OOPAO/closed_loop/run_cl.py:176-217``:

    turbulence OPD of the step  ->  + DM shape (modes @ coefs)
    ->  modulated pyramid frame  ->  slopes
    ->  coefs -= gain * reconstructor @ slopes       (frame delay 1 or 2)
    + residual wavefront RMS over the pupil (logged on the device)
    + optionally the science PSF of the residual, summed into a long-exposure
      image (``Telescope.computePSF`` with zero padding 2,
      ``OOPAO/Telescope.py:251-420``; FFT by cuFFT through torch, a
      diagnostic outside the WFS path), and its Strehl ratio by the OTF ratio
      of ``strehlMeter`` (``OOPAO/tools/tools.py:102-157``)

Every operation is a launch of ``liboopao_gb300`` on preallocated buffers; a
device step counter carries the time index, so the captured graph is
replayed as is for every later step (``ClosedLoop.run``).  The loop takes the
sensor's plan (mask, modulation path, weights of a single-wavefront
measurement), its valid pixels and reference slopes, and the DM's projection
path when it is built: a change to any of them afterwards (a new mask,
modulation, pupil shift or calibration) needs a new ClosedLoop.

The turbulence is either the reference's infinite phase screens
(``oopao_gb300.Atmosphere``, updated on the device inside the captured step)
or a set of periodic von Karman layers translated by frozen flow
(``VonKarmanLayers``, a lighter stand-in).

With a calibrated ``GainSensingCamera`` the loop follows the reference's GSC
tutorial (``tutorials/AO_closed_loop_Pyramid_WFS_GSC.py``): every step also
forms the full-resolution focal-plane (modulation) camera frame, computes the
optical gains from it and, from step ``og_start`` on, applies
coefs -= gain * M2C @ diag(1/og) @ M @ s with the modal reconstructor M.
"""
import numpy as np
import torch

from . import _native as N
from .tools import OopaoError


class VonKarmanLayers:
    """Periodic von Karman OPD layers (FFT method: white Gaussian noise
    filtered by the von Karman phase spectrum 0.023 r0^-5/3 (f^2 + L0^-2)^-11/6,
    seeded), with frozen-flow velocities in pixels per loop step."""

    def __init__(self, tel, r0, L0, fractionalR0=(1.0,), windSpeed=(10.,), windDirection=(0.,),
                 wavelength=500e-9, size_factor=4, seed=0):
        res = tel.resolution
        n = 1
        while n < size_factor * res:
            n *= 2
        dx = tel.D / res
        rng = np.random.default_rng(seed)
        f = np.fft.fftfreq(n, d=dx)
        fx, fy = np.meshgrid(f, f)
        f2 = fx ** 2 + fy ** 2
        self.screens, self.vy, self.vx = [], [], []
        self.size = n
        df = 1.0 / (n * dx)
        for q, frac in enumerate(fractionalR0):
            r0l = r0 * frac ** (-3.0 / 5.0)
            psd = 0.023 * r0l ** (-5.0 / 3.0) * (f2 + 1.0 / L0 ** 2) ** (-11.0 / 6.0)
            psd[0, 0] = 0.0
            noise = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
            phase = np.real(np.fft.ifft2(noise * np.sqrt(psd) * df)) * n * n
            self.screens.append((phase * wavelength / (2 * np.pi)).astype(np.float32))
            v = windSpeed[q] * tel.samplingTime / dx
            ang = np.deg2rad(windDirection[q])
            self.vy.append(v * np.sin(ang))
            self.vx.append(v * np.cos(ang))

    def origin(self, res):
        """Screen pixel under pupil pixel (0, 0) at step 0 (the screen centre)."""
        return (self.size - res) / 2.0

    def opd(self, step, res):
        """Host evaluation of the layers at a step (bilinear, periodic), float64."""
        out = np.zeros((res, res))
        o = self.origin(res)
        ii, jj = np.meshgrid(np.arange(res), np.arange(res), indexing='ij')
        for s, vy, vx in zip(self.screens, self.vy, self.vx):
            n = s.shape[0]
            y = o + ii + vy * step
            x = o + jj + vx * step
            y0, x0 = np.floor(y), np.floor(x)
            dy, dx = y - y0, x - x0
            y0, x0 = y0.astype(int) % n, x0.astype(int) % n
            y1, x1 = (y0 + 1) % n, (x0 + 1) % n
            s64 = s.astype(np.float64)
            out += (1 - dy) * ((1 - dx) * s64[y0, x0] + dx * s64[y0, x1]) + \
                dy * ((1 - dx) * s64[y1, x0] + dx * s64[y1, x1])
        return out


def strehl_meter(psf, psf_ref):
    """Strehl ratio in percent from a focal-plane image and the image of a
    flat wavefront of the same sampling: ratio of the sums of the
    max-normalised OTF moduli (``strehlMeter``, OOPAO/tools/tools.py:102-157)."""
    psf = np.asarray(psf, dtype=np.float64)
    psf_ref = np.asarray(psf_ref, dtype=np.float64)
    if psf.shape != psf_ref.shape:
        raise OopaoError('strehl_meter: PSF and reference PSF must have the same shape')
    otf = np.abs(np.fft.fftshift(np.fft.fft2(psf)))
    otfa = np.abs(np.fft.fftshift(np.fft.fft2(psf_ref)))
    return float(np.sum(otf / otf.max()) / np.sum(otfa / otfa.max()) * 100)


class ClosedLoop:
    """reconstructor: [nValidAct, nSignal] (M2C @ M), or, with ``gsc``, the
    modal reconstructor M [n_modes, nSignal] and ``M2C`` [nValidAct, n_modes]."""

    def __init__(self, tel, ngs, dm, wfs, reconstructor, gain=0.4, frame_delay=1, layers=None,
                 max_steps=100000, science=False, gsc=None, M2C=None, og_start=0):
        if frame_delay not in (1, 2):
            raise OopaoError('frame_delay must be 1 or 2')
        if not wfs.cam._is_plain():
            raise OopaoError('the captured loop reads the noise-free sensor frame: its camera must have the '
                             'default Detector settings (no noise, integration time, ADC or background; QE 1, '
                             'gain 1)')
        self.tel, self.ngs, self.dm, self.wfs = tel, ngs, dm, wfs
        self.dev = wfs._dev
        self.gain = float(gain)
        self.frame_delay = frame_delay
        res = tel.resolution
        self.res = res
        d = self.dev
        self.gsc = gsc
        if gsc is not None:
            if M2C is None:
                raise OopaoError('optical-gain compensation needs M2C and the modal reconstructor M')
            Mr = np.asarray(reconstructor, dtype=np.float32)
            m2c = np.asarray(M2C, dtype=np.float32)
            if Mr.shape != (gsc.n_modes, wfs.nSignal) or m2c.shape != (dm.nValidAct, gsc.n_modes):
                raise OopaoError('with gsc: reconstructor [n_modes, nSignal] and M2C [nValidAct, n_modes]')
            if not gsc.calibration_ready:
                raise OopaoError('the GainSensingCamera must be calibrated first')
            if gsc.n != wfs.resolution:
                raise OopaoError('the GainSensingCamera mask must be the pyramid mask (N x N)')
            if not wfs.psfCentering and wfs.spatialFilter is not None:
                raise OopaoError('optical-gain compensation in the loop takes a pyramid without spatial filter '
                                 'in the 1-pixel-centred branch')
            self.M = torch.as_tensor(np.ascontiguousarray(Mr), device=d)
            self.R = torch.as_tensor(np.ascontiguousarray(m2c), device=d)   # M2C
            self.y = torch.zeros(gsc.n_modes, dtype=torch.float32, device=d)
            self.og = torch.ones((1, gsc.n_modes), dtype=torch.float64, device=d)
            self.focal = torch.zeros((1, wfs.resolution, wfs.resolution), dtype=torch.float32, device=d)
            self.og_start = int(og_start)
            self._gsc_nb = N.load().oopao_gsc_workspace_bytes(gsc._plan, 1)
            self._gsc_ws = torch.empty(self._gsc_nb, dtype=torch.uint8, device=d)
        else:
            R = np.asarray(reconstructor, dtype=np.float32)
            if R.shape != (dm.nValidAct, wfs.nSignal):
                raise OopaoError('reconstructor must be [nValidAct, nSignal]')
            self.R = torch.as_tensor(np.ascontiguousarray(R), device=d)
        self.coefs = torch.zeros(dm.nValidAct, dtype=torch.float32, device=d)
        self.step_counter = torch.zeros(1, dtype=torch.int32, device=d)
        self.opd_atm = torch.zeros((1, res, res), dtype=torch.float32, device=d)
        self.opd = torch.zeros((1, res, res), dtype=torch.float32, device=d)
        cam = wfs._cam_eff
        self.frame = torch.zeros((1, cam, cam), dtype=torch.float32, device=d)
        self.s2d = torch.zeros((1, wfs.validSignal.size), dtype=torch.float32, device=d)
        self.s = torch.zeros((1, wfs.nSignal), dtype=torch.float32, device=d)
        self.s_prev = torch.zeros_like(self.s)
        self.max_steps = max_steps
        self.wfe = torch.zeros(max_steps, dtype=torch.float32, device=d)
        idx = np.flatnonzero(tel.pupil.reshape(-1)).astype(np.int32)
        self.pupil_idx = torch.as_tensor(idx, device=d)
        self.scale = 2 * np.pi / ngs.wavelength
        # static configuration: amplitude, signal processing, workspace
        ngs ** tel
        # one wavefront per step: the weights of a single measurement apply
        plan = wfs._weighted_plan(True) if hasattr(wfs, '_weighted_plan') else wfs.plan
        plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
        wfs._configure_signal(plan)
        self.plan = plan
        self.ws_bytes = plan.workspace_bytes(1)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=d)
        self.layers = layers
        self._atm = None
        self._boil = None
        if layers is not None and hasattr(layers, 'prepare'):
            # infinite-screen Atmosphere: plan the whole horizon, then its
            # device update is one more part of the captured step
            self._atm = layers
            layers.reset_state()
            layers.prepare(max_steps + 2)
            # boiling layers: every step's new screens drawn up front, the
            # device step counter picks them inside the graph
            self._boil = layers.boiling_horizon(max_steps + 2)
            layers._launch(advance=True, boil=self._boil)   # the first step's turbulence (one update)
            self._atm_opd = layers.device_opd().view(1, res, res)
        elif layers is not None:
            self._scr = [torch.as_tensor(s, device=d) for s in layers.screens]
            nl = len(self._scr)
            self._scr_ptr = (N.c_void_p * nl)(*[t.data_ptr() for t in self._scr])
            self._h = (N.ctypes.c_int * nl)(*[t.shape[0] for t in self._scr])
            self._w = (N.ctypes.c_int * nl)(*[t.shape[1] for t in self._scr])
            c = np.array([layers.origin(res)] * nl, np.float32)
            self._y0 = (N.ctypes.c_float * nl)(*c)
            self._x0 = (N.ctypes.c_float * nl)(*c)
            self._vy = (N.ctypes.c_float * nl)(*np.float32(layers.vy))
            self._vx = (N.ctypes.c_float * nl)(*np.float32(layers.vx))
        # the loop owns its projection workspace: the graph keeps its address
        nb = dm.projection_workspace_bytes(1)
        self._dm_ws = torch.zeros(nb, dtype=torch.uint8, device=d) if nb else None
        self._tc_ws = self._dm_ws if dm.projection_path() == 'bf16' else None
        self.science = bool(science)
        if self.science:
            # science camera of the NGS: zero padding 2 (N = 2 res), centring
            # phasor exp(-i pi (N+1)/N (x+y)), EMF = fft2(E * phasor) / N
            n2 = 2 * res
            lo = (n2 - res) // 2
            xx, yy = np.meshgrid(np.arange(n2), np.arange(n2))
            ph = np.exp(-1j * np.pi * (n2 + 1) / n2 * (xx + yy))[lo:lo + res, lo:lo + res]
            amp = np.sqrt(ngs.intensity) * tel.pupil
            self._sci_field0 = torch.as_tensor((amp * ph / n2).astype(np.complex64), device=d)
            self._sci_pad = torch.zeros((n2, n2), dtype=torch.complex64, device=d)
            self._sci_lo = lo
            self.psf_le = torch.zeros((n2, n2), dtype=torch.float64, device=d)
            self._sci_pad[lo:lo + res, lo:lo + res] = self._sci_field0
            f = torch.fft.fft2(self._sci_pad)
            self.psf_ref = (f.real.double() ** 2 + f.imag.double() ** 2).cpu().numpy()
            self._sci_pad.zero_()
        self.graph = None
        self._side = torch.cuda.Stream(device=d)

    def reset(self):
        self.coefs.zero_()
        if self.gsc is not None:
            self.og.fill_(1.0)
        self.step_counter.zero_()
        self.s_prev.zero_()
        self.wfe.zero_()
        if self.science:
            self.psf_le.zero_()
        if self._atm is not None:
            # step t sees the atmosphere after t + 1 updates (the reference
            # tutorial updates it first in every iteration); each step then
            # prepares the next step's turbulence while the sensor runs
            self._atm.reset_state()
            self._atm._launch(advance=True, boil=self._boil)

    def _science(self):
        lo, res = self._sci_lo, self.res
        e = self._sci_field0 * torch.exp(1j * (self.scale * self.opd[0]))
        self._sci_pad[lo:lo + res, lo:lo + res] = e
        f = torch.fft.fft2(self._sci_pad)
        self.psf_le += f.real.double() ** 2 + f.imag.double() ** 2

    def long_exposure_psf(self):
        """Sum of the science PSFs of the steps run since the last reset."""
        if not self.science:
            raise OopaoError('ClosedLoop(science=True) is needed for the science PSF')
        return self.psf_le.cpu().numpy()

    def long_exposure_strehl(self):
        """Strehl ratio (percent) of the long-exposure PSF."""
        return strehl_meter(self.long_exposure_psf(), self.psf_ref)

    def _launch_step(self):
        """One step.  With the infinite-screen Atmosphere, the next step's
        turbulence, this step's pupil RMS and the optional science PSF run on
        a side stream while the sensor runs; the integrator (which advances
        the step counter) waits for them."""
        main = torch.cuda.current_stream()
        st = N.stream_handle(main)
        dm, wfs = self.dm, self.wfs
        base = None
        if self._atm is not None:
            base = self._atm_opd                 # prepared by the previous step (or reset)
        elif self.layers is not None:
            N.call('oopao_cl_screen', len(self._scr), self._scr_ptr, self._h, self._w, self._y0, self._x0,
                   self._vy, self._vx, self.res, self.step_counter, self.opd_atm, st)
            base = self.opd_atm
        dm._launch_projection(self.coefs, 1, 1.0, base, self.opd, st, ws=self._dm_ws)
        fork = torch.cuda.Event()
        fork.record(main)
        side = self._side
        side.wait_event(fork)
        with torch.cuda.stream(side):
            ss = N.stream_handle(side)
            if self._atm is not None:
                self._atm._launch(advance=True, stream=side, boil=self._boil)
            N.call('oopao_cl_pupil_rms', self.opd, self.pupil_idx, self.pupil_idx.numel(), self.step_counter,
                   self.wfe, self.max_steps, ss)
            if self.science:
                self._science()
        join = torch.cuda.Event()
        join.record(side)
        if self.gsc is not None:
            # frame + full-resolution focal-plane camera, then the optical gains
            N.call('oopao_pwfs_measure_focal', self.plan.h, self.opd, self.scale, 1, self.frame, None, self.focal,
                   self.ws, self.ws_bytes, st)
            N.call('oopao_gsc_optical_gains', self.gsc._plan, self.focal, 1, self.og, None, None, self._gsc_ws,
                   self._gsc_nb, st)
        else:
            N.call('oopao_pwfs_measure', self.plan.h, self.opd, self.scale, 1, self.frame, None, self.ws,
                   self.ws_bytes, st)
        N.call('oopao_pwfs_signal', self.plan.h, self.frame, 1, self.s2d, self.s, None, st)
        main.wait_event(join)
        if self.gsc is not None:
            s_in = self.s if self.frame_delay == 1 else self.s_prev
            N.call('oopao_cl_modal', self.M, s_in, self.M.shape[0], self.M.shape[1], self.og, self.og_start,
                   self.step_counter, self.y, st)
            N.call('oopao_cl_integrate', self.R, self.y, self.R.shape[0], self.R.shape[1], self.gain, self.coefs,
                   self.step_counter, st)
            if self.frame_delay == 2:
                self.s_prev.copy_(self.s)
        elif self.frame_delay == 1:
            N.call('oopao_cl_integrate', self.R, self.s, self.R.shape[0], self.R.shape[1], self.gain, self.coefs,
                   self.step_counter, st)
        else:
            N.call('oopao_cl_integrate', self.R, self.s_prev, self.R.shape[0], self.R.shape[1], self.gain,
                   self.coefs, self.step_counter, st)
            self.s_prev.copy_(self.s)

    def step(self):
        """One eager step (no graph)."""
        self._launch_step()

    def capture(self):
        """Capture one step in a CUDA graph (after eager warm-up steps)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(2):
                self._launch_step()
        torch.cuda.current_stream().wait_stream(s)
        self.reset()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._launch_step()
        self.graph = g
        if self._atm is not None:
            self._atm._frozen = True
        self.reset()
        torch.cuda.synchronize()
        return g

    def run(self, n_steps, graph=True):
        """Run n steps (graph replay when captured)."""
        if graph and self.graph is None:
            self.capture()
        for _ in range(n_steps):
            if graph:
                self.graph.replay()
            else:
                self._launch_step()

    @property
    def residual_wfe(self):
        """Residual RMS OPD over the pupil per step so far (m), host copy."""
        n = int(self.step_counter.item())
        return self.wfe[:n].double().cpu().numpy()
