"""WFS and focal-plane camera: drop-in for the reference ``Detector``
(``OOPAO/Detector.py``).

The sensor kernels write noise-free, sum-binned frames on the device; the
camera applies the reference's integrate/readout chain to them there
(``OOPAO/Detector.py:273-354``), in the reference's order:

* integrate, once per loop step: photon noise, background noise, quantum
  efficiency; the frame joins the integration buffer;
* readout, once the integration time is reached (every step when it is
  None): sum of the buffer, dark-current shot noise, full-well saturation,
  EMCCD amplification, detector binning, readout noise, CCD/CMOS gain, ADC
  digitisation, log scale, cast to the output precision, background-map
  removal.

Between two readouts the camera keeps showing the last frame read out, and
the sensor computes its signals from that frame, as the reference's does.
Noise is drawn with torch's device generator (``generator``); the reference
seeds numpy from the wall clock, so noisy frames match it statistically, not
bit for bit.  The stages without random draws run in the library's readout
kernels (``oopao_det_saturate``, ``oopao_det_readout_tail``).  Frames stay
float32 on the device; an unsigned output precision is held as its integer
values.
"""
import numpy as np
import torch

from . import _native as N
from .tools import OopaoError, set_binning, warning

_UNSIGNED_BITS = {np.dtype(np.uint8): 8, np.dtype(np.uint16): 16, np.dtype(np.uint32): 32,
                  np.dtype(np.uint64): 64}


def _bin_sum(f, b):
    """tools.set_binning(..., mode='sum') of [R, n, n] frames (OOPAO/tools/tools.py:464-483)."""
    n = f.shape[-1]
    if n % b != 0:
        raise ValueError('Binning factor %d not compatible with the array size' % b)
    m = int(np.round(n / b))
    return f.reshape(f.shape[0], m, n // m, m, n // m).sum(dim=(2, 4))


class Detector:
    def __init__(self, nRes: int = None, integrationTime: float = None, bits: int = None,
                 output_precision: int = None, FWC: int = None, gain: int = 1, sensor: str = 'CCD',
                 QE: float = 1., binning: int = 1, psf_sampling: float = 2., darkCurrent: float = 0.,
                 readoutNoise: float = 0, photonNoise: bool = False, backgroundNoise: bool = False,
                 backgroundFlux: float = None, backgroundMap: float = None, log_scale: bool = False):
        if sensor not in ['EMCCD', 'CCD', 'CMOS']:
            raise OopaoError("Sensor must be 'EMCCD', 'CCD', or 'CMOS'")
        self.resolution = nRes
        self.bits = bits
        self.output_precision = output_precision
        self.FWC = FWC
        self.gain = gain
        self.sensor = sensor
        self.QE = QE
        self.binning = binning
        self.psf_sampling = psf_sampling
        self.darkCurrent = darkCurrent
        self.readoutNoise = readoutNoise
        self.photonNoise = photonNoise
        self.backgroundFlux = backgroundFlux
        self.backgroundMap = backgroundMap
        self.log_scale = log_scale
        self.tag = 'detector'
        self.saturation = 0
        self.quantification_noise = 0
        self.dark_shot_noise = 0
        self._photon_noise = 0
        self.fov_arcsec = None
        self.pixel_size_rad = None
        self.pixel_size_arcsec = None
        self.is_focal_plane_camera = False
        self._frame_dev = None
        self._frame_host = np.zeros([nRes, nRes]) if nRes is not None else None
        self._perfect_dev = None
        self._perfect_host = None
        self.generator = None
        self.buffer_frame = []
        self._integrated_time = 0
        self.integrationTime = integrationTime
        self.backgroundNoise = backgroundNoise

    # ------------------------------------------------------------------ settings
    @property
    def integrationTime(self):
        return self._integrationTime

    @integrationTime.setter
    def integrationTime(self, val):
        """Setting it restarts the integration (OOPAO/Detector.py:414-419)."""
        self._integrationTime = val
        self._integrated_time = 0
        self.buffer_frame = []

    @property
    def backgroundNoise(self):
        return self._backgroundNoise

    @backgroundNoise.setter
    def backgroundNoise(self, val):
        self._backgroundNoise = val
        if val is True and self.backgroundFlux is None:
            shape = None if self._frame_host is None else self._frame_host.shape
            warning('The background noise is enabled but no property backgroundFlux is set.\nA map of shape ' +
                    str(shape) + ' is expected')

    def _out_kind(self):
        """set_output_precision (OOPAO/Detector.py:192-213): (unsigned bits or 0,
        signed-integer output, ADC clips at 0)."""
        prec = self.output_precision
        if prec is None:
            bits = self.bits if self.bits in (8, 16, 32, 64) else 0
            return bits, False, bits != 0
        dt = np.dtype(prec)
        ub = _UNSIGNED_BITS.get(dt, 0)
        return ub, np.issubdtype(dt, np.signedinteger), ub != 0

    def _is_plain(self):
        return (self.integrationTime is None and self.bits is None and self.FWC is None and self.darkCurrent == 0
                and not self.backgroundNoise and self.backgroundMap is None and not self.log_scale
                and self.sensor != 'EMCCD' and self.binning == 1 and self.output_precision is None
                and not self.photonNoise and self.readoutNoise == 0 and self.QE == 1 and self.gain == 1)

    # ------------------------------------------------------------------ integrate / readout
    def _integrate_device(self, frame_dev, dt=None, wfs=True):
        """integrate() and readout() (OOPAO/Detector.py:273-354) of device
        frames [B, n, n], one loop step each, in order.  dt: loop sampling
        time added to the integrated time before each step (None when the
        caller has added it already).  Returns the camera frame after each
        step [B, n', n']: the frame of that step's readout, or the last frame
        read out while an integration is running."""
        if wfs and self.binning != 1:
            raise OopaoError('The sensor camera bins through the sensor (binning= of the WFS); '
                             'its Detector.binning must be 1')
        f = frame_dev if frame_dev.ndim == 3 else frame_dev[None]
        self._perfect_dev, self._perfect_host = f[-1], None
        if self.photonNoise:
            f = torch.poisson(f.clamp_min(0), generator=self.generator)
        if self.backgroundNoise:
            if self.backgroundFlux is None:
                raise OopaoError('The background map backgroundFlux is not properly set. A map of shape ' +
                                 str(tuple(f.shape[1:])) + ' is expected')
            lam = torch.as_tensor(np.array(np.broadcast_to(
                np.asarray(self.backgroundFlux, dtype=np.float32), tuple(f.shape[1:]))), device=f.device)
            f = f + torch.poisson(lam.expand(f.shape).contiguous(), generator=self.generator)
        if self.QE != 1:
            f = f * self.QE
        if self.integrationTime is None:
            out = self._readout(f)
            self._set_device_frame(out)
            return out
        cur = self._current_frame(f)
        outs = []
        for i in range(f.shape[0]):
            if dt is not None:
                self._integrated_time += dt
            self.buffer_frame.append(f[i])
            if self._integrated_time >= self.integrationTime:
                cur = self._readout(torch.stack(self.buffer_frame).sum(dim=0)[None])[0]
                self.buffer_frame = []
                self._integrated_time = 0
            outs.append(cur)
        out = torch.stack(outs)
        self._set_device_frame(out)
        return out

    def _current_frame(self, f):
        """The frame the camera shows before the running integration ends."""
        if self._frame_dev is not None:
            t = self._frame_dev
            return t[-1] if t.ndim == 3 else t
        shape = f.shape[1:] if self.binning == 1 else (f.shape[1] // self.binning ** 2,) * 2
        if self._frame_host is not None and tuple(self._frame_host.shape) == tuple(shape):
            return torch.as_tensor(np.ascontiguousarray(self._frame_host, dtype=np.float32), device=f.device)
        return torch.zeros(shape, dtype=torch.float32, device=f.device)

    def _readout(self, f):
        """readout() (OOPAO/Detector.py:273-329) of integrated frames [R, n, n]."""
        R = f.shape[0]
        out_bits, signed_int, clip_zero = self._out_kind()
        bg = None
        if self.backgroundMap is not None:
            n_out = f.shape[-1] // self.binning ** 2 if self.binning != 1 else f.shape[-1]
            try:
                if out_bits or signed_int:
                    # an integer frame cannot take the float map in place
                    raise TypeError
                bg = np.broadcast_to(np.asarray(self.backgroundMap, dtype=np.float32), (n_out, n_out))
            except (TypeError, ValueError):
                raise OopaoError('The shape of the backgroung map does not match the detector frame resolution')
            bg = torch.as_tensor(np.array(bg), device=f.device)
        if self.darkCurrent != 0:
            if self.integrationTime is None:
                raise OopaoError('A dark current needs the Detector integrationTime: its shot noise is drawn for '
                                 'darkCurrent * integrationTime electrons')
            self.dark_shot_noise = np.sqrt(self.darkCurrent * self.integrationTime)
            lam = torch.full(f.shape, float(self.darkCurrent * self.integrationTime), device=f.device)
            f = f + torch.poisson(lam, generator=self.generator)
        if self.FWC is not None:
            # the kernels rewrite the frames in place: never the caller's tensor
            f = f.to(torch.float32, copy=True).contiguous()
            mx = torch.empty(R, dtype=torch.float32, device=f.device)
            N.call('oopao_det_saturate', N.ptr(f), R, f[0].numel(), float(self.FWC), N.ptr(mx), N.stream_handle())
            mx = mx.cpu().numpy()
            self.saturation = 100 * float(mx[-1]) / self.FWC
            if mx.max() > self.FWC:
                warning('The detector is saturating, %.1f %%' % self.saturation)
        if self.sensor == 'EMCCD':
            f = torch.poisson(f.clamp_min(0), generator=self.generator) * self.gain
        if self.binning != 1:
            # the reference applies the hardware binning twice (OOPAO/Detector.py:290-297)
            f = _bin_sum(_bin_sum(f, self.binning), self.binning)
        self.clip_unsigned = 0 if clip_zero else -np.inf
        if self.readoutNoise != 0:
            f = f + torch.round(torch.randn(f.shape, device=f.device, generator=self.generator) * self.readoutNoise)
        gain = self.gain if self.sensor in ('CCD', 'CMOS') else 1
        bits = int(self.bits) if self.bits is not None else 0
        if gain != 1 or bits or self.log_scale or out_bits or bg is not None:
            f = f.to(torch.float32, copy=True).contiguous()
            adc = bits and self.FWC is not None
            mx = torch.empty(R, dtype=torch.float32, device=f.device) if adc else None
            N.call('oopao_det_readout_tail', N.ptr(f), R, f[0].numel(), float(gain), bits,
                   float(self.FWC) if self.FWC is not None else 0.0, int(clip_zero), int(bool(self.log_scale)),
                   out_bits, N.ptr(bg), N.ptr(mx), N.stream_handle())
            if adc:
                self.quantification_noise = self.FWC * 2 ** (-bits) / np.sqrt(12)
                mx = mx.cpu().numpy()
                self.saturation = 100 * float(mx[-1]) / self.FWC
                if mx.max() > self.FWC:
                    warning('The ADC is saturating (gain applyed %i), %.1f %%' % (self.gain, self.saturation))
        if signed_int:
            f = torch.trunc(f)
        if self.resolution is None:
            self.resolution = f.shape[-1] * self.binning
        if self.fov_arcsec is not None:
            self.pixel_size_rad = self.fov_rad / self.resolution * self.binning
            self.pixel_size_arcsec = self.fov_arcsec / self.resolution * self.binning
        return f

    def integrate(self, frame):
        """``Detector.integrate`` + ``readout`` (OOPAO/Detector.py:331-354) for a
        frame computed outside the sensor camera path (the focal-plane
        camera): the frame is kept as ``perfect_frame``, then the camera chain
        applies.  The caller has added the loop step to the integrated time,
        as the reference's callers do.  A device tensor stays on the device."""
        if isinstance(frame, torch.Tensor):
            t = frame.to(torch.float32)
            self._set_device_frame(self._integrate_device(t[None], wfs=False))
            self._perfect_dev, self._perfect_host = t, None
            return
        host = np.array(frame, dtype=np.float64)
        if self._is_plain():
            self._perfect_dev, self._perfect_host = None, host
            self.frame = host.copy()
            return
        dev = torch.device('cuda', torch.cuda.current_device())
        t = torch.as_tensor(np.ascontiguousarray(host, dtype=np.float32), device=dev)
        self._set_device_frame(self._integrate_device(t[None], wfs=False))
        self._perfect_dev, self._perfect_host = None, host

    # ------------------------------------------------------------------ frames
    @property
    def perfect_frame(self):
        if self._perfect_host is None and self._perfect_dev is not None:
            self._perfect_host = self._perfect_dev.detach().to('cpu', torch.float64).numpy()
        return self._perfect_host

    @property
    def flux_max_px(self):
        p = self.perfect_frame
        return None if p is None else float(p.max())

    @property
    def signal(self):
        m = self.flux_max_px
        return None if m is None else self.QE * m

    @property
    def photon_noise(self):
        """sqrt(QE * brightest pixel) once photon noise is on (set_photon_noise, :240-242)."""
        if self.photonNoise and self.signal is not None:
            return np.sqrt(self.signal)
        return self._photon_noise

    @property
    def device_frame(self):
        """The frame as a float32 device tensor ([cam, cam], or [B, cam, cam])."""
        if self._frame_dev is not None:
            t = self._frame_dev
            return t[0] if t.ndim == 3 and t.shape[0] == 1 else t
        if self._frame_host is None:
            return None
        return torch.as_tensor(np.ascontiguousarray(self._frame_host, dtype=np.float32),
                               device=torch.device('cuda', torch.cuda.current_device()))

    def _set_device_frame(self, t):
        self._frame_dev = t
        self._frame_host = None

    @property
    def frame(self):
        """The last camera frame, float64 [cam, cam].  After a batch of
        wavefronts it is the batch's last frame, as in the reference, whose
        sensor integrates the frames one after the other
        (OOPAO/Pyramid.py:825-830); ``device_frame`` holds them all."""
        if self._frame_host is None and self._frame_dev is not None:
            t = self._frame_dev.detach()
            self._frame_host = (t[-1] if t.ndim == 3 else t).to('cpu', torch.float64).numpy()
        return self._frame_host

    @frame.setter
    def frame(self, val):
        self._frame_host = np.asarray(val)
        self._frame_dev = None

    # ------------------------------------------------------------------ reports
    def rebin(self, arr, new_shape):
        """Sum-rebin of a host 2-D array to new_shape, as the mean of each
        block times its size (OOPAO/Detector.py:174-179)."""
        arr = np.asarray(arr)
        fy, fx = arr.shape[0] // new_shape[0], arr.shape[1] // new_shape[1]
        return arr.reshape(new_shape[0], fy, new_shape[1], fx).mean(-1).mean(1) * fy * fx

    def set_binning(self, array, binning_factor, mode='sum'):
        """Sum (or mean) binning of a host 2-D array (OOPAO/Detector.py:181-183)."""
        return set_binning(np.asarray(array), binning_factor, mode)

    def computeSNR(self):
        """computeSNR (OOPAO/Detector.py:356-365)."""
        self.SNR_max = self.FWC / np.sqrt(self.FWC) if self.FWC is not None else np.nan
        self.SNR = self.signal / np.sqrt(self.quantification_noise ** 2 + self.photon_noise ** 2 +
                                         self.readoutNoise ** 2 + self.dark_shot_noise ** 2)
        print()
        print('Theoretical maximum SNR: %.2f' % self.SNR_max)
        print('Current SNR: %.2f' % self.SNR)

    def displayNoiseError(self):
        """displayNoiseError (OOPAO/Detector.py:367-383)."""
        print()
        print('------------ Noise error ------------')
        if self.bits is not None:
            print('{:^25s}|{:^9.4f}'.format('Quantization noise [e-]', self.quantification_noise))
        if self.photonNoise is True:
            print('{:^25s}|{:^9.4f}'.format('Photon noise [e-]', self.photon_noise))
        if self.darkCurrent != 0:
            print('{:^25s}|{:^9.4f}'.format('Dark shot noise [e-]', self.dark_shot_noise))
        if self.readoutNoise != 0:
            print('{:^25s}|{:^9.1f}'.format('Readout noise [e-]', self.readoutNoise))
        print('-------------------------------------')

    def properties(self):
        """Display lines of the camera (OOPAO/Detector.py:424-443)."""
        p = {'sensor': f"{'Sensor type':<25s}|{self.sensor:^9s}"}
        if self.resolution is not None:
            p['resolution'] = f"{'Resolution [px]':<25s}|{int(self.resolution // self.binning):^9d}"
        if self.integrationTime is not None:
            p['exposure'] = f"{'Exposure time [ms]':<25s}|{self.integrationTime * 1000:^9.2f}"
        if self.bits is not None:
            p['quantization'] = f"{'Quantization [bits]':<25s}|{self.bits:^9d}"
        if self.FWC is not None:
            p['FWC'] = f"{'Full well capacity [e-]':<25s}|{int(self.FWC):^9d}"
        p['gain'] = f"{'Gain':<25s}|{str(self.gain):^9s}"
        p['QE'] = f"{'Quantum efficiency [%]':<25s}|{int(self.QE * 100):^9d}"
        p['binning'] = f"{'Binning':<25s}|{str(self.binning) + 'x' + str(self.binning):^9s}"
        p['dark_current'] = f"{'Dark current [e-/px/s]':<25s}|{self.darkCurrent:^9.2f}"
        p['photon_noise'] = f"{'Photon noise':<25s}|{str(self.photonNoise):^9s}"
        p['bkg_noise'] = f"{'Bkg noise [e-]':<25s}|{str(self.backgroundNoise):^9s}"
        p['readout_noise'] = f"{'Readout noise [e-/px]':<25s}|{float(self.readoutNoise):^9.1f}"
        self.prop = p
        return p

    def print_properties(self):
        print(self)

    def __mul__(self, obj):
        """Camera * GainSensingCamera (OOPAO/Detector.py:385-393): the first
        product calibrates, the next ones compute the optical gains."""
        if getattr(obj, 'tag', None) == 'GSC':
            frame = self.device_frame
            if frame is None:
                raise OopaoError('The camera has no frame yet')
            if obj.calibration_ready is False:
                obj.calibration(frame)
                obj.detector_properties = self.properties()
            else:
                obj.compute_optical_gains(frame)
            return
        raise OopaoError(f'Coupled object should be a "GSC" but is {getattr(obj, "tag", type(obj).__name__)}')

    def __repr__(self):
        rows = list(self.properties().values())
        n = len(max(rows))
        return f'{"Detector":-^{n}}\n' + ''.join(r + '\n' for r in rows) + f'{"":-^{n}}\n'
