"""WFS camera: drop-in for the reference ``Detector`` (``OOPAO/Detector.py``)
as used by the pyramid.

The pyramid kernels write the noise-free, sum-binned frame on the device
(``integrate``/``readout`` with the default settings reduce to that frame,
``OOPAO/Detector.py:273-354``).  ``frame`` is materialised on the host only
when read.  QE and gain are applied on the device; photon and readout noise,
when switched on, are drawn on the device after the binning (the reference
seeds its noise from the wall clock, so noisy frames are statistical, not
bit-level, matches).
"""
import numpy as np
import torch

from .tools import OopaoError


class Detector:
    def __init__(self, nRes: int = None, integrationTime: float = None, bits: int = None,
                 output_precision: int = None, FWC: int = None, gain: int = 1, sensor: str = 'CCD',
                 QE: float = 1., binning: int = 1, psf_sampling: float = 2., darkCurrent: float = 0.,
                 readoutNoise: float = 0, photonNoise: bool = False, backgroundNoise: bool = False,
                 backgroundFlux: float = None, backgroundMap: float = None, log_scale: bool = False):
        if sensor not in ['EMCCD', 'CCD', 'CMOS']:
            raise OopaoError("Sensor must be 'EMCCD', 'CCD', or 'CMOS'")
        self.resolution = nRes
        self.integrationTime = integrationTime
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
        self.backgroundNoise = backgroundNoise
        self.backgroundFlux = backgroundFlux
        self.backgroundMap = backgroundMap
        self.log_scale = log_scale
        self.tag = 'detector'
        self._integrated_time = 0
        self.is_focal_plane_camera = False
        self._frame_dev = None
        self._frame_host = np.zeros([nRes, nRes]) if nRes is not None else None
        self.generator = None

    def _unsupported(self):
        if self.integrationTime is not None or self.bits is not None or self.FWC is not None or \
                self.darkCurrent != 0 or self.backgroundNoise or self.backgroundMap is not None or \
                self.log_scale or self.sensor == 'EMCCD' or self.binning != 1:
            raise OopaoError('oopao_gb300 Detector supports QE, gain, photon and readout noise only')

    def _integrate_device(self, frame_dev):
        """Apply QE, noise and gain to device frames [B,cam,cam] (in place when possible)."""
        self._unsupported()
        f = frame_dev
        if self.photonNoise:
            f = torch.poisson(f.clamp_min(0), generator=self.generator)
        if self.QE != 1:
            f = f * self.QE
        if self.readoutNoise != 0:
            f = f + torch.round(torch.randn(f.shape, device=f.device, generator=self.generator) *
                                self.readoutNoise)
        if self.gain != 1:
            f = f * self.gain
        return f

    def integrate(self, frame):
        """``Detector.integrate`` + ``readout`` (OOPAO/Detector.py:331-354) for a
        frame computed outside the WFS camera path (the focal-plane camera):
        the frame is kept as ``perfect_frame``, then QE, noise and gain apply.
        A device tensor stays on the device."""
        self._unsupported()
        if isinstance(frame, torch.Tensor):
            t = frame.to(torch.float32)
            self._perfect_dev, self._perfect_host = t, None
            self._set_device_frame(self._integrate_device(t[None]))
            return
        self._perfect_dev, self._perfect_host = None, np.array(frame, dtype=np.float64)
        if self.photonNoise or self.readoutNoise != 0 or self.QE != 1 or self.gain != 1:
            dev = torch.device('cuda', torch.cuda.current_device())
            t = torch.as_tensor(np.ascontiguousarray(frame, dtype=np.float32), device=dev)[None]
            self._set_device_frame(self._integrate_device(t))
        else:
            self.frame = self._perfect_host.copy()

    @property
    def perfect_frame(self):
        if getattr(self, '_perfect_host', None) is None and getattr(self, '_perfect_dev', None) is not None:
            self._perfect_host = self._perfect_dev.detach().to('cpu', torch.float64).numpy()
        return getattr(self, '_perfect_host', None)

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

    def properties(self):
        """Display lines of the camera (the reference's ``properties``, :361-383)."""
        return {'resolution': f'{"Resolution [px]":<25s}|{str(self.resolution):^9s}',
                'qe': f'{"Quantum efficiency":<25s}|{self.QE:^9.2f}',
                'gain': f'{"Gain":<25s}|{str(self.gain):^9s}',
                'photon': f'{"Photon noise":<25s}|{str(self.photonNoise):^9s}',
                'ron': f'{"Readout noise [e-]":<25s}|{float(self.readoutNoise):^9.1f}'}

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

    def _set_device_frame(self, t):
        self._frame_dev = t
        self._frame_host = None

    @property
    def frame(self):
        """The last integrated frame, float64 [cam, cam].  After a batch of
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

    def __repr__(self):
        return 'Detector(%s px, QE=%.2f, gain=%s)' % (self.resolution, self.QE, self.gain)
