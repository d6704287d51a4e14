"""Gain-sensing camera: drop-in for the reference ``GainSensingCamera``
(``OOPAO/GainSensingCamera.py``, Chambouleyron et al. 2021).

It estimates the modal optical gains of a modulated pyramid from the
full-resolution focal-plane (modulation) camera frame with the convolutional
model of the reference: calibration at a working point (``calibration``
:78-95) and gains of later frames against it (``compute_optical_gains``
:104-120).  Every transform and the contraction over pixels run in the
library (``oopao_gsc_*``); the basis product is kept on the device as
float32 [modes][n*n] (the reference keeps complex128 [n, n, modes]), and
frames may stay on the device (``wfs * wfs.focal_plane_camera`` followed by
``wfs.focal_plane_camera * gsc`` never leaves it).

Usage as in the reference::

    gsc = GainSensingCamera(wfs.mask, basis_3D)      # basis [n, n, modes]
    wfs.focal_plane_camera.resolution = wfs.nRes
    ngs ** tel * wfs; wfs * wfs.focal_plane_camera
    wfs.focal_plane_camera * gsc                     # calibration
    ...; wfs.focal_plane_camera * gsc                # gsc.og
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .runtime import Workspace, device
from .tools import OopaoError

_IR_CALIB, _SENSI_CALIB, _BASIS_PRODUCT, _MODE_POWER = 0, 1, 2, 3


class GainSensingCamera:
    def __init__(self, mask: np.ndarray, basis: np.ndarray, n_jobs: int = 10) -> None:
        self.mask = mask
        self.basis = basis
        self.n_modes = int(np.shape(basis)[-1])
        self.n_jobs = n_jobs
        self.calibration_ready = False
        self.detector_properties = None
        self.tag = 'GSC'
        self.og = np.ones(self.n_modes)
        m = np.asarray(mask)
        if m.ndim != 2 or m.shape[0] != m.shape[1]:
            raise OopaoError('The mask must be square')
        self.n = m.shape[0]
        n0 = np.shape(basis)[0]
        if np.ndim(basis) != 3 or np.shape(basis)[1] != n0:
            raise OopaoError('The basis must be [n_pix, n_pix, n_modes]')
        if self.n <= n0:
            raise OopaoError('Output size %d should be higher than input size %d' % (self.n, n0))
        if (self.n - n0) % 2:
            raise OopaoError('The padded basis (%d px) must match the mask size (%d px)' % (n0, self.n))
        if np.iscomplexobj(basis):
            raise OopaoError('The modal basis must be real (OPD maps)')
        self._dev = device()
        self._plan = ctypes.c_void_p()
        N.call('oopao_gsc_plan_create', ctypes.byref(self._plan), self.n, self.n_modes,
               np.ascontiguousarray(m, dtype=np.complex64))
        self._ws = Workspace()
        self._basis_ready = False
        self._og_dev = None
        self._sensi_dev = None
        self._ir_sky_dev = None
        # also return sensitivity(IR_sky, IR_calib) per frame (sensi_sky)
        self.keep_sensitivity = True

    def __del__(self):
        h = getattr(self, '_plan', None)
        if h is not None and h.value:
            try:
                N.load().oopao_gsc_plan_destroy(h)
            except Exception:
                pass
            self._plan = None

    # ------------------------------------------------------------ helpers
    def _frames(self, frame):
        t = frame if isinstance(frame, torch.Tensor) else torch.as_tensor(np.asarray(frame, dtype=np.float32))
        t = t.to(self._dev, torch.float32)
        if t.shape[-2:] != (self.n, self.n):
            raise OopaoError('The focal-plane frame must be %d x %d (set focal_plane_camera.resolution = wfs.nRes)'
                             % (self.n, self.n))
        return t.reshape(-1, self.n, self.n).contiguous()

    def _set_basis(self):
        b = torch.as_tensor(np.ascontiguousarray(np.moveaxis(np.asarray(self.basis, dtype=np.float32), -1, 0)),
                            device=self._dev)
        nb = max(N.load().oopao_gsc_workspace_bytes(self._plan, 1), min(self.n_modes * self.n ** 2 * 8, 1 << 30))
        ws = self._ws.get(nb)
        N.call('oopao_gsc_set_basis', self._plan, N.ptr(b), b.shape[-1], N.ptr(ws), ws.numel(), N.stream_handle())
        self._basis_ready = True

    # ------------------------------------------------------------ reference API
    def calibration(self, frame) -> None:
        """``calibration`` (:78-95): basis product, IR_calib and sensi_calib at this frame."""
        f = self._frames(frame)[0]
        if not self._basis_ready:
            self._set_basis()
        nb = N.load().oopao_gsc_workspace_bytes(self._plan, 1)
        ws = self._ws.get(nb)
        N.call('oopao_gsc_calibrate', self._plan, N.ptr(f), N.ptr(ws), ws.numel(), N.stream_handle())
        self.calibration_ready = True
        self.og = np.ones(self.n_modes)
        self._og_dev = None

    def reset_calibration(self) -> None:
        self.calibration_ready = False
        self.og = np.ones(self.n_modes)

    def compute_optical_gains(self, frame) -> None:
        """``compute_optical_gains`` (:104-120).  A [B, n, n] stack gives
        ``og_batch`` [B, n_modes]; ``og`` is then the last frame's gains."""
        if self.calibration_ready is False:
            raise OopaoError('Optical gains must be initialized first!')
        f = self._frames(frame)
        B = f.shape[0]
        og = torch.empty((B, self.n_modes), dtype=torch.float64, device=self._dev)
        sensi = torch.empty((B, self.n_modes, 2), dtype=torch.float64, device=self._dev) if self.keep_sensitivity \
            else None
        ir = torch.empty((B, self.n, self.n), dtype=torch.float32, device=self._dev)
        nb = N.load().oopao_gsc_workspace_bytes(self._plan, B)
        ws = self._ws.get(nb)
        N.call('oopao_gsc_optical_gains', self._plan, N.ptr(f), B, N.ptr(og), N.ptr(sensi), N.ptr(ir), N.ptr(ws),
               ws.numel(), N.stream_handle())
        self._og_dev, self._sensi_dev, self._ir_sky_dev = og, sensi, ir
        host = og.cpu().numpy()
        self.og_batch = host
        self.og = host[-1].copy()

    # ------------------------------------------------------------ device views
    @property
    def device_og(self):
        """Last gains as a float64 device tensor [B, n_modes] (GPU-resident loops)."""
        return self._og_dev

    def _read(self, what, shape, dtype):
        out = torch.empty(shape, dtype=dtype, device=self._dev)
        N.call('oopao_gsc_read', self._plan, what, N.ptr(out), N.stream_handle())
        return out

    @property
    def IR_calib(self):
        if not self.calibration_ready:
            raise OopaoError('Not calibrated')
        return self._read(_IR_CALIB, (self.n, self.n), torch.float32).double().cpu().numpy()

    @property
    def sensi_calib(self):
        if not self.calibration_ready:
            raise OopaoError('Not calibrated')
        s = self._read(_SENSI_CALIB, (self.n_modes, 2), torch.float64).cpu().numpy()
        return s[:, 0] + 1j * s[:, 1]

    @property
    def IR_sky(self):
        if self._ir_sky_dev is None:
            raise OopaoError('No optical gains computed yet')
        return self._ir_sky_dev[-1].double().cpu().numpy()

    @property
    def sensi_sky(self):
        if self._sensi_dev is None:
            raise OopaoError('No optical gains computed yet')
        s = self._sensi_dev[-1].cpu().numpy()
        return s[:, 0] + 1j * s[:, 1]

    @property
    def basis_product(self):
        """[n, n, n_modes] like the reference's (real here: fft3(b) ifft3(b) = |fft3(b)|^2 for a real basis)."""
        if not self._basis_ready:
            raise OopaoError('The basis product is computed at the calibration')
        bp = self._read(_BASIS_PRODUCT, (self.n_modes, self.n, self.n), torch.float32).double()
        bp *= self._read(_MODE_POWER, (self.n_modes,), torch.float64)[:, None, None]
        return np.moveaxis(bp.cpu().numpy(), 0, -1)

    def __repr__(self) -> str:
        prop = f'{"Calibrated":<16}|{str(self.calibration_ready):^7}\n'
        prop += f'{"Number of modes":<16}|{self.n_modes:^7}\n'
        n_char = len(max(prop.split('\n'), key=len))
        return f'{" GSC ":-^{n_char}}\n' + prop + f'{"":-^{n_char}}\n'
