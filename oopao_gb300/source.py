"""Light carrier: drop-in for the reference ``Source`` (``OOPAO/Source.py``).

Same constructor, photometry table, ``*`` (relay) and ``**`` (reset + relay)
operators, and ``OPD`` / ``OPD_no_pupil`` / ``phase`` / ``fluxMap`` /
``intensity`` attributes.  The optical path difference is also kept on the
GPU: elements that produce it on the device (the deformable mirror) hand
over a device tensor, and the host numpy views are materialised only when a
user reads them.  Device maps are float32 [res,res] or [B,res,res]; host
maps follow the reference layout ([res,res] or [res,res,B], float64).
"""
import numpy as np
import torch

from .tools import OopaoError

_CST = 368.0
# Source.photometry, OOPAO/Source.py:340-405: [wavelength, bandwidth, zero point]
_PHOT = {
    'U': [0.360e-6, 0.070e-6, 1.96e12 / _CST], 'B': [0.440e-6, 0.100e-6, 5.38e12 / _CST],
    'V0': [0.500e-6, 0.090e-6, 3.64e12 / _CST], 'V': [0.550e-6, 0.090e-6, 3.31e12 / _CST],
    'R': [0.640e-6, 0.150e-6, 4.01e12 / _CST], 'R2': [0.650e-6, 0.300e-6, 7.9e12 / _CST],
    'R3': [0.600e-6, 0.300e-6, 8.56e12 / _CST], 'R4': [0.670e-6, 0.300e-6, 7.66e12 / _CST],
    'I': [0.790e-6, 0.150e-6, 2.69e12 / _CST], 'I1': [0.700e-6, 0.033e-6, 0.67e12 / _CST],
    'I2': [0.750e-6, 0.033e-6, 0.62e12 / _CST], 'I3': [0.800e-6, 0.033e-6, 0.58e12 / _CST],
    'I4': [0.700e-6, 0.100e-6, 2.02e12 / _CST], 'I5': [0.850e-6, 0.100e-6, 1.67e12 / _CST],
    'I6': [1.000e-6, 0.100e-6, 1.42e12 / _CST], 'I7': [0.850e-6, 0.300e-6, 5.00e12 / _CST],
    'I8': [0.750e-6, 0.100e-6, 1.89e12 / _CST], 'I9': [0.850e-6, 0.300e-6, 5.00e12 / _CST],
    'I10': [0.900e-6, 0.300e-6, 4.72e12 / _CST], 'J': [1.215e-6, 0.260e-6, 1.90e12 / _CST],
    'J2': [1.550e-6, 0.260e-6, 1.49e12 / _CST], 'H': [1.654e-6, 0.290e-6, 1.05e12 / _CST],
    'Kp': [2.1245e-6, 0.351e-6, 0.62e12 / _CST], 'Ks': [2.157e-6, 0.320e-6, 0.55e12 / _CST],
    'K': [2.179e-6, 0.410e-6, 0.70e12 / _CST], 'K0': [2.000e-6, 0.410e-6, 0.76e12 / _CST],
    'K1': [2.400e-6, 0.410e-6, 0.64e12 / _CST], 'L': [3.547e-6, 0.570e-6, 2.5e11 / _CST],
    'M': [4.769e-6, 0.450e-6, 8.4e10 / _CST], 'Na': [0.589e-6, 0, 3.3e12 / _CST],
    'EOS': [1.064e-6, 0, 3.3e12 / _CST], 'IR1310': [1.310e-6, 0, 2e12 / _CST],
}


def _host_from_device(t):
    a = t.detach().to('cpu', torch.float64).numpy()
    return np.moveaxis(a, 0, -1) if a.ndim == 3 else a


class Source:
    def __init__(self, optBand: str, magnitude: float, coordinates: list = [0, 0],
                 altitude: float = np.inf, laser_coordinates: list = [0, 0], Na_profile=None,
                 fwhm_spot_up=None, display_properties: bool = True, chromatic_shift=None):
        self.display_properties = display_properties
        self.optBand = optBand
        self.wavelength, self.bandwidth, self.zeroPoint = self.photometry(optBand)
        self._magnitude = magnitude
        self._nPhoton = self.zeroPoint * 10 ** (-0.4 * magnitude)
        self.tag = 'source'
        self.altitude = altitude
        self.coordinates = coordinates
        self.laser_coordinates = laser_coordinates
        self.chromatic_shift = chromatic_shift
        if Na_profile is not None and fwhm_spot_up is not None:
            self.Na_profile = Na_profile
            self.fwhm_spot_up = fwhm_spot_up
            self.altitude = np.sum(Na_profile[0, :] * Na_profile[1, :])
            self.type = 'LGS'
        else:
            self.type = 'NGS'
        self.precision = np.float64
        self.mask = 1
        self._fluxMap = None
        self._scintillation = None
        self._intensity = None
        self._intensity_version = 0
        self._intensity_inputs = None
        self._opd_zero = False      # OPD_no_pupil is the all-zero map set by tel.relay
        self._opd = None            # host OPD (masked), reference layout
        self._opd_np = None         # host OPD_no_pupil
        self._dev = None            # device OPD_no_pupil (float32), authoritative if _dev_fresh
        self._dev_fresh = False
        self.optical_path = [[self.type + '(' + self.optBand + ')', self]]
        self.inAsterism = False
        self.ast_idx = -1
        self.tel = None
        if display_properties:
            print(self)

    # ----------------------------------------------------------- operators
    def __pow__(self, obj):
        obj.src = self
        self.optical_path = [[self.type + '(' + self.optBand + ')', self]]
        self.reset()
        self * obj
        return self

    def __mul__(self, obj):
        if obj is not None:
            if isinstance(obj, list):
                for o in obj:
                    self * o
            else:
                obj.relay(self)
        return self

    def print_optical_path(self):
        """The objects the light went through, ' ~~> '-separated
        (OOPAO/Source.py:197-204)."""
        if self.optical_path is not None:
            print(' ~~> '.join(str(o[0]) for o in self.optical_path))

    def reset(self):
        self.mask = 1
        self._opd = None
        self._opd_np = None
        self._dev = None
        self._dev_fresh = False
        self._opd_zero = False
        self._scintillation = None

    # ----------------------------------------------------------- device OPD
    def _set_device_opd(self, t):
        """Hand over a device OPD (no pupil) produced on the GPU."""
        self._opd_zero = False
        self._dev = t
        self._dev_fresh = True
        self._opd = None
        self._opd_np = None

    def _set_zero_opd(self, shape):
        self.OPD_no_pupil = np.zeros(shape)
        self._opd_zero = True

    def _sync_host(self):
        if self._dev_fresh and self._opd_np is None:
            self._opd_np = _host_from_device(self._dev)
            m = self.mask
            if self._opd_np.ndim == 3 and not np.isscalar(m):
                self._opd = self._opd_np * m[:, :, None]
            else:
                self._opd = self._opd_np * m

    def device_opd(self, dev):
        """OPD on the device as float32 [res,res] or [B,res,res] (values
        inside the pupil are those of ``OPD``)."""
        if self._dev_fresh:
            return self._dev
        if self._opd is None:
            raise OopaoError('No OPD propagated: use src**tel first')
        a = np.asarray(self._opd)
        if a.ndim == 3:
            a = np.moveaxis(a, -1, 0)
        self._dev = torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device=dev)
        self._dev_fresh = True
        return self._dev

    # ----------------------------------------------------------- properties
    @property
    def OPD(self):
        self._sync_host()
        return self._opd

    @OPD.setter
    def OPD(self, val):
        self._opd_zero = False
        self._dev_fresh = False
        self._dev = None
        self._opd = None if val is None else np.array(val)
        if val is None:
            self._opd_np = None

    @property
    def OPD_no_pupil(self):
        self._sync_host()
        return self._opd_np

    @OPD_no_pupil.setter
    def OPD_no_pupil(self, val):
        self._opd_zero = False
        self._dev_fresh = False
        self._dev = None
        if val is None:
            self._opd_np = None
            return
        self._opd_np = np.array(val)
        if self._opd_np.ndim > 2 and not np.isscalar(self.mask):
            self._opd = self._opd_np * self.mask[:, :, None]
        else:
            self._opd = self._opd_np * self.mask

    @property
    def phase(self):
        return self.OPD * 2 * np.pi / self.wavelength

    @phase.setter
    def phase(self, val):
        self.OPD = (val * self.wavelength) / (2 * np.pi)

    @property
    def phase_no_pupil(self):
        return self.OPD_no_pupil * 2 * np.pi / self.wavelength

    @phase_no_pupil.setter
    def phase_no_pupil(self, val):
        self.OPD_no_pupil = (val * self.wavelength) / (2 * np.pi)

    def _refresh_intensity(self):
        flux, scint = self._fluxMap, self._scintillation
        last = self._intensity_inputs
        if last is not None and last[0] is flux and last[1] is scint:
            return  # same input arrays: intensity (and its version) unchanged
        self._intensity_inputs = (flux, scint)
        if flux is None or np.size(flux) == 0:
            self._intensity = None
        elif scint is None:
            self._intensity = np.array(flux, dtype=self.precision)
        else:
            self._intensity = (np.array(flux) * np.array(scint)).astype(self.precision)
        self._intensity_version += 1

    @property
    def fluxMap(self):
        return self._fluxMap

    @fluxMap.setter
    def fluxMap(self, val):
        if val is not None and val is self._fluxMap:
            return
        self._fluxMap = None if val is None else np.asarray(val)
        self._refresh_intensity()

    @property
    def scintillation(self):
        return self._scintillation

    @scintillation.setter
    def scintillation(self, val):
        if val is not None and val is self._scintillation:
            return
        self._scintillation = None if val is None else np.asarray(val)
        self._refresh_intensity()

    @property
    def intensity(self):
        return self._intensity

    @intensity.setter
    def intensity(self, val):
        self._intensity = None if val is None else np.array(val, dtype=self.precision)
        self._intensity_inputs = None
        self._intensity_version += 1

    @property
    def nPhoton(self):
        return self._nPhoton

    @nPhoton.setter
    def nPhoton(self, val):
        self._nPhoton = val
        self._magnitude = -2.5 * np.log10(val / self.zeroPoint)

    @property
    def magnitude(self):
        return self._magnitude

    @magnitude.setter
    def magnitude(self, val):
        self._magnitude = val
        self._nPhoton = self.zeroPoint * 10 ** (-0.4 * val)

    def photometry(self, arg):
        if not isinstance(arg, str):
            raise OopaoError('The photometry object takes a string as an input')
        if arg not in _PHOT:
            raise OopaoError('Wrong name for the photometry object')
        w, b, z = _PHOT[arg]
        return w, b, z

    def __repr__(self):
        return ('Source(%s, mag=%.2f, lambda=%.3e m, nPhoton=%.3e ph/m2/s)'
                % (self.optBand, self._magnitude, self.wavelength, self._nPhoton))
