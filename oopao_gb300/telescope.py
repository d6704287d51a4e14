"""Pupil and flux carrier: drop-in for the reference ``Telescope``
(``OOPAO/Telescope.py``).  Only the parts on the PWFS path are provided:
pupil definition (``set_pupil`` :226-246), ``relay`` (:199-224) and the OPD
accessors forwarding to the coupled source."""
import numpy as np

from .tools import OopaoError, warning


class Telescope:
    def __init__(self, resolution: int, diameter: float, samplingTime: float = 0.001,
                 centralObstruction: float = 0., fov: float = 0., pupil=None,
                 pupilReflectivity: float = 1., display_optical_path: bool = False):
        self.isInitialized = False
        self.resolution = resolution
        self.D = diameter
        self.initial_D = diameter
        self.initial_resolution = resolution
        self.pixelSize = self.D / self.resolution
        self.centralObstruction = centralObstruction
        self.fov = fov
        self.rad2arcsec = (180 / np.pi) * 3600
        self.fov_rad = fov / self.rad2arcsec
        self.samplingTime = samplingTime
        self.user_defined_pupil = pupil
        self.pupilReflectivity = np.float64(pupilReflectivity)
        self.precision = np.float64
        self.set_pupil()
        self.src = None
        self.tag = 'telescope'
        self.isPaired = False
        self.spatialFilter = None
        self.display_optical_path = display_optical_path
        self.optical_path = None
        self.isInitialized = True
        self.initial_pupil = self.pupil.copy()

    def set_pupil(self):
        if self.user_defined_pupil is None:
            D = self.resolution + 1
            x = np.linspace(-self.resolution / 2, self.resolution / 2, self.resolution, dtype=np.float64)
            xx, yy = np.meshgrid(x, x)
            circle = xx ** 2 + yy ** 2
            obs = circle >= (self.centralObstruction * D / 2) ** 2
            pupil = (circle < (D / 2) ** 2) * obs
        else:
            warning('User-defined pupil, the central obstruction will not be taken into account...')
            pupil = self.user_defined_pupil.copy().astype(np.float64)
        self._pupil = pupil.astype(bool)
        self.pupilReflectivity = (self._pupil * self.pupilReflectivity).astype(np.float64)
        self.pixelArea = np.sum(self._pupil)
        self.pupilLogical = np.where(np.reshape(self._pupil, self.resolution ** 2) > 0)

    @property
    def pupil(self):
        return self._pupil

    @pupil.setter
    def pupil(self, val):
        self._pupil = np.asarray(val).astype(bool)
        self.pixelArea = np.sum(self._pupil)
        self.pupilLogical = np.where(np.reshape(self._pupil, self.resolution ** 2) > 0)
        self.pupilReflectivity = self._pupil.astype(np.float64)

    def print_optical_path(self):
        """OOPAO/Telescope.py:575-585: the telescope's own optical path (which
        the light's relays do not fill), else a notice."""
        if self.optical_path is not None:
            print(' ~~> '.join(str(o[0]) for o in self.optical_path))
        else:
            print('No light propagated through the telescope')

    def relay(self, src):
        if src.tag != 'source':
            raise OopaoError('Only a single Source can be propagated (asterisms are not supported)')
        self.src = src
        src.optical_path.append([self.tag, self])
        src.tel = self
        src.mask = self.pupil.copy()
        if src._opd is None and not src._dev_fresh:
            src._set_zero_opd(self.pupil.shape)
        elif np.ndim(src.OPD) == 2:
            src.OPD_no_pupil = src.OPD_no_pupil
        else:
            src._set_zero_opd(self.pupil.shape)
        if src.scintillation is None or np.ndim(src.scintillation) != 2:
            src.scintillation = self._cached('scint', (id(self._pupil),),
                                             lambda: np.ones(self.pupil.shape) * src.mask)
        key = (id(self.pupilReflectivity), src.nPhoton, self.samplingTime, self.D, self.resolution)
        src.fluxMap = self._cached('flux', key, lambda: self.pupilReflectivity * src.nPhoton *
                                   self.samplingTime * (self.D / self.resolution) ** 2)

    def _cached(self, name, key, make):
        # the same array object is handed out while its inputs are unchanged,
        # so a Source can tell that its intensity did not change
        cache = self.__dict__.setdefault('_relay_cache', {})
        hit = cache.get(name)
        if hit is None or hit[0] != key:
            hit = (key, make())
            cache[name] = hit
        return hit[1]

    @property
    def OPD(self):
        return self.src.OPD

    @OPD.setter
    def OPD(self, val):
        self.src.OPD = val

    @property
    def OPD_no_pupil(self):
        return self.src.OPD_no_pupil

    @OPD_no_pupil.setter
    def OPD_no_pupil(self, val):
        self.src.OPD_no_pupil = val

    def resetOPD(self):
        self.src ** self

    def __mul__(self, obj):
        self.relay(self.src)
        obj.relay(self.src)
        return self

    def __repr__(self):
        return 'Telescope(D=%.2f m, resolution=%d px, obstruction=%.2f)' % (
            self.D, self.resolution, self.centralObstruction)
