"""Modulated pyramid wavefront sensor: drop-in for the reference ``Pyramid``
(``OOPAO/Pyramid.py``) backed by the GB300 kernels of ``liboopao_gb300``.

Host-side (setup, float64 numpy, same formulas as the reference):
  * FFT grid N, camera size, zero padding        (:276-285)
  * pyramid phase mask, stored complex64          (:368-391, :453-539)
  * modulation path and nTheta                    (:1112-1132)
  * quadrant geometry of ``grabQuadrant``         (:946-961)
Device-side (every measurement): the fused propagation, K-sum and binning
(``oopao_pwfs_measure``) and the signal processing (``oopao_pwfs_signal``).
Valid pixels (``initialization`` :541-589) and the reference slopes
(``wfs_calibration`` :591-610) are measured with the same device path.
"""
import numpy as np
import torch

from . import _native as N
from .detector import Detector
from .runtime import Workspace, device
from .tools import OopaoError, warning

SP_MODES = {'slopesMaps': 0, 'slopesMaps_incidence_flux': 1, 'slopesMaps_camera_flux': 2,
            'fullFrame': 3, 'fullFrame_incidence_flux': 4, 'fullFrame_camera_flux': 5,
            'fullFrame_sum_flux': 6}


class _Plan:
    """Owner of one ``oopao_pwfs_plan`` (geometry + modulation path)."""

    def __init__(self, res, n, cam, mask_c64, path, tt_scale, psf_centering):
        self.res, self.n, self.cam = res, n, cam
        self.k = 1 if path is None else len(path)
        h = N.c_void_p()
        m = np.ascontiguousarray(mask_c64, dtype=np.complex64)
        p = None if path is None else np.ascontiguousarray(np.asarray(path, dtype=np.float64))
        N.call('oopao_pwfs_plan_create', N.ctypes.byref(h), res, n, cam, self.k, m, p,
               float(tt_scale), int(bool(psf_centering)))
        self.h = h
        self._amp_key = None
        self._weights = None

    def __del__(self):
        try:
            if self.h:
                N.load().oopao_pwfs_plan_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def set_amplitude(self, intensity, key):
        if key is not None and key == self._amp_key:
            return
        amp = N.host(np.sqrt(np.asarray(intensity, dtype=np.float64) / self.k), np.float32)
        N.call('oopao_pwfs_set_amplitude', self.h, amp)
        self._amp_key = key

    def set_weights(self, w):
        """Per-point factors of the sum over modulation points (None: the
        plain sum); uploaded only when they change."""
        if w is None and self._weights is None:
            return
        if w is not None:
            w = np.asarray(w, dtype=np.float64).ravel()
            if w.size != self.k:
                raise OopaoError('weight_vector has %d entries for %d modulation points' % (w.size, self.k))
            if self._weights is not None and np.array_equal(w, self._weights):
                return
        N.call('oopao_pwfs_set_weights', self.h, None if w is None else N.host(w, np.float32))
        self._weights = w

    def workspace_bytes(self, batch):
        return N.load().oopao_pwfs_workspace_bytes(self.h, batch)


class Pyramid:
    def __init__(self, nSubap: float, telescope, modulation: float, lightRatio: float,
                 postProcessing: str = 'slopesMaps', psfCentering: bool = True,
                 n_pix_separation: float = 2., calibModulation: float = 50., n_pix_edge: float = None,
                 extraModulationFactor: int = 0, binning: int = 1, nTheta_user_defined: int = None,
                 userValidSignal: bool = None, old_mask: bool = False, rooftop: float = 0,
                 theta_rotation: float = 0, delta_theta: float = 0., user_modulation_path: list = None,
                 pupilSeparationRatio: float = None, edgePixel: int = None, zeroPadding: int = None,
                 max_batch: int = 64):
        self.gpu_available = True
        self._dev = device()
        self.telescope = telescope
        if (telescope.resolution / nSubap) % 2 != 0 and telescope.resolution / nSubap != 1:
            raise OopaoError('The resolution should be an even number and be a multiple of 2**i where i>=2')
        if telescope.src is None:
            raise OopaoError('The telescope was not coupled to any source object! Make sure to couple '
                             'it with an src object using src*tel')
        if edgePixel is not None:
            raise OopaoError('The use of the edgePixel property has been deprecated. Consider using '
                             'n_pix_edge instead')
        if pupilSeparationRatio is not None:
            raise OopaoError('The use of the pupilSeparationRatio property has been deprecated. '
                             'Consider using n_pix_separation instead')
        if zeroPadding is not None:
            raise OopaoError('The use of the zeroPadding property has been deprecated')
        if postProcessing not in SP_MODES:
            raise OopaoError('Unknown postProcessing %r' % postProcessing)
        self.src = telescope.src
        self.wavelength_calibration = self.src.wavelength
        self.delta_theta = delta_theta
        self.nTheta_user_defined = nTheta_user_defined
        self.extraModulationFactor = extraModulationFactor
        self.nSubap = nSubap
        self.edgePixel = n_pix_edge
        self.centerPixel = 0
        self.postProcessing = postProcessing
        self.userValidSignal = userValidSignal
        self.psfCentering = psfCentering
        self.binning = binning
        self.old_mask = old_mask
        self.user_modulation_path = user_modulation_path
        self.modulation_length = 2 * np.pi
        self.weight_vector = None
        self.n_pix_separation = n_pix_separation
        self.sx = [0, 0, 0, 0]
        self.sy = [0, 0, 0, 0]
        if n_pix_edge is None:
            self.n_pix_edge = self.n_pix_separation // 2
        else:
            self.n_pix_edge = n_pix_edge
            if n_pix_edge != self.n_pix_separation // 2:
                warning('The recommanded value for n_pix_edge is ' + str(self.n_pix_separation // 2) +
                        ' instead of ' + str(n_pix_edge))
        self.rooftop = rooftop
        self.theta_rotation = theta_rotation
        res = telescope.resolution
        self.resolution = int((self.nSubap * 2 + self.n_pix_separation + self.n_pix_edge * 2) * res / self.nSubap)
        self.nRes = self.resolution
        self.zeroPaddingFactor = self.resolution / res
        self.zeroPadding = (self.resolution - res) // 2
        self.tag = 'pyramid'
        self.cam = Detector(round(nSubap * self.zeroPaddingFactor))
        self.focal_plane_camera = Detector(int((modulation * 4 + 12) * self.zeroPaddingFactor *
                                               res / telescope.initial_resolution))
        self.focal_plane_camera.is_focal_plane_camera = True
        if self.binning != 1 and self.cam.resolution % self.binning != 0:
            warning('The shape of the detector is not valid with the binning value requested: ' +
                    str(self.binning) + '! -- Ignoring the binning.')
            self.binning = 1
        self._cam_eff = self.cam.resolution // self.binning
        self._lightRatio = lightRatio
        self.calibModulation = res / 2 - 1 if calibModulation >= res / 2 else calibModulation
        self.isInitialized = False
        self.isCalibrated = False
        self._delta_Tip = 0
        self._delta_Tilt = 0
        self.center = self.resolution // 2
        self.spatialFilter = None
        self.rad2arcsec = (180 / np.pi) * 3600
        self.fov = self.rad2arcsec * self.resolution / self.zeroPaddingFactor * (self.src.wavelength / telescope.D)
        self.fov_l_d = self.resolution / self.zeroPaddingFactor
        self.max_fov_arcsec = self.fov / 2
        self.max_batch = max_batch
        self.keep_raw_data = True
        self._ws = Workspace()
        self._plan = None
        self.mask_computation()
        self.slopesUnits = 1
        self.referenceSignal = 0
        self.referenceSignal_2D = 0
        self.referencePyramidFrame = 0
        self.modulation = modulation
        self.initialization()
        self.modulation = modulation
        self.wfs_calibration()
        self.src ** self.telescope
        self.wfs_measure()

    # ------------------------------------------------------------------ geometry
    def get_phase_mask(self, resolution, n_subap, n_pix_separation, n_pix_edge, psf_centering=False,
                       sx=[0, 0, 0, 0], sy=[0, 0, 0, 0]):
        """Four-face mask with rooftop and rotation (OOPAO/Pyramid.py:453-480)."""
        rooftop_pixels = self.rooftop / np.sqrt(2)
        n_tot = int((n_subap * 2 + n_pix_separation + n_pix_edge * 2) * self.telescope.resolution / self.nSubap)
        norma = self.telescope.resolution / self.nSubap
        lim = np.pi
        x = np.linspace(-(1 - self.psfCentering * 1 / n_tot) * lim, (1 - self.psfCentering * 1 / n_tot) * lim,
                        n_tot, endpoint=self.psfCentering)
        x_, y_ = np.meshgrid(x, x)
        xr = x_ * np.cos(self.theta_rotation) - y_ * np.sin(self.theta_rotation)
        yr = y_ * np.cos(self.theta_rotation) + x_ * np.sin(self.theta_rotation)
        r = (self.nSubap + self.n_pix_separation) / 2
        P1 = xr * r + x_ * sx[0] + yr * r - y_ * sy[0] + rooftop_pixels
        P2 = -xr * r + x_ * sx[1] + yr * r - y_ * sy[1]
        P3 = -xr * r + x_ * sx[2] - yr * r - y_ * sy[2] + rooftop_pixels
        P4 = xr * r + x_ * sx[3] - yr * r - y_ * sy[3]
        return -np.max(np.stack([P1, P2, P3, P4]) * norma, axis=0)

    def get_phase_mask_old(self, resolution, n_subap, n_pix_separation, n_pix_edge, psf_centering=False,
                           sx=[0, 0, 0, 0], sy=[0, 0, 0, 0]):
        """Quadrant tip/tilt mask (OOPAO/Pyramid.py:482-539)."""
        n_tot = int((n_subap * 2 + n_pix_separation + n_pix_edge * 2) * self.telescope.resolution / self.nSubap)
        norma = self.telescope.resolution / self.nSubap / 4
        m = np.zeros([n_tot, n_tot])
        s = n_subap + n_pix_separation
        h = n_tot // 2
        if psf_centering:
            lim = np.pi
            Tip, Tilt = np.meshgrid(np.linspace(-lim, lim, h, endpoint=False),
                                    np.linspace(-lim, lim, h, endpoint=False))
            Tip -= np.mean(Tip)
            Tilt -= np.mean(Tilt)
            m[:h, :h] = (Tip * (s + sx[0]) + Tilt * (s - sy[0])) * norma
            m[:h, -h:] = (-Tip * (s - sx[1]) + Tilt * (s - sy[1])) * norma
            m[-h:, -h:] = (-Tip * (s - sx[2]) - Tilt * (s + sy[2])) * norma
            m[-h:, :h] = (Tip * (s + sx[3]) - Tilt * (s + sy[3])) * norma
        else:
            d_pix = np.pi / n_tot
            lp, lm = np.pi, np.pi - 2 * d_pix
            T1 = np.meshgrid(np.linspace(-lp, lp, h + 1, endpoint=True), np.linspace(-lp, lp, h + 1, endpoint=True))
            T2 = np.meshgrid(np.linspace(-lp, lp, h + 1, endpoint=True), np.linspace(-lm, lm, h - 1, endpoint=False))
            T3 = np.meshgrid(np.linspace(-lm, lm, h - 1, endpoint=False), np.linspace(-lm, lm, h - 1, endpoint=False))
            T4 = np.meshgrid(np.linspace(-lm, lm, h - 1, endpoint=False), np.linspace(-lp, lp, h + 1, endpoint=True))
            T = []
            for tip, tilt in (T1, T2, T3, T4):
                T.append((tip - np.mean(tip), tilt - np.mean(tilt)))
            (Tip_1, Tilt_1), (Tip_2, Tilt_2), (Tip_3, Tilt_3), (Tip_4, Tilt_4) = T
            m[:h + 1, :h + 1] = (Tip_1 * (s + sx[0]) + Tilt_1 * (s - sy[0])) * norma
            m[:h + 1, -h + 1:] = (-Tip_4 * (s - sx[1]) + Tilt_4 * (s - sy[1])) * norma
            m[-h + 1:, -h + 1:] = (-Tip_3 * (s - sx[2]) - Tilt_3 * (s + sy[2])) * norma
            m[-h + 1:, :h + 1] = (Tip_2 * (s + sx[3]) - Tilt_2 * (s + sy[3])) * norma
        return -m

    def mask_computation(self):
        fn = self.get_phase_mask_old if self.old_mask else self.get_phase_mask
        self.m = fn(resolution=self.resolution, n_subap=self.nSubap, n_pix_separation=self.n_pix_separation,
                    n_pix_edge=self.n_pix_edge, psf_centering=self.psfCentering, sx=self.sx, sy=self.sy)
        self.initial_m = self.m.copy()
        self.mask = np.complex64(np.exp(1j * self.m))
        self.initial_mask = np.copy(self.mask)
        self._plan = None

    def apply_shift_wfs(self, sx=None, sy=None, mis_reg=None, units='pixels'):
        """Moves the four pupil images by tilting the faces of the mask
        (OOPAO/Pyramid.py:400-451).  sx, sy: one shift for every face or four,
        in detector pixels or, with units='m', in metres at the pupil; a
        MisRegistration object gives them as dX_1..4 / dY_1..4.  The
        quadrant-tilt mask of old_mask takes twice the value for the same
        shift.  The new mask carries no spatial filter (initial_mask keeps the
        unshifted one) and the reference slopes are measured again."""
        sx = 0 if sx is None else sx
        sy = 0 if sy is None else sy
        if mis_reg is not None:
            sx = [mis_reg.dX_1, mis_reg.dX_2, mis_reg.dX_3, mis_reg.dX_4]
            sy = [mis_reg.dY_1, mis_reg.dY_2, mis_reg.dY_3, mis_reg.dY_4]
        f = 2 if self.old_mask else 1
        if units == 'pixels':
            factor = f
        elif units == 'm':
            factor = f / (self.telescope.D / self.nSubap)
        else:
            raise OopaoError("units must be 'pixels' or 'm'")
        if np.isscalar(sx) and np.isscalar(sy):
            shift_x, shift_y = [factor * sx] * 4, [factor * sy] * 4
        elif len(sx) == 4 and len(sy) == 4:
            shift_x, shift_y = [factor * v for v in sx], [factor * v for v in sy]
        else:
            raise OopaoError('Wrong size for sx and/or sy, a list of 4 values is expected.')
        if np.max(np.abs(shift_x)) > self.n_pix_edge or np.max(np.abs(shift_y)) > self.n_pix_edge:
            warning('The Pyramid pupils have been shifted outside of the detector!'
                    'Wrapping of the signal is currently occuring!!')
        self.sx = np.asarray(shift_x) / factor
        self.sy = np.asarray(shift_y) / factor
        fn = self.get_phase_mask_old if self.old_mask else self.get_phase_mask
        self.m = fn(resolution=self.resolution, n_subap=self.nSubap, n_pix_separation=self.n_pix_separation,
                    n_pix_edge=self.n_pix_edge, psf_centering=self.psfCentering, sx=shift_x, sy=shift_y)
        self.mask = np.complex64(np.exp(1j * self.m))
        self.slopesUnits = 1
        self.referenceSignal = 0
        self.referenceSignal_2D = 0
        self.wfs_calibration()

    @property
    def phasor(self):
        n = self.resolution
        xx, yy = np.meshgrid(np.linspace(0, n - 1, n), np.linspace(0, n - 1, n))
        return np.exp(-(1j * np.pi * (n + 1) / n) * (xx + yy))

    @property
    def Tip(self):
        t = np.meshgrid(np.linspace(-np.pi, np.pi, self.telescope.resolution),
                        np.linspace(-np.pi, np.pi, self.telescope.resolution))[0]
        return t * self.telescope.resolution / self.telescope.initial_resolution

    @property
    def Tilt(self):
        t = np.meshgrid(np.linspace(-np.pi, np.pi, self.telescope.resolution),
                        np.linspace(-np.pi, np.pi, self.telescope.resolution))[1]
        return t * self.telescope.resolution / self.telescope.initial_resolution

    @property
    def phaseBuffModulationLowres(self):
        """Per-point tip/tilt buffers, float32 [nTheta,res,res] (OOPAO/Pyramid.py:1133-1139)."""
        res = self.telescope.resolution
        out = np.zeros([self.nTheta, res, res], dtype=np.float32)
        if self.modulation_path is not None:
            tip, tilt = self.Tip, self.Tilt
            for i, (px, py) in enumerate(self.modulation_path):
                out[i] = px * tip + py * tilt
        return out

    def _effective_mask(self):
        """Focal-plane multiplier of one modulation point.  The mask carries the
        spatial filter; the 1-pixel-centred branch multiplies the shifted
        focal field by the filter once more (OOPAO/Pyramid.py:634-637)."""
        m = self.mask
        if not self.psfCentering and self.spatialFilter is not None:
            if np.shape(self.spatialFilter) != np.shape(m):
                raise OopaoError('spatialFilter must have the shape of the mask %s' % (np.shape(m),))
            m = m * self.spatialFilter
        return np.asarray(m).astype(np.complex64)

    def _make_plan(self, path):
        tel = self.telescope
        return _Plan(tel.resolution, self.resolution, self._cam_eff, self._effective_mask(), path,
                     tel.resolution / tel.initial_resolution, self.psfCentering)

    # ------------------------------------------------------------------ modulation
    @property
    def modulation(self):
        return self._modulation

    @modulation.setter
    def modulation(self, val):
        self._modulation = val
        if self._modulation >= (self.telescope.resolution // 2):
            raise OopaoError('Error the modulation radius is too large for this resolution!'
                             'Consider using a larger telescope resolution!')
        if val != 0 or self.user_modulation_path is not None:
            if self.user_modulation_path is not None:
                path = [list(p) for p in self.user_modulation_path]
                self.nTheta = len(path)
            else:
                perimeter = self.modulation_length * self._modulation
                if self.nTheta_user_defined is None:
                    self.nTheta = 4 * int((self.extraModulationFactor + np.ceil(perimeter / 4)))
                else:
                    self.nTheta = self.nTheta_user_defined
                self.thetaModulation = np.linspace(0 + self.delta_theta, 2 * np.pi + self.delta_theta,
                                                   self.nTheta, endpoint=False)
                path = [[self.modulation * np.cos(t) + self.delta_Tip,
                         self.modulation * np.sin(t) + self.delta_Tilt] for t in self.thetaModulation]
            self.modulation_path = path
        else:
            self.nTheta = 1
            self.modulation_path = None
        self._plan = None
        if getattr(self, 'isCalibrated', False):
            self.slopesUnits = 1
            self.referenceSignal = 0
            self.referenceSignal_2D = 0
            self.wfs_calibration()

    @property
    def spatialFilter(self):
        return self._spatialFilter

    @spatialFilter.setter
    def spatialFilter(self, val):
        """``spatialFilter`` setter (OOPAO/Pyramid.py:1051-1085): the mask becomes
        initial_mask * val (or initial_mask again for None / a wrong shape) and
        a calibrated sensor is recalibrated."""
        self._spatialFilter = val
        if not getattr(self, 'isInitialized', False):
            return
        if val is None:
            print('No spatial filter considered')
            self.mask = self.initial_mask
        elif np.shape(val) == self.mask.shape:
            print('A spatial filter is now considered')
            self.mask = self.initial_mask * val
        else:
            warning('Wrong shape for the spatial filter. No spatial filter attached to the mask')
            self.mask = self.initial_mask
        self._plan = None
        if self.isCalibrated:
            print('Updating the reference slopes and Wavelength Calibration for the new modulation...')
            self.slopesUnits = 1
            self.referenceSignal = 0
            self.referenceSignal_2D = 0
            self.wfs_calibration()
            print('Done!')

    @property
    def delta_Tip(self):
        return self._delta_Tip

    @delta_Tip.setter
    def delta_Tip(self, val):
        self._delta_Tip = val
        if self.isCalibrated:
            self.modulation = self.modulation

    @property
    def delta_Tilt(self):
        return self._delta_Tilt

    @delta_Tilt.setter
    def delta_Tilt(self, val):
        self._delta_Tilt = val
        if self.isCalibrated:
            self.modulation = self.modulation

    @property
    def lightRatio(self):
        return self._lightRatio

    @lightRatio.setter
    def lightRatio(self, val):
        self._lightRatio = val
        if self.isInitialized:
            self._select_valid(self.initFrame)
            self._configure_signal()

    @property
    def plan(self):
        if self._plan is None:
            self._plan = self._make_plan(self.modulation_path)
            self._signal_configured = False
        return self._plan

    @property
    def weight_vector(self):
        return self._weight_vector

    @weight_vector.setter
    def weight_vector(self, val):
        """Weights of the modulation points in the measurement of one
        wavefront: raw = sum_k w_k I_k / nTheta (OOPAO/Pyramid.py:750-755).
        As in the reference, a batch of wavefronts (its 3-D phase path, the
        one the interaction matrix takes) sums the points unweighted."""
        self._weight_vector = None if val is None else np.asarray(val, dtype=np.float64).ravel()

    def _weighted_plan(self, single):
        """The plan with the weights of a single-wavefront (True) or a batch
        (False) measurement in place."""
        plan = self.plan
        w = self._weight_vector
        plan.set_weights(w / self.nTheta if single and w is not None else None)
        return plan

    @property
    def mask(self):
        return self._mask

    @mask.setter
    def mask(self, val):
        """The complex focal-plane mask; assigning a new one takes effect at
        the next measurement, as the reference's attribute does."""
        self._mask = val
        self._plan = None

    # ------------------------------------------------------------------ geometry of quadrants
    def _quadrant_origins(self):
        res, ns = self.telescope.resolution, self.nSubap
        nE = int(np.round((self.n_pix_separation / ns) * res / (res / ns) / 2 / self.binning))
        cp = int(np.round((self.cam.resolution / self.binning) / 2))
        npx = int(np.ceil(ns / self.binning))
        o = {1: (-nE + cp - npx, -nE + cp - npx), 2: (-nE + cp - npx, nE + cp),
             3: (nE + cp, nE + cp), 4: (nE + cp, -nE + cp - npx)}
        for q, (r, c) in o.items():
            if r < 0 or c < 0 or r + npx > self._cam_eff or c + npx > self._cam_eff:
                raise OopaoError('Pyramid quadrant %d falls outside the detector' % q)
        return npx, np.array([o[1], o[2], o[3], o[4]], dtype=np.int32).reshape(-1)

    def grabQuadrant(self, n, cameraFrame=None):
        npx, org = self._quadrant_origins()
        f = self.cam.frame if cameraFrame is None else cameraFrame
        r, c = org[2 * (n - 1)], org[2 * (n - 1) + 1]
        return f[r:r + npx, c:c + npx]

    def grabFullQuadrant(self, n, cameraFrame=None):
        """Half-frame block n of a camera frame (OOPAO/Pyramid.py:963-976); the
        half size is taken from the camera's resolution, the negative starts
        as -n_tot // 2 (one more pixel for an odd size), as in the reference."""
        n_tot = self.cam.resolution
        f = np.array(self.cam.frame) if cameraFrame is None else cameraFrame
        if n == 3:
            return f[:n_tot // 2, :n_tot // 2]
        if n == 4:
            return f[:n_tot // 2, -n_tot // 2:]
        if n == 1:
            return f[-n_tot // 2:, -n_tot // 2:]
        if n == 2:
            return f[-n_tot // 2:, :n_tot // 2]
        raise OopaoError('quadrant number must be 1, 2, 3 or 4')

    def signalProcessing(self, cameraFrame=None):
        """(signal_2D, signal) of a camera frame through the signal kernel,
        float64 host arrays (OOPAO/Pyramid.py:835-926).  As in the reference,
        the slopes-maps modes read their quadrants (and the camera_flux
        normalisation) from the camera's own frame whatever the argument; the
        full-frame modes map the argument, fullFrame_camera_flux and
        fullFrame_sum_flux normalised by the camera frame's mean or sum."""
        own = self.cam.frame
        if own is None:
            raise OopaoError('The camera has no frame yet')
        full = self.postProcessing.startswith('fullFrame')
        use_arg = full and cameraFrame is not None
        f = np.asarray(cameraFrame if use_arg else own, dtype=np.float64)
        if f.shape != np.shape(own):
            raise OopaoError('cameraFrame must have the camera frame shape %s' % (np.shape(own),))
        x = torch.as_tensor(np.ascontiguousarray(f, dtype=np.float32), device=self._dev)[None]
        s2d, sig = self._signals(x)
        s2d = s2d[0].to('cpu', torch.float64).numpy()
        if use_arg and self.postProcessing in ('fullFrame_camera_flux', 'fullFrame_sum_flux'):
            own = np.asarray(own, dtype=np.float64)
            if self.postProcessing == 'fullFrame_camera_flux':
                ratio = f.mean() / own.mean()
            else:
                ratio = f.sum() / own.sum()
            ref = self.referenceSignal_2D
            s2d = (s2d + ref) * ratio - ref
            return s2d, s2d[np.where(self.validSignal == 1)]
        return s2d, sig[0].to('cpu', torch.float64).numpy()

    # ------------------------------------------------------------------ device measurement
    def _amplitude_key(self):
        return (id(self.src), self.src._intensity_version)

    def _measure_frames(self, opd_dev, scale, plan=None, want_raw=False, want_focal=False):
        plan = plan or self._weighted_plan(opd_dev.ndim == 2)
        if self.src.intensity is None:
            raise OopaoError('No flux: propagate the source through the telescope first (src**tel)')
        plan.set_amplitude(self.src.intensity, self._amplitude_key())
        x = opd_dev if opd_dev.ndim == 3 else opd_dev[None]
        x = x.contiguous()
        B = x.shape[0]
        cam = self._cam_eff
        frame = torch.empty((B, cam, cam), dtype=torch.float32, device=self._dev)
        raw = torch.empty((B, self.resolution, self.resolution), dtype=torch.float32,
                          device=self._dev) if want_raw else None
        nb = plan.workspace_bytes(min(B, self.max_batch))
        ws = self._ws.get(nb)
        if want_focal:
            focal = torch.empty((B, self.resolution, self.resolution), dtype=torch.float32, device=self._dev)
            N.call('oopao_pwfs_measure_focal', plan.h, N.ptr(x), float(scale), B, N.ptr(frame), N.ptr(raw),
                   N.ptr(focal), N.ptr(ws), nb, N.stream_handle())
            return frame, raw, focal
        N.call('oopao_pwfs_measure', plan.h, N.ptr(x), float(scale), B, N.ptr(frame), N.ptr(raw),
               N.ptr(ws), nb, N.stream_handle())
        return frame, raw

    def _focal_device(self):
        """Sum over modulation points of |F_k/N|^2 for the last measured
        wavefront, float32 device tensor [N,N] (or [B,N,N])."""
        last = getattr(self, '_last_measure', None)
        if last is None:
            raise OopaoError('No wavefront measured yet')
        opd, scale = last
        _, _, focal = self._measure_frames(opd, scale, want_focal=True)
        img = focal[0] if opd.ndim == 2 else focal
        if not self.psfCentering and self.spatialFilter is not None:
            f = torch.as_tensor(np.abs(np.asarray(self.spatialFilter)) ** 2, dtype=torch.float32, device=self._dev)
            img = img * f
        return img

    def focal_plane_image(self):
        """Sum over modulation points of |F_k/N|^2 for the last measured wavefront
        (the intensity the reference's focal-plane camera reads from
        modulation_camera_em, OOPAO/Pyramid.py:642, :1182-1190), [N,N] float64.
        In the 1-pixel-centred branch the field carries the spatial filter."""
        a = self._focal_device().double().cpu().numpy()
        return np.moveaxis(a, 0, -1) if a.ndim == 3 else a

    def get_modulation_frame(self, radius=6, norma=True):
        """Zoom of the focal-plane camera frame on +-radius lambda/D
        (OOPAO/Pyramid.py:928-944)."""
        if radius <= 0:
            warning('radius for the field of view must be a strictly positive number. Ignoring the input value.')
            radius = self.telescope.resolution // 2
        self.modulation_camera_frame = np.asarray(self.focal_plane_camera.frame, dtype=float)
        n_trunc = int(self.resolution / 2 - radius * self.zeroPaddingFactor)
        if n_trunc <= 0:
            warning('radius Value is too high as the field of view is limited to ' + str(int(self.fov_l_d / 2)) +
                    ' lambda/D -- ignoring')
            zoom = self.modulation_camera_frame.copy()
        else:
            zoom = self.modulation_camera_frame[n_trunc:-n_trunc, n_trunc:-n_trunc]
        if norma:
            zoom = zoom / zoom.max()
        return zoom

    def _select_valid(self, frame):
        """Valid pixels from a camera frame (OOPAO/Pyramid.py:557-579)."""
        self.initFrame = frame
        if self.postProcessing[:10] == 'slopesMaps':
            I4Q = sum(self.grabQuadrant(q, frame) for q in (1, 2, 3, 4))
            self.I4Q = I4Q
            self.validI4Q = I4Q >= self._lightRatio * I4Q.max()
            self.validSignal = np.concatenate((self.validI4Q, self.validI4Q))
        else:
            self.validSignal = frame >= self._lightRatio * frame.max()
        self.validPix = frame >= self._lightRatio * frame.max()
        self.nSignal = int(np.sum(self.validSignal))

    def _norma_const(self):
        sub = (self.telescope.D / self.nSubap) ** 2
        v = self.src.nPhoton * self.telescope.samplingTime * sub
        return v / 4 if self.postProcessing == 'fullFrame_incidence_flux' else v

    def _configure_signal(self, plan=None):
        plan = plan or self.plan
        mode = SP_MODES[self.postProcessing]
        ref = self.referenceSignal_2D
        ref_arr = None if np.isscalar(ref) else N.host(ref, np.float32)
        if mode <= 2:
            npx, org = self._quadrant_origins()
            valid = N.host(self.validI4Q, np.uint8)
            org = N.host(org, np.int32)
            N.call('oopao_pwfs_set_signal_processing', plan.h, mode, npx, org, valid, ref_arr,
                   float(self.slopesUnits), float(self._norma_const()))
        else:
            valid = N.host(self.validSignal, np.uint8)
            N.call('oopao_pwfs_set_signal_processing', plan.h, mode, 0, None, valid, ref_arr,
                   float(self.slopesUnits), float(self._norma_const()))
        self._signal_configured = True

    def _signals(self, frame_dev, plan=None):
        plan = plan or self.plan
        if not getattr(self, '_signal_configured', False):
            self._configure_signal(plan)
        B = frame_dev.shape[0]
        n2d = self.validSignal.size
        ns = N.load().oopao_pwfs_n_signal(plan.h)
        s2d = torch.empty((B, n2d), dtype=torch.float32, device=self._dev)
        sig = torch.empty((B, ns), dtype=torch.float32, device=self._dev)
        N.call('oopao_pwfs_signal', plan.h, N.ptr(frame_dev), B, N.ptr(s2d), N.ptr(sig), None,
               N.stream_handle())
        return s2d.view((B,) + self.validSignal.shape), sig

    # ------------------------------------------------------------------ reference API
    def initialization(self):
        self.src ** self.telescope
        if self.userValidSignal is None:
            if self._lightRatio == 0:
                frame = np.ones([self._cam_eff, self._cam_eff])
            else:
                self.modulation = self.calibModulation
                f, _ = self._measure_frames(self.src.device_opd(self._dev),
                                            2 * np.pi / self.src.wavelength)
                f = self.cam._integrate_device(f, dt=self.telescope.samplingTime)
                frame = f[0].to('cpu', torch.float64).numpy()
                self.cam._set_device_frame(f)
            self._select_valid(frame)
        else:
            if self.postProcessing[:10] == 'slopesMaps':
                self.validI4Q = np.asarray(self.userValidSignal).astype(bool)
                self.validSignal = np.concatenate((self.validI4Q, self.validI4Q))
            else:
                self.validSignal = np.asarray(self.userValidSignal).astype(bool)
            self.nSignal = int(np.sum(self.validSignal))
            self.initFrame = None
        self._signal_configured = False
        self.isInitialized = True

    def wfs_calibration(self, src=None):
        tmp_dev = (self.src._dev, self.src._dev_fresh, self.src._opd, self.src._opd_np, self.src._opd_zero)
        if src is None:
            self.src ** self.telescope
        else:
            self.src = src
        self.referenceSignal_2D = 0
        self._signal_configured = False
        frame, raw = self._measure_frames(self.src.device_opd(self._dev), 2 * np.pi / self.src.wavelength,
                                          want_raw=True)
        s2d, sig = self._signals(frame)
        self.referenceSignal_2D = s2d[0].to('cpu', torch.float64).numpy()
        self.referenceSignal = sig[0].to('cpu', torch.float64).numpy()
        self.referencePyramidFrame = raw[0].to('cpu', torch.float64).numpy()
        self._signal_configured = False
        self.isCalibrated = True
        (self.src._dev, self.src._dev_fresh, self.src._opd, self.src._opd_np, self.src._opd_zero) = tmp_dev

    def wfs_measure(self, phase_in=None, integrate=True):
        if self.isInitialized and self.isCalibrated and self.wavelength_calibration != self.src.wavelength:
            raise OopaoError('A change in wavelength was detected in the WFS object \n'
                             'Make sure that the correct source is propagated in the WFS object or '
                             're-calibrate with the correct source.')
        if phase_in is not None:
            if torch.is_tensor(phase_in):
                opd, scale = phase_in.to(self._dev, torch.float32), 1.0
            else:
                self.src.phase = phase_in
                opd, scale = self.src.device_opd(self._dev), 2 * np.pi / self.src.wavelength
        else:
            opd, scale = self.src.device_opd(self._dev), 2 * np.pi / self.src.wavelength
        single = opd.ndim == 2
        self._last_measure = (opd, scale)
        want_raw = self.keep_raw_data and (single or opd.shape[0] == 1)
        frame, raw = self._measure_frames(opd, scale, want_raw=want_raw)
        frame = self.cam._integrate_device(frame, dt=self.telescope.samplingTime)
        self.cam._set_device_frame(frame if not single else frame)
        self._raw_dev = raw
        self._raw_host = None
        if integrate and self.isInitialized and self.isCalibrated:
            s2d, sig = self._signals(frame)
            self._set_signals(s2d, sig, single)
        return

    def _set_signals(self, s2d, sig, single):
        self._s2d_dev = s2d[0] if single else s2d
        self._sig_dev = sig[0] if single else sig
        self._s2d_host = None
        self._sig_host = None

    # ---------------------------------------------------------------- outputs
    @property
    def device_signal(self):
        return self._sig_dev

    @property
    def device_signal_2D(self):
        return self._s2d_dev

    @property
    def signal(self):
        if getattr(self, '_sig_host', None) is None and getattr(self, '_sig_dev', None) is not None:
            a = self._sig_dev.detach().to('cpu', torch.float64).numpy()
            self._sig_host = a.T if a.ndim == 2 else a
        return getattr(self, '_sig_host', None)

    @signal.setter
    def signal(self, val):
        self._sig_host = val
        self._sig_dev = None

    @property
    def signal_2D(self):
        if getattr(self, '_s2d_host', None) is None and getattr(self, '_s2d_dev', None) is not None:
            a = self._s2d_dev.detach().to('cpu', torch.float64).numpy()
            self._s2d_host = np.moveaxis(a, 0, -1) if a.ndim == 3 else a
        return getattr(self, '_s2d_host', None)

    @signal_2D.setter
    def signal_2D(self, val):
        self._s2d_host = val
        self._s2d_dev = None

    @property
    def pyramidSignal(self):
        return self.signal

    @property
    def pyramidSignal_2D(self):
        return self.signal_2D

    @property
    def raw_data(self):
        if getattr(self, '_raw_host', None) is None and getattr(self, '_raw_dev', None) is not None:
            self._raw_host = self._raw_dev[0].to('cpu', torch.float64).numpy()
        return getattr(self, '_raw_host', None)

    @property
    def pyramidFrame(self):
        return self.raw_data

    @property
    def valid_signal_2D(self):
        return self.validSignal

    # ---------------------------------------------------------------- operators
    def relay(self, src):
        if src.tag != 'source':
            raise OopaoError('Asterisms are not supported by the oopao_gb300 Pyramid')
        src.optical_path.append([self.tag, self])
        self.src = src
        self.wfs_measure()

    @property
    def frames(self):
        return self.cam.frame

    def __mul__(self, obj):
        if obj.tag == 'detector':
            if obj.is_focal_plane_camera:
                # OOPAO/Pyramid.py:1182-1190: centred crop of the focal-plane
                # intensity to the camera size, then the camera's integration
                intensity = self._focal_device()
                if intensity.ndim == 3:
                    intensity = intensity.sum(dim=0)
                n = intensity.shape[0]
                if obj.resolution > self.resolution:
                    frame = intensity
                    warning('Maximum resolution for focal plane camera is %i, cropping field to this dimension'
                            % self.resolution)
                else:
                    h = obj.resolution // 2
                    frame = intensity[n // 2 - h:n // 2 + h, n // 2 - h:n // 2 + h]
                obj._integrated_time = getattr(obj, '_integrated_time', 0) + self.telescope.samplingTime
                obj.integrate(frame)
                return
            if obj is not self.cam:
                raise OopaoError('Only the pyramid camera wfs.cam is supported')
            return
        raise OopaoError('Error light propagated to the wrong type of object')

    def print_properties(self):
        print(self)

    def __repr__(self):
        return ('Pyramid(nSubap=%d, N=%d, cam=%d, modulation=%.1f l/D, nTheta=%d, nSignal=%d, %s)'
                % (self.nSubap, self.resolution, self.cam.resolution, self.modulation, self.nTheta,
                   self.nSignal if self.isInitialized else -1, self.postProcessing))
