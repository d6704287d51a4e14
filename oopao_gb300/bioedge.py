"""Bi-O Edge wavefront sensor: drop-in for the reference ``BioEdge``
(``OOPAO/BioEdge.py``) on the same GPU pipeline as the pyramid.

Per modulation point the reference forms the focal field once and filters it
by four Fourier masks (two complementary half-plane amplitude edges, their
transposes, optional grey transition and tilt), each giving a pupil image;
the four images are tiled 2x2 into the raw frame (``bio_edge_transform``
:510-544).  Sum-binning is local and the tile size N is a multiple of the
binning factor, so each camera quadrant is exactly the binned image of one
mask: here every mask is one ``oopao_pwfs_plan`` (same modulation path, the
reference's sqrt(0.5) field amplitude) and the four camera tiles are written
side by side.  The slopes use the reference's ``grabQuadrant`` (:840-853),
four (cam/2)-pixel blocks of the first tile, through the plan's signal
kernel.
"""
import numpy as np
import torch

from . import _native as N
from .detector import Detector
from .pyramid import _Plan
from .runtime import Workspace, device
from .tools import OopaoError, warning

_MODES = {'slopesMaps': 0, 'slopesMaps_incidence_flux': 1}


def bioedge_masks(n_fft, res, n_subap, zero_padding_factor, grey_width=0., grey_length=False,
                  quadrants_numbering=(0, 1, 2, 3), sx=(0, 0, 0, 0), sy=(0, 0, 0, 0), initial_res=None):
    """The four complex Fourier masks [4, N, N] (``mask_computation`` :331-392)."""
    N_ = n_fft
    initial_res = res if initial_res is None else initial_res
    norma = (n_subap * 2) * (res / n_subap) * (1 / (n_subap * 2))
    g = np.linspace(-np.pi, np.pi, N_, endpoint=False)
    tip, tilt = np.meshgrid(g, g)
    bw = np.zeros(N_)
    bw[0:N_ // 2] = 1.
    r = int(np.round(zero_padding_factor * grey_width * res / initial_res))
    if grey_width != 0:
        bw[N_ // 2 - r:N_ // 2 + r] = np.hstack([np.linspace(1, 0.5, r, endpoint=True),
                                                np.linspace(0.5, 0, r, endpoint=True)])
    a = np.sqrt(np.meshgrid(bw, bw)[0])
    if grey_length is not False:
        rl = int(np.round(zero_padding_factor * grey_length))
        a[0:N_ // 2 - rl, 0:N_ // 2] = 1.
        a[N_ // 2 + rl:, 0:N_ // 2] = 1.
        a[0:N_ // 2 - rl, N_ // 2:] = 0.
        a[N_ // 2 + rl:, N_ // 2:] = 0.
    b = np.sqrt(1 - a ** 2)
    base = [a, b, a.T.copy(), b.T.copy()]
    if np.isscalar(sx):
        sx = [sx] * 4
    if np.isscalar(sy):
        sy = [sy] * 4
    tts = [-sx[3] * tip * norma + sy[3] * tilt * norma, -sx[2] * tip * norma + sy[2] * tilt * norma,
           -sx[1] * tip * norma + sy[1] * tilt * norma, -sx[0] * tip * norma + sy[0] * tilt * norma]
    return [base[quadrants_numbering[i]] * np.exp(1j * tts[i]) for i in range(4)]


class BioEdge:
    def __init__(self, nSubap: float, telescope, modulation: float, lightRatio: float,
                 postProcessing: str = 'slopesMaps', n_pix_separation: float = 2., n_pix_edge: float = None,
                 calibModulation: float = 50., extraModulationFactor: int = 0, binning: int = 1,
                 nTheta_user_defined: int = None, userValidSignal: bool = None, grey_width: float = 0,
                 grey_length: bool = False, delta_theta: float = 0., user_modulation_path: list = None,
                 quadrants_numbering: list = [0, 1, 2, 3], max_batch: int = 64):
        res = telescope.resolution
        if (res / nSubap) % 2 != 0 and res / nSubap != 1:
            raise OopaoError('The resolution should be an even number and be a multiple of 2**i where i>=2')
        if telescope.src is None:
            raise OopaoError('The telescope was not coupled to any source object! Make sure to couple it with an '
                             'src object using src*tel')
        if postProcessing not in _MODES:
            raise OopaoError('oopao_gb300 BioEdge supports postProcessing %s' % sorted(_MODES))
        if binning != 1:
            raise OopaoError('oopao_gb300 BioEdge supports binning=1 only')
        self.telescope = telescope
        self.src = telescope.src
        self.wavelength_calibration = self.src.wavelength
        self.nSubap = nSubap
        self.postProcessing = postProcessing
        self.userValidSignal = userValidSignal
        self.psfCentering = True
        self.binning = binning
        self.quadrants_numbering = list(quadrants_numbering)
        self.user_modulation_path = user_modulation_path
        self.nTheta_user_defined = nTheta_user_defined
        self.extraModulationFactor = extraModulationFactor
        self.delta_theta = delta_theta
        self.weight_vector = None
        self.n_pix_separation = n_pix_separation
        self.n_pix_edge = n_pix_separation // 2 if n_pix_edge is None else n_pix_edge
        if n_pix_edge is not None and n_pix_edge != n_pix_separation // 2:
            warning('The recommanded value for n_pix_edge is ' + str(n_pix_separation // 2) + ' instead of ' +
                    str(n_pix_edge))
        self.sx = [0, 0, 0, 0]
        self.sy = [0, 0, 0, 0]
        self.grey_width = grey_width
        self.grey_length = grey_length
        self.resolution = int((nSubap * 2 + n_pix_separation + self.n_pix_edge * 2) * res / nSubap)
        self.zeroPaddingFactor = self.resolution / res
        self.zeroPadding = (self.resolution - res) // 2
        self.tag = 'pyramid'
        self.cam = Detector(round(nSubap * self.zeroPaddingFactor))
        self._cam_eff = self.cam.resolution
        self.cam._frame_host = np.zeros([2 * self._cam_eff, 2 * self._cam_eff])
        self.focal_plane_camera = Detector(int((modulation * 4 + 12) * self.zeroPaddingFactor))
        self.focal_plane_camera.is_focal_plane_camera = True
        self.fov_l_d = self.resolution / self.zeroPaddingFactor
        self._lightRatio = lightRatio
        self.calibModulation = res / 2 - 1 if calibModulation >= res / 2 else calibModulation
        self.isInitialized = False
        self.isCalibrated = False
        self._delta_Tip = 0
        self._delta_Tilt = 0
        self.max_batch = max_batch
        self.keep_raw_data = True
        self._dev = device()
        self._ws = Workspace()
        self._plans = None
        self._shared_forward = False
        self._signal_configured = False
        self.mask_computation()
        self.slopesUnits = 1
        self.referenceSignal = 0
        self.referenceSignal_2D = 0
        self.modulation = modulation
        self.initialization()
        self.modulation = modulation
        self.wfs_calibration()
        self.src ** self.telescope
        self.wfs_measure()

    # ------------------------------------------------------------------ masks / plans
    def mask_computation(self, sx=[0] * 4, sy=[0] * 4):
        self.mask = bioedge_masks(self.resolution, self.telescope.resolution, self.nSubap, self.zeroPaddingFactor,
                                  self.grey_width, self.grey_length, self.quadrants_numbering, sx, sy,
                                  self.telescope.initial_resolution)
        self.initial_mask = [m.copy() for m in self.mask]
        self._plans = None

    @property
    def plans(self):
        """One plan holding the four masks (forward transforms shared), or,
        for FFT sizes without a several-mask column pass, one plan per mask."""
        if self._plans is None:
            tel = self.telescope
            mk = lambda m: _Plan(tel.resolution, self.resolution, self._cam_eff, m, self.modulation_path,
                                 tel.resolution / tel.initial_resolution, True)
            p0 = mk(self.mask[0])
            try:
                N.call('oopao_pwfs_set_masks', p0.h, len(self.mask),
                       np.ascontiguousarray(np.stack(self.mask), dtype=np.complex64))
                self._plans, self._shared_forward = [p0], True
            except OopaoError:
                self._plans, self._shared_forward = [p0] + [mk(m) for m in self.mask[1:]], False
            self._signal_configured = False
        return self._plans

    @property
    def plan(self):
        return self.plans[0]

    def _weighted_plans(self, single):
        """The plans with the weights of a single-wavefront (True) or a batch
        (False) measurement in place (BioEdge.py:643-648 weights one 2-D
        phase only)."""
        plans = self.plans
        w = self._weight_vector
        for p in plans:
            p.set_weights(w / self.nTheta if single and w is not None else None)
        return plans

    @property
    def weight_vector(self):
        return self._weight_vector

    @weight_vector.setter
    def weight_vector(self, val):
        self._weight_vector = None if val is None else np.asarray(val, dtype=np.float64).ravel()

    @property
    def mask(self):
        return self._mask

    @mask.setter
    def mask(self, val):
        """The four complex masks; a new list takes effect at the next
        measurement."""
        self._mask = val
        self._plans = None

    def apply_shift_wfs(self, sx=None, sy=None, mis_reg=None, units='pixels'):
        """Moves the four pupil images by a tip/tilt on each mask
        (BioEdge.py:394-433).  As in the reference, the masks are rebuilt
        from sx, sy as given (one value or four); units only scales the
        shifts recorded in self.sx / self.sy and the range warning.  The
        reference slopes are measured again."""
        sx = 0 if sx is None else sx
        sy = 0 if sy is None else sy
        if mis_reg is not None:
            sx = [mis_reg.dX_1, mis_reg.dX_2, mis_reg.dX_3, mis_reg.dX_4]
            sy = [mis_reg.dY_1, mis_reg.dY_2, mis_reg.dY_3, mis_reg.dY_4]
        f = 2
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
        if np.max(np.abs(shift_x) / factor) > self.n_pix_edge or np.max(np.abs(shift_y) / factor) > self.n_pix_edge:
            warning('The Bi-O Edge pupils have been shifted outside of the detector!'
                    'Wrapping of the signal is currently occuring!!')
        self.mask_computation(sx=sx, sy=sy)
        self.sx = np.asarray(shift_x) / factor
        self.sy = np.asarray(shift_y) / factor
        self.slopesUnits = 1
        self.referenceSignal = 0
        self.referenceSignal_2D = 0
        self.wfs_calibration()

    # ------------------------------------------------------------------ modulation (BioEdge.py:963-1009)
    @property
    def modulation(self):
        return self._modulation

    @modulation.setter
    def modulation(self, val):
        self._modulation = val
        if val >= self.telescope.resolution // 2:
            raise OopaoError('Error the modulation radius is too large for this resolution!' +
                             'Consider using a larger telescope resolution!')
        if val != 0 or self.user_modulation_path is not None:
            if self.user_modulation_path is not None:
                path = [list(p) for p in self.user_modulation_path]
                self.nTheta = len(path)
            else:
                perimeter = np.pi * 2 * val
                self.nTheta = (4 * int(self.extraModulationFactor + np.ceil(perimeter / 4))
                               if self.nTheta_user_defined is None else self.nTheta_user_defined)
                self.thetaModulation = np.linspace(self.delta_theta, 2 * np.pi + self.delta_theta, self.nTheta,
                                                   endpoint=False)
                path = [[val * np.cos(t) + self._delta_Tip, val * np.sin(t) + self._delta_Tilt]
                        for t in self.thetaModulation]
            self.modulation_path = path
        else:
            self.nTheta = 1
            self.modulation_path = None
        self._plans = None
        if getattr(self, 'isCalibrated', False):
            self.slopesUnits = 1
            self.referenceSignal = 0
            self.referenceSignal_2D = 0
            self.wfs_calibration()

    @property
    def delta_Tip(self):
        return self._delta_Tip

    @delta_Tip.setter
    def delta_Tip(self, val):
        """Offset of the modulation circle along x (BioEdge.py:933-941); a
        calibrated sensor rebuilds its path and reference slopes."""
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

    # ------------------------------------------------------------------ propagation
    def _amplitude_key(self):
        return ('bioedge', id(self.src), self.src._intensity_version)

    def _measure_frames(self, opd_dev, scale, want_raw=False):
        """Camera frames [B, 2cam, 2cam] (and raw [B, 2N, 2N]) for device OPDs."""
        if self.src.intensity is None:
            raise OopaoError('No flux: propagate the source through the telescope first (src**tel)')
        half = 0.5 * np.asarray(self.src.intensity, dtype=np.float64)   # the reference's sqrt(0.5) field
        x = opd_dev if opd_dev.ndim == 3 else opd_dev[None]
        x = x.contiguous()
        B, cam, n = x.shape[0], self._cam_eff, self.resolution
        plans = self._weighted_plans(opd_dev.ndim == 2)
        if self._shared_forward:
            # one launch sequence; tiles [B][4][.][.] laid out 2 x 2
            plan = plans[0]
            plan.set_amplitude(half, self._amplitude_key())
            tiles = torch.empty((B, 4, cam, cam), dtype=torch.float32, device=self._dev)
            rtiles = torch.empty((B, 4, n, n), dtype=torch.float32, device=self._dev) if want_raw else None
            nb = plan.workspace_bytes(min(B, self.max_batch))
            ws = self._ws.get(nb)
            N.call('oopao_pwfs_measure', plan.h, N.ptr(x), float(scale), B, N.ptr(tiles), N.ptr(rtiles), N.ptr(ws),
                   nb, N.stream_handle())
            frame = tiles.view(B, 2, 2, cam, cam).permute(0, 1, 3, 2, 4).reshape(B, 2 * cam, 2 * cam)
            raw = rtiles.view(B, 2, 2, n, n).permute(0, 1, 3, 2, 4).reshape(B, 2 * n, 2 * n) if want_raw else None
            return frame, raw
        frame = torch.empty((B, 2 * cam, 2 * cam), dtype=torch.float32, device=self._dev)
        raw = torch.empty((B, 2 * n, 2 * n), dtype=torch.float32, device=self._dev) if want_raw else None
        tile = torch.empty((B, cam, cam), dtype=torch.float32, device=self._dev)
        rtile = torch.empty((B, n, n), dtype=torch.float32, device=self._dev) if want_raw else None
        for q, plan in enumerate(plans):
            plan.set_amplitude(half, self._amplitude_key())
            nb = plan.workspace_bytes(min(B, self.max_batch))
            ws = self._ws.get(nb)
            N.call('oopao_pwfs_measure', plan.h, N.ptr(x), float(scale), B, N.ptr(tile), N.ptr(rtile), N.ptr(ws), nb,
                   N.stream_handle())
            i, j = divmod(q, 2)
            frame[:, i * cam:(i + 1) * cam, j * cam:(j + 1) * cam] = tile
            if want_raw:
                raw[:, i * n:(i + 1) * n, j * n:(j + 1) * n] = rtile
        return frame, raw

    # ------------------------------------------------------------------ focal-plane camera
    def _focal_plan(self):
        """One-mask plan for the focal-plane intensity: the field before the
        masks is the same for the four of them.  Rebuilt with the masks'
        plans (mask, modulation or geometry changes)."""
        plans = self.plans
        if getattr(self, '_focal_for', None) is not plans:
            tel = self.telescope
            self._focal = _Plan(tel.resolution, self.resolution, self._cam_eff, self.mask[0], self.modulation_path,
                                tel.resolution / tel.initial_resolution, True)
            self._focal_for = plans
        return self._focal

    def _focal_device(self):
        """Focal-plane intensity of the last measured wavefront, float32 device
        tensor [N,N] (or [B,N,N]).  The reference keeps each modulation point's
        focal field fft2(sqrt(0.5) A exp(i phi) phasor) once per mask
        (OOPAO/BioEdge.py:435-443) and sums |.|^2 over that list, unweighted
        (:1036-1038): 4 N^2 times the sum over points of |F_k/N|^2 of the
        sqrt(0.5) field, which the plan's focal output gives."""
        last = getattr(self, '_last_measure', None)
        if last is None:
            raise OopaoError('No wavefront measured yet')
        opd, scale = last
        plan = self._focal_plan()
        plan.set_weights(None)
        plan.set_amplitude(0.5 * np.asarray(self.src.intensity, dtype=np.float64), self._amplitude_key())
        x = (opd if opd.ndim == 3 else opd[None]).contiguous()
        B, n = x.shape[0], self.resolution
        frame = torch.empty((B, self._cam_eff, self._cam_eff), dtype=torch.float32, device=self._dev)
        focal = torch.empty((B, n, n), dtype=torch.float32, device=self._dev)
        nb = plan.workspace_bytes(min(B, self.max_batch))
        ws = self._ws.get(nb)
        N.call('oopao_pwfs_measure_focal', plan.h, N.ptr(x), float(scale), B, N.ptr(frame), None, N.ptr(focal),
               N.ptr(ws), nb, N.stream_handle())
        focal *= 4.0 * n * n
        return focal[0] if opd.ndim == 2 else focal

    def get_modulation_frame(self, radius=6, norma=True):
        """Zoom of the focal-plane camera frame on +-radius lambda/D
        (OOPAO/BioEdge.py:822-838)."""
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

    # ------------------------------------------------------------------ signals
    def _quadrant_origins(self):
        cp = int(np.round((self._cam_eff / self.binning) / 2))
        return cp, np.array([0, 0, 0, cp, cp, 0, cp, cp], dtype=np.int32)

    def grabQuadrant(self, n, cameraFrame=None):
        """(cam/2)-pixel block n of the frame (OOPAO/BioEdge.py:840-853)."""
        cp, org = self._quadrant_origins()
        f = self.cam.frame if cameraFrame is None else cameraFrame
        r, c = org[2 * (n - 1)], org[2 * (n - 1) + 1]
        return f[r:r + cp, c:c + cp]

    def grabFullQuadrant(self, n, cameraFrame=None):
        """Half-frame block n of a camera frame (OOPAO/BioEdge.py:855-868), the
        half size from the frame itself, the negative starts as -n_tot // 2."""
        f = np.array(self.cam.frame) if cameraFrame is None else cameraFrame
        n_tot = f.shape[0]
        if n == 4:
            return f[:n_tot // 2, :n_tot // 2]
        if n == 3:
            return f[:n_tot // 2, -n_tot // 2:]
        if n == 1:
            return f[-n_tot // 2:, -n_tot // 2:]
        if n == 2:
            return f[-n_tot // 2:, :n_tot // 2]
        raise OopaoError('quadrant number must be 1, 2, 3 or 4')

    def signalProcessing(self, cameraFrame=None):
        """(signal_2D, signal) through the signal kernel, float64 host arrays
        (OOPAO/BioEdge.py:729-767).  Both supported modes read their quadrants
        from the camera's own frame whatever the argument, as the reference
        does."""
        own = self.cam.frame
        if own is None:
            raise OopaoError('The camera has no frame yet')
        x = torch.as_tensor(np.ascontiguousarray(own, dtype=np.float32), device=self._dev)[None]
        s2d, sig = self._signals(x)
        return s2d[0].to('cpu', torch.float64).numpy(), sig[0].to('cpu', torch.float64).numpy()

    def _norma_const(self):
        return self.src.nPhoton * self.telescope.samplingTime * (self.telescope.D / self.nSubap) ** 2

    def _configure_signal(self):
        ref = self.referenceSignal_2D
        ref_arr = None if np.isscalar(ref) else N.host(ref, np.float32)
        npx, org = self._quadrant_origins()
        N.call('oopao_pwfs_set_signal_processing', self.plan.h, _MODES[self.postProcessing], npx, N.host(org, np.int32),
               N.host(self.validI4Q, np.uint8), ref_arr, float(self.slopesUnits), float(self._norma_const()))
        self._signal_configured = True

    def _signals(self, frame_dev):
        """Slopes of frames [B, 2cam, 2cam]: the quadrants lie in the first tile."""
        if not self._signal_configured:
            self._configure_signal()
        cam = self._cam_eff
        first = frame_dev[:, :cam, :cam].contiguous()
        B = first.shape[0]
        ns = N.load().oopao_pwfs_n_signal(self.plan.h)
        s2d = torch.empty((B, self.validSignal.size), dtype=torch.float32, device=self._dev)
        sig = torch.empty((B, ns), dtype=torch.float32, device=self._dev)
        N.call('oopao_pwfs_signal', self.plan.h, N.ptr(first), B, N.ptr(s2d), N.ptr(sig), None, N.stream_handle())
        return s2d.view((B,) + self.validSignal.shape), sig

    def _select_valid(self, frame):
        self.initFrame = frame
        self.I4Q = sum(self.grabQuadrant(q, frame) for q in (1, 2, 3, 4))
        self.validI4Q = self.I4Q >= self._lightRatio * self.I4Q.max()
        self.validSignal = np.concatenate((self.validI4Q, self.validI4Q))
        self.nSignal = int(np.sum(self.validSignal))
        self._signal_configured = False

    # ------------------------------------------------------------------ reference API
    def initialization(self):
        """Valid pixels on flux at the calibration modulation (BioEdge.py:445-490)."""
        self.src ** self.telescope
        if self.userValidSignal is None:
            if self._lightRatio == 0:
                frame = np.ones([2 * self._cam_eff, 2 * self._cam_eff])
            else:
                self.modulation = self.calibModulation
                f, _ = self._measure_frames(self.src.device_opd(self._dev), 2 * np.pi / self.src.wavelength)
                f = self.cam._integrate_device(f, dt=self.telescope.samplingTime)
                frame = f[0].to('cpu', torch.float64).numpy()
                self.cam._set_device_frame(f)
            self._select_valid(frame)
        else:
            self.validI4Q = np.asarray(self.userValidSignal).astype(bool)
            self.validSignal = np.concatenate((self.validI4Q, self.validI4Q))
            self.nSignal = int(np.sum(self.validSignal))
            self.initFrame = None
        self.isInitialized = True

    def wfs_calibration(self):
        """Flat-wavefront reference slopes at the current modulation (BioEdge.py:492-507)."""
        saved = (self.src._dev, self.src._dev_fresh, self.src._opd, self.src._opd_np, self.src._opd_zero)
        self.src ** self.telescope
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
        (self.src._dev, self.src._dev_fresh, self.src._opd, self.src._opd_np, self.src._opd_zero) = saved

    def wfs_measure(self, phase_in=None, integrate=True):
        if self.isInitialized and self.isCalibrated and self.wavelength_calibration != self.src.wavelength:
            raise OopaoError('A change in wavelength was detected in the WFS object \nMake sure that the correct '
                             'source is propagated in the WFS object or re-calibrate with the correct source.')
        if phase_in is not None:
            if torch.is_tensor(phase_in):
                opd, scale = phase_in.to(self._dev, torch.float32), 1.0
            else:
                self.src.phase = phase_in
                opd, scale = self.src.device_opd(self._dev), 2 * np.pi / self.src.wavelength
        else:
            opd, scale = self.src.device_opd(self._dev), 2 * np.pi / self.src.wavelength
        single = opd.ndim == 2
        want_raw = self.keep_raw_data and (single or opd.shape[0] == 1)
        frame, raw = self._measure_frames(opd, scale, want_raw=want_raw)
        self._last_measure = (opd, scale)
        frame = self.cam._integrate_device(frame, dt=self.telescope.samplingTime)
        self.cam._set_device_frame(frame)
        self._raw_dev = raw
        self._raw_host = None
        if integrate and self.isInitialized and self.isCalibrated:
            s2d, sig = self._signals(frame)
            self._s2d_dev = s2d[0] if single else s2d
            self._sig_dev = sig[0] if single else sig
            self._s2d_host = None
            self._sig_host = None

    # ------------------------------------------------------------------ outputs
    @property
    def device_signal(self):
        return self._sig_dev

    @property
    def signal(self):
        if getattr(self, '_sig_host', None) is None and getattr(self, '_sig_dev', None) is not None:
            a = self._sig_dev.detach().to('cpu', torch.float64).numpy()
            self._sig_host = a.T if a.ndim == 2 else a
        return getattr(self, '_sig_host', None)

    @property
    def signal_2D(self):
        if getattr(self, '_s2d_host', None) is None and getattr(self, '_s2d_dev', None) is not None:
            a = self._s2d_dev.detach().to('cpu', torch.float64).numpy()
            self._s2d_host = np.moveaxis(a, 0, -1) if a.ndim == 3 else a
        return getattr(self, '_s2d_host', None)

    @property
    def raw_data(self):
        if getattr(self, '_raw_host', None) is None and getattr(self, '_raw_dev', None) is not None:
            self._raw_host = self._raw_dev[0].to('cpu', torch.float64).numpy()
        return getattr(self, '_raw_host', None)

    # ------------------------------------------------------------------ operators
    def relay(self, src):
        if src.tag != 'source':
            raise OopaoError('Asterisms are not supported by the oopao_gb300 BioEdge')
        src.optical_path.append([self.tag, self])
        self.src = src
        self.wfs_measure()

    def __mul__(self, obj):
        if obj.tag == 'detector':
            if obj.is_focal_plane_camera:
                # OOPAO/BioEdge.py:1036-1044: centred crop of the focal-plane
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
                raise OopaoError('Only the sensor camera wfs.cam is supported')
            return
        raise OopaoError('Error light propagated to the wrong type of object')

    def __repr__(self):
        return 'BioEdge(nSubap=%d, N=%d, cam=%d, modulation=%.1f l/D, nTheta=%d, nSignal=%d)' % (
            self.nSubap, self.resolution, self._cam_eff, self.modulation, self.nTheta,
            self.nSignal if self.isInitialized else -1)
