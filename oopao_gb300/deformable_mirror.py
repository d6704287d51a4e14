"""Deformable mirror: drop-in for the reference ``DeformableMirror``
(``OOPAO/DeformableMirror.py``) on the PWFS path.

Construction builds the Gaussian influence functions on the host in float64
exactly as the reference (Fried grid and radial actuator selection
:306-340, mis-registration of the grid :359-386, ``modesComputation``
:572-600), or takes user ``modes`` (the grid is still mis-registered, the
modes are not, as in the reference).  The IF
matrix is then kept on the GPU, transposed ([n_act][n_pix]), and every
``dm.coefs = ...`` runs the projection OPD = modes @ coefs on the device.
Gaussian IFs on a Cartesian grid without rotation or anamorphosis angle
factorise as gx(x) gy(y): they are projected exactly by two small
contractions (``oopao_dm_opd_sep_f32``).  Other IFs go through
``oopao_dm_opd_f32`` (FP32) or, with ``if_dtype='bf16'``, the tensor-core
GEMM.  ``dm.OPD`` is materialised on the host only when read.
"""
import numpy as np
import torch

from . import _native as N
from .mis_registration import MisRegistration
from .runtime import device
from .tools import OopaoError, print_


class DeformableMirror:
    def __init__(self, telescope, nSubap: float, mechCoupling: float = 0.35, coordinates=None,
                 pitch: float = None, modes=None, misReg=None, M4_param=None, nJobs: int = 30,
                 nThreads: int = 20, print_dm_properties: bool = True, floating_precision: int = 64,
                 altitude: float = None, flip=False, flip_lr=False, sign=1, actuator_selection=None,
                 user_defined_influence_functions_tag=None, if_dtype: str = 'fp32'):
        if M4_param is not None:
            raise OopaoError('M4 influence functions are not supported by oopao_gb300')
        if altitude is not None:
            raise OopaoError('Altitude-conjugated DMs are not supported by oopao_gb300')
        if mechCoupling <= 0:
            raise OopaoError('The value of mechanical coupling should be positive.')
        self.telescope = telescope
        self.altitude = None
        self.print_dm_properties = print_dm_properties
        self.floating_precision = floating_precision
        self.flip_ = flip
        self.flip_lr = flip_lr
        self.sign = sign
        self.actuator_selection = actuator_selection
        self.resolution = telescope.resolution
        self.mechCoupling = mechCoupling
        self.tag = 'deformableMirror'
        self.D = telescope.D
        self.isM4 = False
        self.precision = np.float64
        self.pitch = self.D / nSubap if pitch is None else pitch
        self.if_dtype = if_dtype
        self.misReg = MisRegistration() if misReg is None else misReg
        if coordinates is None:
            self.nAct = nSubap + 1
            self.nActAlongDiameter = self.nAct - 1
            x = np.linspace(-self.D / 2, self.D / 2, self.nAct)
            X, Y = np.meshgrid(x, x)
            self.xIF0 = np.reshape(X, [self.nAct ** 2])
            self.yIF0 = np.reshape(Y, [self.nAct ** 2])
            r = np.sqrt(self.xIF0 ** 2 + self.yIF0 ** 2)
            if self.actuator_selection is None:
                r_in = telescope.centralObstruction * telescope.initial_D / 2 - 0.5 * self.pitch
                r_out = telescope.initial_D / 2 + 0.7533 * self.pitch
                self.actuator_selection = [r_in, r_out]
            if np.isscalar(self.actuator_selection):
                self.validAct = np.ones_like(r, dtype=bool)
            else:
                if len(self.actuator_selection) != 2:
                    raise OopaoError('actuator_selection must be either a scalar or a vector of length 2 '
                                     'to specify the inner and outer radius.')
                self.validAct = (r >= self.actuator_selection[0]) * (r <= self.actuator_selection[1])
            self.nValidAct = int(np.sum(self.validAct))
        else:
            coordinates = np.asarray(coordinates)
            if coordinates.ndim != 2 or coordinates.shape[1] != 2:
                raise OopaoError('Wrong size for the DM coordinates, the (x,y) coordinates should be '
                                 'input as a 2D array of dimension [nAct,2]')
            self.xIF0 = coordinates[:, 0]
            self.yIF0 = coordinates[:, 1]
            self.nAct = len(self.xIF0)
            self.nActAlongDiameter = self.D / self.pitch
            self.validAct = np.arange(self.nAct)
            self.nValidAct = self.nAct
        xIF0 = self.xIF0[self.validAct]
        yIF0 = self.yIF0[self.validAct]
        self.nIF = len(xIF0)
        self.initial_coordinates = np.stack([xIF0, yIF0], axis=1)
        # mis-registration of the grid (:359-386): anamorphosis, rotation, shift
        mr = self.misReg
        x3, y3 = self.anamorphosis_coordinates(xIF0, yIF0, mr.anamorphosisAngle * np.pi / 180,
                                               mr.tangentialScaling, mr.radialScaling)
        x4, y4 = self.rotate_coordinates(x3, y3, mr.rotationAngle * np.pi / 180)
        xIF = x4 - mr.shiftX
        yIF = y4 - mr.shiftY
        self.coordinates = np.stack([xIF, yIF], axis=1)
        self.xIF, self.yIF = xIF, yIF
        self._sep_host = None
        self._modes = None
        self._modes_t_dev = None
        if modes is None:
            u0x = self.resolution / 2 + xIF * self.resolution / self.D
            u0y = self.resolution / 2 + yIF * self.resolution / self.D
            self._u0 = (u0x, u0y)
            sep = self._separable_factors(u0x, u0y)
            if np.isscalar(self.actuator_selection):
                std = self._if_std(telescope.pupil, sep)
                keep = np.where(std > self.actuator_selection * np.max(std))[0]
                if self._modes is not None:
                    self._modes = self._modes[:, keep]
                self.validAct = keep
                self.nValidAct = len(keep)
                self.nIF = self.nValidAct
                self.xIF, self.yIF = self.xIF[keep], self.yIF[keep]
                self.coordinates = self.coordinates[keep]
                u0x, u0y = u0x[keep], u0y[keep]
                self._u0 = (u0x, u0y)
                if sep is not None:
                    sep = self._separable_factors(u0x, u0y)
            self._sep_host = sep
            if sep is None and self._modes is None:
                self._modes = self._gaussian_modes(u0x, u0y)
        else:
            self._modes = np.asarray(modes) * self.sign
            self.nValidAct = self._modes.shape[1]
            if self._modes.shape[0] != self.resolution ** 2:
                raise OopaoError('modes must be [resolution**2, n_modes]')
        self._dev = device()
        self._upload_modes()
        # the separable projection serves every batch when the IFs factorise
        self.separable_projection = self._sep_host is not None
        # batches above this go to the BF16 tensor-core GEMM (if_dtype='bf16'),
        # and the GEMM's batch tile per batch size: [(max batch, 64 or 128)],
        # empty for the library's rule; both set by autotune.tune_dm
        self.separable_max_batch = self.SEPARABLE_MAX_BATCH_VS_TC
        self.tf32_min_batch = self.TF32_MIN_BATCH
        self.tc_tile_rule = []
        self._sep = None
        self._sep_ws = None
        if self._sep_host is not None:
            gx, gy, cells = self._sep_host
            self._sep = (torch.as_tensor(gx, dtype=torch.float32, device=self._dev),
                         torch.as_tensor(gy, dtype=torch.float32, device=self._dev),
                         torch.as_tensor(cells, device=self._dev), gx.shape[0], gy.shape[0])
        self._opd_dev = None
        self._opd_host = None
        self._coefs = None
        self.coefs = np.zeros(self.nValidAct, dtype=np.float32 if floating_precision == 32 else np.float64)
        self.current_coefs = self.coefs.copy()
        print_(self, print_dm_properties)

    # ------------------------------------------------------------ IF build
    @property
    def modes(self):
        """Influence functions [res**2, nValidAct] (OOPAO/DeformableMirror.py:
        572-600).  When the Gaussian IFs factorise per axis the projections
        run on the factors, and this dense matrix (9.6 GB in float64 for an
        80x80 DM at 480 px) is built on first access only."""
        if self._modes is None:
            self._modes = self._gaussian_modes(*self._u0)
        return self._modes

    @modes.setter
    def modes(self, value):
        self._modes = value
        self._modes_t_dev = None

    @property
    def _modes_t(self):
        """The IFs transposed, [nValidAct, res**2] float32 on the device (the
        dense FP32 projection and the DM adjoint), uploaded on first use."""
        if self._modes_t_dev is None:
            mt = np.ascontiguousarray(np.asarray(self.modes, dtype=np.float32).T)
            self._modes_t_dev = torch.as_tensor(mt, device=self._dev)
        return self._modes_t_dev

    def _if_std(self, pupil, sep):
        """Standard deviation of each IF over the pupil pixels (the reference's
        actuator selection, np.std(modes[pupil, :], axis=0)), from the factors
        when they exist: with P the pupil, the IF of the actuator in grid cell
        (iy, ix) has mean (gy P gx^T)[iy, ix] / n and second moment
        (gy^2 P (gx^2)^T)[iy, ix] / n."""
        if sep is None:
            pup = pupil.flatten() == 1
            return np.std(self.modes[pup, :], axis=0)
        gx, gy, cells = sep
        P = (np.asarray(pupil) == 1).astype(np.float64)
        n = P.sum()
        m1 = gy @ P @ gx.T / n
        m2 = (gy ** 2) @ P @ (gx ** 2).T / n
        std_cell = np.sqrt(np.maximum(m2 - m1 ** 2, 0.0)).reshape(-1)
        out = np.empty(len(self._u0[0]))
        live = cells >= 0
        out[cells[live]] = std_cell[live]
        return out

    @staticmethod
    def rotate_coordinates(x, y, angle):
        """Rotation of the actuator grid by `angle` radians (:559-562)."""
        return x * np.cos(angle) - y * np.sin(angle), y * np.cos(angle) + x * np.sin(angle)

    @staticmethod
    def anamorphosis_coordinates(x, y, angle, mRad, mNorm):
        """Stretch of the grid by 1+mRad along direction `angle` and 1+mNorm
        across it (:564-570).  The reference passes the tangential scaling as
        mRad and the radial one as mNorm; the same order is kept."""
        mRad = mRad + 1
        mNorm = mNorm + 1
        s2 = np.sin(2 * angle) / 2
        x_out = x * (mRad * np.cos(angle) ** 2 + mNorm * np.sin(angle) ** 2) + y * (mNorm * s2 - mRad * s2)
        y_out = y * (mRad * np.sin(angle) ** 2 + mNorm * np.cos(angle) ** 2) + x * (mNorm * s2 - mRad * s2)
        return x_out, y_out

    def _gaussian_modes(self, u0x, u0y):
        """``modesComputation`` (OOPAO/DeformableMirror.py:572-600): Gaussian
        IFs whose widths are scaled by 1+radialScaling along the anamorphosis
        direction and 1+tangentialScaling across it."""
        res = self.resolution
        w = (self.resolution / self.nActAlongDiameter) / np.sqrt(2 * np.log(1. / self.mechCoupling))
        cx = (1 + self.misReg.radialScaling) * w
        cy = (1 + self.misReg.tangentialScaling) * w
        theta = self.misReg.anamorphosisAngle * np.pi / 180
        x = np.linspace(0, 1, res) * res
        X, Y = np.meshgrid(x, x)
        a = np.cos(theta) ** 2 / (2 * cx ** 2) + np.sin(theta) ** 2 / (2 * cy ** 2)
        b = -np.sin(2 * theta) / (4 * cx ** 2) + np.sin(2 * theta) / (4 * cy ** 2)
        c = np.sin(theta) ** 2 / (2 * cx ** 2) + np.cos(theta) ** 2 / (2 * cy ** 2)
        out = np.empty((res * res, len(u0x)))
        for i, (x0, y0) in enumerate(zip(u0x, u0y)):
            G = self.sign * np.exp(-(a * (X - x0) ** 2 + 2 * b * (X - x0) * (Y - y0) + c * (Y - y0) ** 2))
            if self.flip_lr:
                G = np.fliplr(G)
            if self.flip_:
                G = np.flip(G)
            out[:, i] = G.reshape(res * res)
        if self.floating_precision == 32:
            out = np.float32(out)
        return out

    def _separable_factors(self, u0x, u0y):
        """(gx [nx,res], gy [ny,res] float32, grid cell -> actuator [ny*nx]
        int32) with modes[y*res+x, a] = gx[i_a, x] * gy[j_a, y], or None when
        the IFs do not factorise that way: an anamorphosis angle couples x and
        y, a rotated grid has no common columns, and a grid with a cell shared
        by two actuators has no cell map.  The factors are checked against
        the float64 modes before use."""
        if self.misReg.anamorphosisAngle != 0:
            return None
        xs, ix = np.unique(u0x, return_inverse=True)
        ys, iy = np.unique(u0y, return_inverse=True)
        nx, ny = len(xs), len(ys)
        if nx * ny > 4 * len(u0x) + 64:
            return None
        cells = np.full(nx * ny, -1, dtype=np.int32)
        flat = iy * nx + ix
        if len(np.unique(flat)) != len(flat):
            return None
        cells[flat] = np.arange(len(flat), dtype=np.int32)
        res = self.resolution
        w = (res / self.nActAlongDiameter) / np.sqrt(2 * np.log(1. / self.mechCoupling))
        a = 1 / (2 * ((1 + self.misReg.radialScaling) * w) ** 2)
        c = 1 / (2 * ((1 + self.misReg.tangentialScaling) * w) ** 2)
        X = np.linspace(0, 1, res) * res
        gx = self.sign * np.exp(-a * (X[None, :] - xs[:, None]) ** 2)
        gy = np.exp(-c * (X[None, :] - ys[:, None]) ** 2)
        if self.flip_lr:
            gx = gx[:, ::-1]
        if self.flip_:
            gx, gy = gx[:, ::-1], gy[:, ::-1]
        # the dense IFs are the reference: the factors must reproduce them (to
        # round-off of the modes' own precision, float32 with
        # floating_precision=32) on a spread sample of actuators; the product
        # of the two 1-D Gaussians is the 2-D one by construction
        cols = np.unique(np.linspace(0, len(u0x) - 1, min(len(u0x), 128)).astype(int))
        dense = self._gaussian_modes(u0x[cols], u0y[cols])
        tol = (2e-7 if dense.dtype == np.float32 else 1e-12) * np.max(np.abs(dense))
        rebuilt = (gy[iy[cols]][:, :, None] * gx[ix[cols]][:, None, :]).reshape(len(cols), res * res)
        if np.max(np.abs(rebuilt.T - dense)) > tol:
            return None
        return (np.ascontiguousarray(gx), np.ascontiguousarray(gy), cells)

    def _upload_modes(self):
        self._modes_bf16 = None
        self._modes_tf32 = None
        self._tc_ws = None
        if self.if_dtype == 'bf16':
            self._n_act_pad = (self.nValidAct + 63) // 64 * 64
            npix = self.resolution ** 2
            self._modes_bf16 = torch.empty((npix, self._n_act_pad), dtype=torch.bfloat16, device=self._dev)
            N.call('oopao_dm_modes_bf16', self._modes_t, self.nValidAct, npix, self._n_act_pad, self._modes_bf16,
                   N.stream_handle())
            self._tc_ws = None
        elif self.if_dtype != 'fp32':
            raise OopaoError("if_dtype must be 'fp32' or 'bf16'")

    # ------------------------------------------------------------ projection
    def opd_device(self, coefs_dev, scale=1.0, out=None, base=None):
        """Device projection: coefs [n_act] or [n_act, B] float32 -> opd
        [B, res, res] float32 (= (modes @ coefs)^T * scale [+ base]) by the
        path projection_path() names."""
        c = coefs_dev if coefs_dev.ndim == 2 else coefs_dev[:, None]
        c = c.contiguous()
        B = c.shape[1]
        res = self.resolution
        if out is None:
            out = torch.empty((B, res, res), dtype=torch.float32, device=self._dev)
        self._launch_projection(c, B, scale, base, out, N.stream_handle())
        return out

    # Batches above this go to the BF16 tensor-core GEMM even when the IFs
    # factorise.  Measured on GB300 the separable projection (fused kernel up
    # to 15 columns, then the tiled FP32 GEMM of the second contraction) is
    # faster at every batch: 80x80 at 300 columns 0.60 ms against 1.30 ms,
    # 40x40 0.097 against 0.128 ms; autotune.tune_dm measures the cut-over
    # per mirror.
    SEPARABLE_MAX_BATCH_VS_TC = 1 << 30
    # FP32 IFs that do not factorise: from this many columns on the projection
    # runs on the tensor cores at FP32 accuracy (three TF32 products); below
    # it the FP32 GEMV/SGEMM on the CUDA cores.  None: never.
    TF32_MIN_BATCH = 16

    def projection_path(self, B=1):
        """Path of a projection of B coefficient vectors: 'separable', 'bf16'
        (BF16 IFs on the tensor cores), 'tf32' (FP32 IFs on the tensor cores,
        three TF32 products) or 'fp32' (dense CUDA cores)."""
        if self._sep is not None and self.separable_projection and (
                self._modes_bf16 is None or B <= self.separable_max_batch):
            return 'separable'
        if self._modes_bf16 is not None:
            return 'bf16'
        if self.tf32_min_batch is not None and B >= self.tf32_min_batch:
            return 'tf32'
        return 'fp32'

    def projection_workspace_bytes(self, B):
        """Device workspace bytes the projection of B coefficient vectors needs."""
        path = self.projection_path(B)
        if path == 'separable':
            return N.load().oopao_dm_sep_workspace_bytes(self._sep[4], self.resolution, B)
        if path == 'bf16':
            return N.load().oopao_dm_bf16_workspace_bytes(self._n_act_pad, B)
        if path == 'tf32':
            return N.load().oopao_dm_tf32_workspace_bytes(self._tf32_pad(), B)
        return 0

    def _tf32_pad(self):
        return (self.nValidAct + 31) // 32 * 32

    def _tf32_modes(self, stream):
        """The IFs as TF32 values and FP32 remainders [2][n_pix][n_act_pad],
        built on the first tensor-core projection of FP32 IFs."""
        if self._modes_tf32 is None:
            npix, pad = self.resolution ** 2, self._tf32_pad()
            m = torch.empty((2, npix, pad), dtype=torch.float32, device=self._dev)
            N.call('oopao_dm_modes_tf32x2', self._modes_t, self.nValidAct, npix, pad, m, stream)
            self._modes_tf32 = m
        return self._modes_tf32

    def _projection_workspace(self, B):
        """The DM's own projection workspace, grown on demand (a captured
        graph must hold its own buffer instead: this one may be replaced)."""
        nb = self.projection_workspace_bytes(B)
        if nb == 0:
            return None
        if self.projection_path(B) == 'separable':
            if self._sep_ws is None or self._sep_ws.numel() < nb:
                self._sep_ws = torch.empty(nb, dtype=torch.uint8, device=self._dev)
            return self._sep_ws
        if self._tc_ws is None or self._tc_ws.numel() < nb:
            self._tc_ws = torch.empty(nb, dtype=torch.uint8, device=self._dev)
        return self._tc_ws

    def _launch_projection(self, c, B, scale, base, out, stream, ws=None):
        """out = (modes @ c)^T * scale + base on `stream` by
        projection_path(B): the separable factors when the IFs factorise
        (exact, 2*ny*res*(nx+res) flops per frame), else the BF16 tensor-core
        GEMM (if_dtype='bf16') or the FP32 GEMV/SGEMM over the dense IF
        matrix.  ws: a caller-owned workspace of projection_workspace_bytes(B)
        bytes, or None for the DM's own."""
        res = self.resolution
        if ws is None:
            ws = self._projection_workspace(B)
        path = self.projection_path(B)
        if path == 'separable':
            gx, gy, cells, nx, ny = self._sep
            N.call('oopao_dm_opd_sep_f32', gx, gy, cells, nx, ny, c, self.nValidAct, res, B, float(scale), base, out,
                   ws, ws.numel(), stream)
        elif path == 'bf16':
            tile = next((t for bound, t in self.tc_tile_rule if B <= bound), 0)
            N.call('oopao_dm_opd_bf16_tiled', self._modes_bf16, self._n_act_pad, c, self.nValidAct, res * res, B,
                   float(scale), base, out, ws, ws.numel(), tile, stream)
        elif path == 'tf32':
            N.call('oopao_dm_opd_tf32x3', self._tf32_modes(stream), self._tf32_pad(), c, self.nValidAct, res * res, B,
                   float(scale), base, out, ws, ws.numel(), stream)
        else:
            N.call('oopao_dm_opd_acc_f32', self._modes_t, c, self.nValidAct, res * res, B, float(scale), base, out,
                   stream)

    def tensor_core_status(self):
        """0, or the code of a timed-out pipeline wait of the last tensor-core
        projection (BF16 or TF32)."""
        if self._tc_ws is None:
            return 0
        return int(self._tc_ws[:4].view(torch.int32).item())

    @property
    def coefs(self):
        return self._coefs

    @coefs.setter
    def coefs(self, val):
        if torch.is_tensor(val):
            cd = val.to(device=self._dev, dtype=torch.float32)
            self._coefs = val
            if cd.shape[0] != self.nValidAct:
                raise OopaoError('Error: wrong value for the coefficients')
        else:
            if self.floating_precision == 32:
                val = np.float32(val)
            if np.isscalar(val):
                if val != 0:
                    raise OopaoError('Error: wrong value for the coefficients')
                val = np.zeros(self.nValidAct, dtype=self.precision)
            val = np.asarray(val)
            if len(val) != self.nValidAct:
                raise OopaoError('Error: wrong value for the coefficients')
            self._coefs = val
            cd = torch.as_tensor(np.ascontiguousarray(val, dtype=np.float32), device=self._dev)
        opd = self.opd_device(cd)
        self._opd_dev = opd[0] if cd.ndim == 1 else opd
        self._opd_host = None
        self.current_coefs = self._coefs.copy() if hasattr(self._coefs, 'copy') else self._coefs.clone()

    @property
    def OPD(self):
        if self._opd_host is None:
            a = self._opd_dev.detach().to('cpu', torch.float64).numpy()
            self._opd_host = np.moveaxis(a, 0, -1) if a.ndim == 3 else a
        return self._opd_host

    def relay(self, src):
        if src.tag != 'source':
            raise OopaoError('Only a single Source can be propagated (asterisms are not supported)')
        src.optical_path.append([self.tag, self])
        if self._opd_dev.ndim == 2 and (src._opd_zero or src._opd_np is None and not src._dev_fresh):
            # OPD_no_pupil = 0 + dm.OPD
            src._set_device_opd(self._opd_dev)
        elif self._opd_dev.ndim == 2:
            base = src.device_opd(self._dev)
            if base.ndim != 2:
                base = torch.zeros_like(self._opd_dev)
            src._set_device_opd(base + self._opd_dev)
        else:
            # several OPDs at once replace the current one (DeformableMirror.py:447-449)
            src._set_device_opd(self._opd_dev)

    def __repr__(self):
        return 'DeformableMirror(nValidAct=%d, pitch=%.3f m, coupling=%.2f)' % (
            self.nValidAct, self.pitch, self.mechCoupling)
