"""Interaction matrix and reconstructor: drop-ins for the reference
``InteractionMatrix`` (``OOPAO/calibration/InteractionMatrix.py:13-169``) and
``CalibrationVault`` (``OOPAO/calibration/CalibrationVault.py:14-122``).

``InteractionMatrix`` keeps the reference signature and column rule
(column = factor * 0.5 * (s+ - s-) / stroke, factor 2 and s- = 0 for
``single_pass``).  Three GPU schedules compute the same matrix:

* ``method='batched'`` (default): the DM projection of a chunk of modes
  (one GEMM) feeds one batched pyramid launch over all (mode, modulation
  point) pairs of the chunk; nothing returns to the host until the end.
* ``method='per_mode'``: the plain schedule, one mode at a time through the
  public operator path ``dm.coefs = c; ngs**tel*dm*wfs`` (push, then pull).
* ``method='jvp'``: columns from the hand-written tangent of the sensor
  (``oopao_gb300.autodiff``), exact in the limit stroke -> 0.

The SVD of ``CalibrationVault`` runs in float64 on the GPU (an optional host
eigensolver is described at ``_vault_fp64``).
"""
import time

import numpy as np
import torch

from .tools import OopaoError


def _vault_fp64(D, n_ev, host_eigensolver=False):
    """Thin SVD D = U diag(s) V of an interaction matrix and the products of
    ``CalibrationVault`` (D, M, Mtrunc, Dtrunc), float64 on the GPU.

    Tall, well-conditioned matrices go through the Gram matrix:
    eigh(D^T D) = V^T diag(s^2) V (cuSOLVER syevd), U = D V^T / s, then the
    products, which return to the host in one copy.  Squaring the condition
    number costs at most ~1e-16 * cond^2 relative accuracy on the smallest
    singular values, so a full SVD (cuSOLVER gesvd) is used instead when
    cond(D) > 1e6 or D is wide.  Diagonal products are row/column scalings,
    which give the same numbers as the reference's products with diag(s).

    host_eigensolver: solve the small symmetric eigenproblem with LAPACK
    dsyevd on the host cores instead (the Gram matrix and the products stay
    on the GPU).  At n = 300 it takes 4.5 ms on GB300's Grace cores against
    9.3 ms for cuSOLVER syevd, whose float64 units are narrow; off by default,
    which keeps the float64 linear algebra on the GPU."""
    from .runtime import device
    dev = device()
    Dt = torch.as_tensor(np.asarray(D, dtype=np.float64), device=dev)
    m, n = Dt.shape
    if m >= n:
        G = Dt.T @ Dt
        if host_eigensolver:
            ev_h, W_h = np.linalg.eigh(G.cpu().numpy())
            ev, W = torch.as_tensor(ev_h, device=dev), torch.as_tensor(W_h, device=dev)
        else:
            ev, W = torch.linalg.eigh(G)
        ev = torch.flip(ev, [0])
        W = torch.flip(W, [1])
        lo_hi = torch.sqrt(torch.clamp(ev[[0, -1]], min=0)).cpu().numpy()
        if lo_hi[1] > 1e-6 * lo_hi[0]:
            s = torch.sqrt(ev)
            U = (Dt @ W) / s[None, :]
            return _vault_products(U, s, W.T.contiguous(), n_ev)
    U, s, Vh = torch.linalg.svd(Dt, full_matrices=False, driver='gesvd')
    return _vault_products(U, s, Vh, n_ev)


def _vault_products(U, s, V, n_ev):
    """U [m, n], s [n], V [n, n] on the device -> host arrays
    (U, s, V, U S V, V^T S^-1 U^T, and the two truncated products)."""
    Drec = (U * s[None, :]) @ V
    M = (V.T / s[None, :]) @ U.T
    Mtrunc = (V[:n_ev].T / s[None, :n_ev]) @ U[:, :n_ev].T
    Dtrunc = (U[:, :n_ev] * s[None, :n_ev]) @ V[:n_ev]
    parts = (U, s, V, Drec, M, Mtrunc, Dtrunc)
    # one device-to-host copy for all of them
    flat = torch.cat([t.reshape(-1) for t in parts]).cpu().numpy()
    out, o = [], 0
    for t in parts:
        out.append(flat[o:o + t.numel()].reshape(tuple(t.shape)))
        o += t.numel()
    return out


class CalibrationVault:
    def __init__(self, D, nTrunc: int = 0, display: bool = False, print_details: bool = False,
                 invert: bool = True, host_eigensolver: bool = False):
        if invert:
            n_ev = min(np.shape(D)) - nTrunc
            U, s, V, Drec, M, Mtrunc, Dtrunc = _vault_fp64(D, n_ev, host_eigensolver)
            self.s = s
            self.S = np.diag(s)
            self.eigenValues = s
            self.D = Drec
            self.U = np.transpose(U)
            self.V = V
            self._nTrunc = nTrunc
            self.iS = np.diag(1 / self.eigenValues)
            self.M = M
            self._set_truncation(n_ev, Mtrunc, Dtrunc)
        else:
            self.D = D

    def _set_truncation(self, n_ev, Mtrunc, Dtrunc):
        self.iStrunc = np.diag(1 / self.eigenValues[:n_ev])
        self.Vtrunc = self.V[:n_ev, :]
        self.Utrunc = self.U[:n_ev, :]
        self.VtruncT = np.transpose(self.Vtrunc)
        self.UtruncT = np.transpose(self.Utrunc)
        self.Mtrunc = Mtrunc
        self.Dtrunc = Dtrunc
        self.cond = self.eigenValues[0] / self.eigenValues[(-self._nTrunc - 1)]

    def _truncate(self, n_ev):
        self.iStrunc = np.diag(1 / self.eigenValues[:n_ev])
        self.Vtrunc = self.V[:n_ev, :]
        self.Utrunc = self.U[:n_ev, :]
        self.VtruncT = np.transpose(self.Vtrunc)
        self.UtruncT = np.transpose(self.Utrunc)
        self.Mtrunc = self.VtruncT @ self.iStrunc @ self.Utrunc
        self.Dtrunc = self.UtruncT @ np.diag(self.eigenValues[:n_ev]) @ self.Vtrunc
        self.cond = self.eigenValues[0] / self.eigenValues[(-self._nTrunc - 1)]

    @property
    def nTrunc(self):
        return self._nTrunc

    @nTrunc.setter
    def nTrunc(self, val):
        self._nTrunc = val
        self._truncate(len(self.s) - val)


def _signals_batched(ngs, tel, dm, wfs, commands, phase_offset=None):
    """Device signals [B, nSignal] for DM command columns [nAct, B]."""
    dev = wfs._dev
    c = torch.as_tensor(np.ascontiguousarray(commands, dtype=np.float32), device=dev)
    scale = 2 * np.pi / ngs.wavelength
    out = []
    B = c.shape[1]
    step = max(1, wfs.max_batch)
    for b0 in range(0, B, step):
        cb = c[:, b0:b0 + step].contiguous()
        opd = dm.opd_device(cb)
        if phase_offset is not None:
            opd = opd + torch.as_tensor(np.asarray(phase_offset) / scale, dtype=torch.float32, device=dev)
        frame, _ = wfs._measure_frames(opd, scale)
        frame = wfs.cam._integrate_device(frame, dt=wfs.telescope.samplingTime)
        _, sig = wfs._signals(frame)
        out.append(sig)
    return torch.cat(out, dim=0)


def InteractionMatrix(ngs, tel, dm, wfs, M2C, stroke, atm=None, phaseOffset=0, nMeasurements=50,
                      noise='off', invert=True, nTrunc=0, print_time=False, display=False,
                      single_pass=True, method='batched'):
    if noise == 'off':
        wfs.cam.photonNoise = 0
        wfs.cam.readoutNoise = 0
        wfs.cam.backgroundNoise = 0
    tel.isPaired = False
    ngs ** tel
    M2C = np.asarray(M2C)
    if M2C.ndim == 1:
        M2C = M2C[:, None]
    n_modes = M2C.shape[1]
    t0 = time.time()
    if method == 'batched':
        # phaseOffset: the reference adds it to ngs.phase only after the pull
        # has been measured (OOPAO/calibration/InteractionMatrix.py:126-133),
        # so no measured signal sees it and D does not depend on it
        off = None
        sp = _signals_batched(ngs, tel, dm, wfs, M2C * stroke, off)
        if single_pass:
            intmat = (0.5 * sp / stroke).T
            factor = 2
        else:
            sm = _signals_batched(ngs, tel, dm, wfs, -M2C * stroke, off)
            intmat = (0.5 * (sp - sm) / stroke).T
            factor = 1
        intmat = intmat.double().cpu().numpy()
    elif method == 'per_mode':
        intmat = np.zeros([wfs.nSignal, n_modes])
        for i in range(n_modes):
            dm.coefs = M2C[:, i] * stroke
            ngs ** tel * dm * wfs
            s_plus = wfs.device_signal
            if single_pass:
                col = 0.5 * s_plus / stroke
                factor = 2
            else:
                dm.coefs = -M2C[:, i] * stroke
                ngs ** tel * dm * wfs
                col = 0.5 * (s_plus - wfs.device_signal) / stroke
                factor = 1
            intmat[:, i] = col.double().cpu().numpy()
    elif method == 'jvp':
        from .autodiff import jvp_interaction_matrix
        intmat = jvp_interaction_matrix(ngs, tel, dm, wfs, M2C).double().cpu().numpy()
        factor = 1
    else:
        raise OopaoError('unknown InteractionMatrix method %r' % method)
    if print_time:
        print('Interaction matrix: %d modes in %.3f s' % (n_modes, time.time() - t0))
    dm.coefs = 0
    ngs ** tel
    return CalibrationVault(factor * intmat, invert=invert, nTrunc=nTrunc)
