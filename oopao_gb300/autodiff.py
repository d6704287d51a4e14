"""Differentiable pyramid WFS: hand-written tangent and adjoint behind
``torch.autograd.Function``.

The reference only differentiates by finite push-pull differences
(``OOPAO/calibration/InteractionMatrix.py:117-158``).  Here the whole chain
— DM projection, pupil field, modulated Fourier filtering, |.|^2, sum over
modulation points, binning, slopes with their normalisation — has an exact
tangent (``oopao_pwfs_jvp`` + ``oopao_pwfs_signal_jvp``) and adjoint
(``oopao_pwfs_signal_vjp`` + ``oopao_pwfs_vjp`` + ``oopao_dm_vjp_f32``), the
adjoint recomputing each modulation point's field rather than storing it.

* ``pyramid_signal(wfs, opd)``  -> signal [B, nSignal], differentiable in opd
  (reverse mode: ``.backward()``; forward mode: ``torch.func.jvp`` /
  ``torch.autograd.forward_ad``)
* ``dm_signal(wfs, dm, coefs)`` -> the same from DM coefficients [nAct, B]
* ``jvp_interaction_matrix(ngs, tel, dm, wfs, M2C)`` -> d signal / d modal
  coefficient at the flat wavefront, all modes in one batched tangent pass
* ``lift_estimate`` / ``modal_gradient_descent`` -> LiFT-style modal
  estimation (``OOPAO/LiFT.py:182-349`` estimates from PSFs; here from
  pyramid signals with the analytic Jacobian / gradient)
"""
import numpy as np
import torch

from . import _native as N
from .tools import OopaoError


def _scale(wfs):
    return 2 * np.pi / wfs.src.wavelength


def _plan(wfs):
    """The sensor's plan as the interaction matrix sees it: a batch
    measurement, whose sum over modulation points is unweighted."""
    return wfs._weighted_plan(False) if hasattr(wfs, '_weighted_plan') else wfs.plan


def _ws(wfs, batch, ad=True):
    plan = _plan(wfs)
    nb = N.load().oopao_pwfs_ad_workspace_bytes(plan.h, batch) if ad else plan.workspace_bytes(batch)
    return wfs._ws.get(nb), nb


def frames(wfs, opd, scale=None):
    """Camera frames [B, cam, cam] of OPD maps [B, res, res] (metres)."""
    scale = _scale(wfs) if scale is None else scale
    f, _ = wfs._measure_frames(opd, scale)
    return f


def frame_jvp(wfs, opd0, dopd, scale=None):
    """Tangent of the camera frames at opd0 ([1 or B, res, res]) along dopd [B, res, res]."""
    scale = _scale(wfs) if scale is None else scale
    plan = _plan(wfs)
    dopd = dopd.contiguous()
    opd0 = opd0.contiguous()
    B = dopd.shape[0]
    cam = wfs._cam_eff
    out = torch.empty((B, cam, cam), dtype=torch.float32, device=dopd.device)
    ws, nb = _ws(wfs, B)
    N.call('oopao_pwfs_jvp', plan.h, N.ptr(opd0), opd0.shape[0], N.ptr(dopd), float(scale), B, N.ptr(out),
           N.ptr(ws), nb, N.stream_handle())
    return out


def frame_vjp(wfs, opd, fbar, scale=None):
    """Adjoint of the camera frames at opd [B, res, res] applied to fbar [B, cam, cam]."""
    scale = _scale(wfs) if scale is None else scale
    plan = _plan(wfs)
    opd = opd.contiguous()
    fbar = fbar.contiguous()
    B = opd.shape[0]
    out = torch.empty_like(opd)
    ws, nb = _ws(wfs, B)
    N.call('oopao_pwfs_vjp', plan.h, N.ptr(opd), N.ptr(fbar), float(scale), B, N.ptr(out), N.ptr(ws), nb,
           N.stream_handle())
    return out


def signal_jvp(wfs, frame0, dframe):
    plan = _plan(wfs)
    if not getattr(wfs, '_signal_configured', False):
        wfs._configure_signal(plan)
    frame0 = frame0.contiguous()
    dframe = dframe.contiguous()
    B = dframe.shape[0]
    n2d = wfs.validSignal.size
    ns = N.load().oopao_pwfs_n_signal(plan.h)
    s2 = torch.empty((B, n2d), dtype=torch.float32, device=dframe.device)
    s = torch.empty((B, ns), dtype=torch.float32, device=dframe.device)
    N.call('oopao_pwfs_signal_jvp', plan.h, N.ptr(frame0), frame0.shape[0], N.ptr(dframe), B, N.ptr(s2), N.ptr(s),
           N.stream_handle())
    return s2, s


def signal_vjp(wfs, frame0, sbar):
    plan = _plan(wfs)
    if not getattr(wfs, '_signal_configured', False):
        wfs._configure_signal(plan)
    frame0 = frame0.contiguous()
    sbar = sbar.contiguous().to(torch.float32)
    B = sbar.shape[0]
    fbar = torch.empty((B,) + frame0.shape[1:], dtype=torch.float32, device=sbar.device)
    N.call('oopao_pwfs_signal_vjp', plan.h, N.ptr(frame0), frame0.shape[0], N.ptr(sbar), B, N.ptr(fbar),
           N.stream_handle())
    return fbar


class _PyramidSignal(torch.autograd.Function):
    """signal [B, nSignal] = wfs(opd [B, res, res]); opd in metres."""

    @staticmethod
    def forward(opd, wfs):
        frame = frames(wfs, opd.detach())
        _, s = wfs._signals(frame)
        return s, frame

    @staticmethod
    def setup_context(ctx, inputs, output):
        opd, wfs = inputs
        _, frame = output
        ctx.wfs = wfs
        ctx.save_for_backward(opd, frame)
        ctx.save_for_forward(opd, frame)
        ctx.mark_non_differentiable(frame)

    @staticmethod
    def backward(ctx, sbar, _fbar_unused):
        opd, frame = ctx.saved_tensors
        fbar = signal_vjp(ctx.wfs, frame, sbar)
        return frame_vjp(ctx.wfs, opd.detach(), fbar), None

    @staticmethod
    def jvp(ctx, dopd, _):
        opd, frame = ctx.saved_tensors
        dframe = frame_jvp(ctx.wfs, opd.detach(), dopd.contiguous())
        _, ds = signal_jvp(ctx.wfs, frame, dframe)
        return ds, None


def pyramid_signal(wfs, opd):
    """Differentiable ``wfs.signal`` of OPD maps [B, res, res] (or [res, res])."""
    single = opd.ndim == 2
    x = opd[None] if single else opd
    s, _ = _PyramidSignal.apply(x.contiguous(), wfs)
    return s[0] if single else s


class _DMProject(torch.autograd.Function):
    """opd [B, res, res] = (dm.modes @ coefs)^T for coefs [nAct, B]."""

    @staticmethod
    def forward(coefs, dm):
        return dm.opd_device(coefs.detach().contiguous())

    @staticmethod
    def setup_context(ctx, inputs, output):
        ctx.dm = inputs[1]

    @staticmethod
    def backward(ctx, g):
        dm = ctx.dm
        g = g.contiguous()
        B = g.shape[0]
        out = torch.empty((dm.nValidAct, B), dtype=torch.float32, device=g.device)
        N.call('oopao_dm_vjp_f32', N.ptr(dm._modes_t), N.ptr(g), dm.nValidAct, dm.resolution ** 2, B, 1.0,
               N.ptr(out), N.stream_handle())
        return out, None

    @staticmethod
    def jvp(ctx, dc, _):
        return ctx.dm.opd_device(dc.contiguous())


def dm_signal(wfs, dm, coefs):
    """Differentiable ``wfs.signal`` [B, nSignal] of DM coefficients [nAct, B]."""
    return pyramid_signal(wfs, _DMProject.apply(coefs, dm))


def jvp_interaction_matrix(ngs, tel, dm, wfs, M2C, phase_offset=None, chunk=256):
    """Interaction matrix [nSignal, nModes] = d wfs.signal / d modal
    coefficient at the flat wavefront (plus an optional phase offset, rad),
    from batched tangents: one operating point, every mode a tangent."""
    dev = wfs._dev
    scale = _scale(wfs)
    res = tel.resolution
    opd0 = torch.zeros((1, res, res), dtype=torch.float32, device=dev)
    if phase_offset is not None:
        opd0 = torch.as_tensor(np.asarray(phase_offset) / scale, dtype=torch.float32, device=dev)[None]
    ngs ** tel
    _plan(wfs).set_amplitude(ngs.intensity, wfs._amplitude_key())
    frame0 = frames(wfs, opd0)
    m2c = torch.as_tensor(np.ascontiguousarray(M2C, dtype=np.float32), device=dev)
    cols = []
    for b0 in range(0, m2c.shape[1], chunk):
        dopd = dm.opd_device(m2c[:, b0:b0 + chunk].contiguous())
        dframe = frame_jvp(wfs, opd0, dopd, scale)
        _, ds = signal_jvp(wfs, frame0, dframe)
        cols.append(ds)
    return torch.cat(cols).T


def _as_device(a, dev):
    if torch.is_tensor(a):
        return a.detach().to(device=dev, dtype=torch.float32)
    return torch.as_tensor(np.asarray(a), dtype=torch.float32, device=dev)


def lift_estimate(wfs, dm, M2C, target, n_iter=5, x0=None, damping=0.0):
    """Gauss-Newton modal estimation (the LiFT update of OOPAO/LiFT.py:297-330,
    P_ML = (H^T H)^-1 H^T, with the pyramid signal in place of the PSF):
    x <- x + (H^T H + damping I)^-1 H^T (target - s(x)), H = d s / d x from
    batched tangents at the current estimate.  Returns x [nModes]."""
    dev = wfs._dev
    m2c = torch.as_tensor(np.ascontiguousarray(M2C, dtype=np.float32), device=dev)
    t = _as_device(target, dev).reshape(-1)
    x = torch.zeros(m2c.shape[1], dtype=torch.float32, device=dev) if x0 is None else \
        _as_device(x0, dev).clone()
    scale = _scale(wfs)
    for _ in range(n_iter):
        opd = dm.opd_device((m2c @ x)[:, None].contiguous())
        frame0 = frames(wfs, opd, scale)
        _, s = wfs._signals(frame0)
        dopd = dm.opd_device(m2c)
        dframe = frame_jvp(wfs, opd, dopd, scale)
        _, H = signal_jvp(wfs, frame0, dframe)
        H = H.T.double()
        r = (t - s[0]).double()
        A = H.T @ H + damping * torch.eye(H.shape[1], dtype=torch.float64, device=dev)
        x = x + torch.linalg.solve(A, H.T @ r).float()
    return x


def modal_loss(wfs, dm, M2C, x, targets):
    """Per-item loss ||s(M2C x_b) - t_b||^2 [B] (float64 sums of the float32
    signals) for modal coefficients x [nModes, B] (metres)."""
    dev = wfs._dev
    m2c = torch.as_tensor(np.ascontiguousarray(M2C, dtype=np.float32), device=dev)
    t = _as_device(targets, dev)
    with torch.no_grad():
        s = dm_signal(wfs, dm, m2c @ _as_device(x, dev))
        return ((s.double() - t.double()) ** 2).sum(dim=1)


def modal_loss_grad(wfs, dm, M2C, x, targets):
    """Per-item loss [B] and its gradient d loss_b / d x_b [nModes, B] by the
    hand-written adjoint (signal VJP, propagation VJP with each modulation
    point's field recomputed, DM adjoint, M2C^T)."""
    dev = wfs._dev
    m2c = torch.as_tensor(np.ascontiguousarray(M2C, dtype=np.float32), device=dev)
    t = _as_device(targets, dev)
    xv = _as_device(x, dev).clone().requires_grad_(True)
    s = dm_signal(wfs, dm, m2c @ xv)
    loss = ((s - t) ** 2).sum(dim=1)
    loss.sum().backward()
    return ((s.detach().double() - t.double()) ** 2).sum(dim=1), xv.grad.detach()


def modal_gradient_descent(wfs, dm, M2C, targets, n_iter=200, lr=1e-2, x0=None):
    """Batched modal estimation by gradient descent on ||s(M2C x_b) - t_b||^2
    with the hand-written adjoint.  targets [B, nSignal]; returns x [nModes, B]
    and the loss history."""
    dev = wfs._dev
    m2c = torch.as_tensor(np.ascontiguousarray(M2C, dtype=np.float32), device=dev)
    t = _as_device(targets, dev)
    B = t.shape[0]
    x = torch.zeros((m2c.shape[1], B), dtype=torch.float32, device=dev) if x0 is None else \
        _as_device(x0, dev).clone()
    x.requires_grad_(True)
    opt = torch.optim.Adam([x], lr=lr)
    hist = []
    for _ in range(n_iter):
        opt.zero_grad()
        s = dm_signal(wfs, dm, m2c @ x)
        loss = ((s - t) ** 2).sum()
        loss.backward()
        opt.step()
        hist.append(float(loss.detach()))
    return x.detach(), hist


__all__ = ['pyramid_signal', 'dm_signal', 'jvp_interaction_matrix', 'lift_estimate', 'modal_gradient_descent',
           'modal_loss', 'modal_loss_grad',
           'frames', 'frame_jvp', 'frame_vjp', 'signal_jvp', 'signal_vjp']
