"""Hand-written tangent/adjoint of the pyramid signal (GPU, FP32).

Checks: JVP against float64 central differences of the oracle, the adjoint
by the dot-product identity <J v, w> = <v, J^T w>, the JVP interaction
matrix against the reference's push-pull matrix and a float64 derivative,
torch reverse and forward mode, and LiFT-style modal recovery.
"""
import contextlib
import io

import numpy as np
import pytest

from oracle import pwfs_oracle as O
from tests import goldens as G

pytestmark = pytest.mark.gpu


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


def build(name):
    import oopao_gb300 as og
    d = G.load(name)
    p = d['params']
    kw = {k: v for k, v in p.items() if k not in ('res', 'n_subap', 'modulation', 'light_ratio', 'co')}
    with _quiet():
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3, centralObstruction=p['co'])
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'],
                         lightRatio=p['light_ratio'], **kw)
    return d, tel, ngs, dm, wfs


@pytest.fixture(scope='module', params=['tiny', 'c1'])
def system(request):
    return build(request.param)


def oracle_signal_derivative(d, wfs_o, phase0, dphase, h=1e-4):
    """float64 central difference of the oracle signal along dphase (rad)."""
    sp = wfs_o.measure(phase0 + h * dphase)[3]
    sm = wfs_o.measure(phase0 - h * dphase)[3]
    return (sp - sm) / (2 * h)


def test_jvp_matches_float64_central_difference(system):
    import torch
    from oopao_gb300 import autodiff as AD
    d, tel, ngs, dm, wfs = system
    wo = G.oracle_pyramid(d)
    res = tel.resolution
    rng = np.random.default_rng(1)
    phase0 = O.dm_opd(O.dm_modes(res, 8.0, d['params']['n_subap']), d['dm_coefs'], res) * tel.pupil * \
        2 * np.pi / ngs.wavelength
    dphase = rng.standard_normal((res, res)) * tel.pupil
    ref = oracle_signal_derivative(d, wo, phase0, dphase)
    scale = 2 * np.pi / ngs.wavelength
    ngs ** tel
    wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
    opd0 = torch.as_tensor((phase0 / scale)[None], dtype=torch.float32, device='cuda')
    dopd = torch.as_tensor((dphase / scale)[None], dtype=torch.float32, device='cuda')
    frame0 = AD.frames(wfs, opd0)
    dframe = AD.frame_jvp(wfs, opd0, dopd)
    _, ds = AD.signal_jvp(wfs, frame0, dframe)
    err = O.rel_l2(ds[0].double().cpu().numpy(), ref)
    assert err < 1e-4, err


def test_vjp_is_the_adjoint_of_the_jvp(system):
    import torch
    from oopao_gb300 import autodiff as AD
    d, tel, ngs, dm, wfs = system
    res = tel.resolution
    g = torch.Generator(device='cuda').manual_seed(3)
    ngs ** tel
    wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
    pupil = torch.as_tensor(tel.pupil, dtype=torch.float32, device='cuda')
    opd = torch.randn((2, res, res), device='cuda', generator=g) * 2e-8 * pupil
    v = torch.randn((2, res, res), device='cuda', generator=g) * 1e-8 * pupil
    frame0 = AD.frames(wfs, opd)
    # frame level
    jv = AD.frame_jvp(wfs, opd, v)
    w = torch.randn(jv.shape, device='cuda', generator=g)
    jtw = AD.frame_vjp(wfs, opd, w)
    lhs = (jv.double() * w.double()).sum(dim=(1, 2))
    rhs = (v.double() * jtw.double()).sum(dim=(1, 2))
    assert torch.allclose(lhs, rhs, rtol=2e-4, atol=0), (lhs, rhs)
    # signal level
    _, js = AD.signal_jvp(wfs, frame0, jv)
    ws = torch.randn(js.shape, device='cuda', generator=g)
    fbar = AD.signal_vjp(wfs, frame0, ws)
    lhs = (js.double() * ws.double()).sum(dim=1)
    rhs = (jv.double() * fbar.double()).sum(dim=(1, 2))
    assert torch.allclose(lhs, rhs, rtol=2e-4, atol=0), (lhs, rhs)


def test_jvp_interaction_matrix(system):
    import oopao_gb300 as og
    d, tel, ngs, dm, wfs = system
    if 'im_pp_D' not in d:
        pytest.skip('no push-pull matrix in this fixture')
    calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=d['im_m2c'], stroke=1e-8, method='jvp')
    # against the reference's push-pull matrix (stroke 1e-8 m: O(stroke^2) apart)
    assert O.rel_l2(calib.D, d['im_pp_D']) < 2e-3
    # against a float64 derivative (oracle push-pull at 1e-12 m)
    wo = G.oracle_pyramid(d)
    p = d['params']
    Dref = O.interaction_matrix(wo, O.dm_modes(p['res'], 8.0, p['n_subap'], 0.35, p['co']), d['im_m2c'], 1e-12,
                                float(d['wavelength']), d['pupil'], single_pass=False)
    err = O.rel_l2(calib.D, Dref)
    assert err < 1e-4, err


def test_autograd_reverse_and_forward_mode():
    import torch
    import torch.autograd.forward_ad as fwAD
    from oopao_gb300 import autodiff as AD
    d, tel, ngs, dm, wfs = build('tiny')
    ngs ** tel
    wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
    g = torch.Generator(device='cuda').manual_seed(5)
    c = (torch.randn((dm.nValidAct, 2), device='cuda', generator=g) * 3e-8).requires_grad_(True)
    t = torch.randn((2, wfs.nSignal), device='cuda', generator=g) * 0.1
    s = AD.dm_signal(wfs, dm, c)
    loss = ((s - t) ** 2).sum()
    loss.backward()
    # directional derivative of the loss along u via forward mode == <grad, u>
    u = torch.randn(c.shape, device='cuda', generator=g) * 1e-8
    with fwAD.dual_level():
        cd = fwAD.make_dual(c.detach(), u)
        sd = AD.dm_signal(wfs, dm, cd)
        primal, tangent = fwAD.unpack_dual(sd)
    dloss = (2 * (primal - t) * tangent).sum()
    gu = (c.grad * u).sum()
    assert torch.allclose(dloss.double(), gu.double(), rtol=1e-3), (dloss, gu)


def test_lift_estimate_recovers_modes():
    import torch
    from oopao_gb300 import autodiff as AD
    d, tel, ngs, dm, wfs = build('tiny')
    ngs ** tel
    wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
    m2c = np.eye(dm.nValidAct)[:, :6]
    x_true = torch.tensor([20e-9, -15e-9, 10e-9, 5e-9, -8e-9, 12e-9], device='cuda')
    opd = dm.opd_device((torch.as_tensor(m2c, dtype=torch.float32, device='cuda') @ x_true)[:, None].contiguous())
    target = AD.pyramid_signal(wfs, opd)[0]
    x = AD.lift_estimate(wfs, dm, m2c, target, n_iter=6)
    assert O.rel_l2(x.double().cpu().numpy(), x_true.double().cpu().numpy()) < 1e-3
    xs, hist = AD.modal_gradient_descent(wfs, dm, m2c, target[None], n_iter=200, lr=1e-9)
    assert hist[-1] < 5e-2 * hist[0], (hist[0], hist[-1])
