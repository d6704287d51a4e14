"""The differentiable-PWFS pipeline of the 40x40 modal-estimation
configuration, at a reduced size: 20x20 pyramid (N=264, 48 points), the
reference's first 40 KL modes of the 21x21 DM, 4 seeded modal screens with
coefficients ~N(0, 50 nm), loss ||signal(M2C x) - target||^2.

Checks of the hand-written adjoint gradient (signal VJP, propagation VJP
with each modulation point's field recomputed, DM adjoint):
  * against central finite differences of the loss, step 1e-3 rad RMS of
    phase along seeded unit directions: <= 2e-3 relative;
  * against the gradient the reference's push-pull interaction matrix gives
    at the same point, 2 D^T (s - t) (stroke 1e-8 m): <= 2e-2 relative, the
    push-pull truncation at this stroke;
  * gradient descent (Adam) on all items at once lowers the loss.
"""
import contextlib
import io
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_MODES, N_SCREENS, SIGMA = 40, 4, 50e-9


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


@pytest.fixture(scope='module')
def problem():
    import torch
    import oopao_gb300 as og
    from oopao_gb300 import autodiff as AD
    with _quiet():
        tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=20, mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=20, telescope=tel, modulation=3, lightRatio=0.5, nTheta_user_defined=48)
    with np.load(os.path.join(os.path.dirname(__file__), 'golden', 'kl_c1.npz')) as z:
        m2c = np.ascontiguousarray(z['m2c'][:, :N_MODES])
    ngs ** tel
    truth = np.random.default_rng(4).standard_normal((N_MODES, N_SCREENS)) * SIGMA
    t = torch.as_tensor(truth, dtype=torch.float32, device='cuda')
    m = torch.as_tensor(m2c, dtype=torch.float32, device='cuda')
    with torch.no_grad():
        targets = AD.dm_signal(wfs, dm, m @ t)
    return tel, ngs, dm, wfs, m2c, truth, targets


def test_adjoint_gradient_against_finite_differences(problem):
    from oopao_gb300 import autodiff as AD
    tel, ngs, dm, wfs, m2c, truth, targets = problem
    rng = np.random.default_rng(5)
    x0 = truth + rng.standard_normal(truth.shape) * SIGMA   # an estimate away from the truth
    _, g = AD.modal_loss_grad(wfs, dm, m2c, x0, targets)
    g = g.double().cpu().numpy()
    h = 1e-3 * ngs.wavelength / (2 * np.pi)   # 1e-3 rad RMS: the modes are 1 m RMS per unit coefficient
    for _ in range(3):
        u = rng.standard_normal(truth.shape)
        u /= np.linalg.norm(u, axis=0)
        lp = AD.modal_loss(wfs, dm, m2c, x0 + h * u, targets).cpu().numpy()
        lm = AD.modal_loss(wfs, dm, m2c, x0 - h * u, targets).cpu().numpy()
        fd = (lp - lm) / (2 * h)
        ad = (g * u).sum(axis=0)
        assert np.max(np.abs(fd - ad)) / np.max(np.abs(ad)) < 2e-3


def test_adjoint_gradient_against_push_pull_matrix(problem):
    import torch
    import oopao_gb300 as og
    from oopao_gb300 import autodiff as AD
    tel, ngs, dm, wfs, m2c, truth, targets = problem
    x0 = np.zeros_like(truth)
    _, g = AD.modal_loss_grad(wfs, dm, m2c, x0, targets)
    calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=1, single_pass=False,
                                 invert=False)
    with torch.no_grad():
        s0 = AD.dm_signal(wfs, dm, torch.zeros((dm.nValidAct, 1), device='cuda'))
    r = s0.double().cpu().numpy()[0][:, None] - targets.double().cpu().numpy().T
    g_pp = 2 * np.asarray(calib.D).T @ r
    gd = g.double().cpu().numpy()
    assert np.linalg.norm(gd - g_pp) / np.linalg.norm(g_pp) < 2e-2


def test_gradient_descent_lowers_the_loss(problem):
    from oopao_gb300 import autodiff as AD
    tel, ngs, dm, wfs, m2c, truth, targets = problem
    x, hist = AD.modal_gradient_descent(wfs, dm, m2c, targets, n_iter=30, lr=0.2 * SIGMA)
    assert len(hist) == 30
    assert hist[-1] < 0.5 * hist[0]
    loss = AD.modal_loss(wfs, dm, m2c, x, targets).cpu().numpy()
    assert np.isfinite(loss).all()


def test_lift_gauss_newton_recovers_kl_modes(problem):
    """LiFT's Gauss-Newton modal estimation (OOPAO/LiFT.py:297-330 pattern,
    the pyramid signal as the measurement) on this configuration: 40 KL
    coefficients ~N(0, 5 nm) (wavefronts of ~30 nm RMS, 0.4 rad at 500 nm,
    where the sensor is already non-linear) are recovered from their signal to
    1e-3 relative in six iterations, the Jacobian re-formed from batched
    tangents at each estimate."""
    import torch
    from oopao_gb300 import autodiff as AD
    tel, ngs, dm, wfs, m2c, truth, targets = problem
    small = np.random.default_rng(8).standard_normal((N_MODES, 2)) * 5e-9
    m = torch.as_tensor(m2c, dtype=torch.float32, device='cuda')
    with torch.no_grad():
        t = AD.dm_signal(wfs, dm, m @ torch.as_tensor(small, dtype=torch.float32, device='cuda'))
    for b in range(2):
        x = AD.lift_estimate(wfs, dm, m2c, t[b], n_iter=6)
        err = np.linalg.norm(x.double().cpu().numpy() - small[:, b]) / np.linalg.norm(small[:, b])
        assert err < 1e-3, (b, err)
