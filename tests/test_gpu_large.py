"""80x80 pyramid on a 39 m, 480 px pupil (N = 1920, 320x320 camera, 128
modulation points) against the reference's own measurement of a seeded
screen (golden made by the unmodified reference): geometry, valid pixels,
reference slopes, camera frame and slopes.  FP32 path bound: 1e-5."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'c5_screen.npz')


def _large(max_batch=2):
    import oopao_gb300 as og
    z = np.load(GOLDEN)
    p = json.loads(str(z['params']))
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=p['diameter'], samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'], lightRatio=p['light_ratio'],
                         n_pix_separation=p['n_pix_separation'], n_pix_edge=p['n_pix_edge'],
                         nTheta_user_defined=p['nTheta_user_defined'], max_batch=max_batch)
    return z, tel, ngs, wfs


def test_large_tangent_and_adjoint():
    """N = 1920 tangent against a central difference of the FP32 frames and
    the adjoint against the tangent through the dot-product identity
    <J v, u> = <v, J^T u>.  The step moves the phase by ~0.013 rad: large
    enough that FP32 rounding of the frames stays far below the bound, small
    enough that the difference's truncation error (~1e-5) does too."""
    import torch
    from oopao_gb300 import autodiff as AD
    z, tel, ngs, wfs = _large()
    ngs ** tel
    wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
    g = torch.Generator(device='cuda').manual_seed(0)
    pup = torch.as_tensor(tel.pupil, dtype=torch.float32, device='cuda')
    opd0 = (torch.as_tensor(z['screen_phase'], dtype=torch.float32, device='cuda') * ngs.wavelength / (2 * np.pi))[None]
    x = torch.linspace(-1, 1, tel.resolution, device='cuda')
    v = ((x[None, :] * x[:, None]) * 20e-9 * pup)[None]                  # smooth direction (astigmatism-like)
    jv = AD.frame_jvp(wfs, opd0, v)
    h = 0.05
    fd = (AD.frames(wfs, opd0 + h * v) - AD.frames(wfs, opd0 - h * v)) / (2 * h)
    assert O.rel_l2(jv.double().cpu().numpy(), fd.double().cpu().numpy()) < 1e-3
    u = torch.randn(jv.shape, device='cuda', generator=g)
    jtu = AD.frame_vjp(wfs, opd0, u)
    lhs = float((jv.double() * u.double()).sum())
    rhs = float((v.double() * jtu.double()).sum())
    assert abs(lhs - rhs) < 1e-4 * abs(lhs)


def test_large_pyramid_matches_reference():
    import oopao_gb300 as og
    z = np.load(GOLDEN)
    p = json.loads(str(z['params']))
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=p['diameter'], samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'], lightRatio=p['light_ratio'],
                         n_pix_separation=p['n_pix_separation'], n_pix_edge=p['n_pix_edge'],
                         nTheta_user_defined=p['nTheta_user_defined'], max_batch=2)
    assert wfs.resolution == int(z['N']) and wfs.cam.resolution == int(z['cam'])
    assert wfs.nTheta == int(z['n_theta'])
    np.testing.assert_array_equal(wfs.validI4Q, z['valid_i4q'])
    assert wfs.nSignal == int(z['n_signal'])
    assert O.rel_l2(wfs.referenceSignal_2D, z['reference_2d']) < 1e-5
    ngs ** tel
    wfs.wfs_measure(phase_in=z['screen_phase'])
    assert O.rel_l2(wfs.cam.frame, z['screen_frame']) < 1e-5
    assert O.rel_l2(wfs.signal_2D, z['screen_signal_2D']) < 1e-5
    assert O.rel_l2(wfs.signal, z['screen_signal']) < 1e-5
