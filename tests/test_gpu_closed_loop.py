"""Closed-loop step on the GPU (screen -> DM -> WFS -> MVM -> integrator),
eager and replayed from a captured CUDA graph."""
import contextlib
import io

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


@pytest.fixture(scope='module')
def system():
    import oopao_gb300 as og
    with _quiet():
        tel = og.Telescope(resolution=40, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=10, mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=10, telescope=tel, modulation=2, lightRatio=0.5, n_pix_separation=4,
                         n_pix_edge=2, nTheta_user_defined=12)
        calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=np.eye(dm.nValidAct), stroke=1e-8, method='jvp')
    return tel, ngs, dm, wfs, calib


def test_screen_kernel_matches_host(system):
    import torch
    from oopao_gb300.closed_loop import ClosedLoop, VonKarmanLayers
    tel, ngs, dm, wfs, calib = system
    layers = VonKarmanLayers(tel, r0=0.15, L0=25, fractionalR0=(0.6, 0.4), windSpeed=(10., 17.),
                             windDirection=(0., 60.), seed=1)
    cl = ClosedLoop(tel, ngs, dm, wfs, calib.M, gain=0.0, layers=layers)
    for step in (0, 3):
        cl.step_counter.fill_(step)
        cl.coefs.zero_()
        cl.step()
        torch.cuda.synchronize()
        host = layers.opd(step, tel.resolution)
        assert O.rel_l2(cl.opd_atm[0].double().cpu().numpy(), host) < 1e-5


def test_graph_replay_equals_eager(system):
    import torch
    from oopao_gb300.closed_loop import ClosedLoop, VonKarmanLayers
    tel, ngs, dm, wfs, calib = system
    layers = VonKarmanLayers(tel, r0=0.15, L0=25, windSpeed=(10.,), seed=2)
    cl = ClosedLoop(tel, ngs, dm, wfs, calib.M, gain=0.4, layers=layers)
    cl.reset()
    cl.run(20, graph=False)
    torch.cuda.synchronize()
    coefs_e, wfe_e = cl.coefs.clone(), cl.residual_wfe.copy()
    cl.capture()
    cl.run(20, graph=True)
    torch.cuda.synchronize()
    assert torch.equal(cl.coefs, coefs_e)
    np.testing.assert_array_equal(cl.residual_wfe, wfe_e)


def test_one_step_matches_operator_path(system):
    """coefs after one step == coefs - g R s with s measured by ngs**tel*dm*wfs."""
    import torch
    from oopao_gb300.closed_loop import ClosedLoop
    tel, ngs, dm, wfs, calib = system
    rng = np.random.default_rng(4)
    c0 = rng.standard_normal(dm.nValidAct) * 30e-9
    cl = ClosedLoop(tel, ngs, dm, wfs, calib.M, gain=0.3, layers=None)
    cl.coefs.copy_(torch.as_tensor(c0, dtype=torch.float32))
    cl.step()
    torch.cuda.synchronize()
    dm.coefs = c0
    ngs ** tel * dm * wfs
    ref = c0 - 0.3 * calib.M @ wfs.signal
    assert O.rel_l2(cl.coefs.double().cpu().numpy(), ref) < 1e-5


def test_loop_converges_on_static_aberration(system):
    import torch
    from oopao_gb300.closed_loop import ClosedLoop, VonKarmanLayers
    tel, ngs, dm, wfs, calib = system
    layers = VonKarmanLayers(tel, r0=0.5, L0=25, windSpeed=(0.,), seed=3)
    cl = ClosedLoop(tel, ngs, dm, wfs, calib.M, gain=0.5, layers=layers)
    cl.run(30)
    torch.cuda.synchronize()
    w = cl.residual_wfe
    assert len(w) == 30
    assert w[-1] < 0.35 * w[0], (w[0], w[-1])


def test_long_exposure_strehl_vs_fp64_oracle(system):
    """Graph-replayed FP32 loop against the float64 oracle loop (oracle IM,
    float64 pseudo-inverse, same frozen-flow turbulence): residual WFE per
    step, long-exposure PSF and its Strehl ratio within 1e-4 relative."""
    import torch
    from oopao_gb300.closed_loop import ClosedLoop, VonKarmanLayers
    tel, ngs, dm, wfs, _ = system
    res = tel.resolution
    pup = O.telescope_pupil(res)
    inten = O.source_intensity(pup, O.n_photon('V0', 8), 1e-3, 8.0)
    ow = O.build_pyramid(res, 10, 2, 0.5, inten, n_pix_separation=4, n_pix_edge=2, n_theta_user=12, workers=4)
    modes = O.dm_modes(res, 8.0, 10)
    D = O.interaction_matrix(ow, modes, np.eye(modes.shape[1]), 1e-8, ngs.wavelength, pup, single_pass=False,
                             workers=4)
    R = np.linalg.pinv(D, rcond=1e-6)   # drops the modes the sensor does not see
    layers = VonKarmanLayers(tel, r0=0.5, L0=25, windSpeed=(10.,), seed=5)
    n = 60
    cl = ClosedLoop(tel, ngs, dm, wfs, R, gain=0.4, layers=layers, max_steps=n + 5, science=True)
    cl.run(n)
    torch.cuda.synchronize()
    wfe, psf, sr = cl.residual_wfe, cl.long_exposure_psf(), cl.long_exposure_strehl()
    ref = O.closed_loop(ow, modes, R, lambda t: layers.opd(t, res), pup, ngs.wavelength, 0.4, n, workers=4)
    assert ref['wfe'][-1] < 0.5 * ref['wfe'][0]          # the loop closes
    assert O.rel_l2(wfe, ref['wfe']) < 1e-4
    assert O.rel_l2(psf, ref['psf_le']) < 1e-4
    assert abs(sr - ref['strehl_le']) < 1e-4 * ref['strehl_le']


@pytest.fixture(scope='module')
def gsc_system(system):
    """Modal loop of 20 modes (zonal M2C slice) with a GainSensingCamera
    calibrated on the flat-wavefront focal-plane frame."""
    import oopao_gb300 as og
    tel, ngs, dm, wfs, _ = system
    rng = np.random.default_rng(3)
    m2c = rng.standard_normal((dm.nValidAct, 20))
    with _quiet():
        calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, method='jvp')
        dm.coefs = m2c
        ngs ** tel * dm
        basis = np.array(tel.OPD)
        dm.coefs = 0
        gsc = og.GainSensingCamera(wfs.mask, basis)
        wfs.focal_plane_camera.resolution = wfs.nRes
        ngs ** tel * wfs
        wfs * wfs.focal_plane_camera
        wfs.focal_plane_camera * gsc
    return m2c, np.asarray(calib.M), gsc


def test_gsc_loop_graph_equals_eager(system, gsc_system):
    import torch
    from oopao_gb300.closed_loop import ClosedLoop, VonKarmanLayers
    tel, ngs, dm, wfs, _ = system
    m2c, M, gsc = gsc_system
    layers = VonKarmanLayers(tel, r0=0.15, L0=25, windSpeed=(10.,), seed=4)
    cl = ClosedLoop(tel, ngs, dm, wfs, M, gain=0.3, layers=layers, gsc=gsc, M2C=m2c, og_start=3, max_steps=40)
    cl.reset()
    cl.run(8, graph=False)
    eager = cl.coefs.clone()
    og_eager = cl.og.clone()
    cl.capture()
    cl.run(8)
    # the focal-plane frame is summed over modulation points with float
    # atomics, so the gains (and the commands after og_start) agree to
    # round-off rather than bit for bit
    assert O.rel_l2(cl.coefs.double().cpu().numpy(), eager.double().cpu().numpy()) < 1e-5
    assert O.rel_l2(cl.og.cpu().numpy(), og_eager.cpu().numpy()) < 1e-6
    # the gains inside the loop are the camera's gains of the loop's focal frame
    gsc.compute_optical_gains(cl.focal[0])
    assert O.rel_l2(cl.og[0].cpu().numpy(), gsc.og) < 1e-6
    assert np.all(np.isfinite(gsc.og)) and not np.allclose(gsc.og, 1.0)


def test_gsc_loop_without_compensation_is_the_plain_loop(system, gsc_system):
    """og_start beyond the run: M2C @ (M @ s) in two GEMVs equals the plain
    loop with R = M2C @ M (float32 summation order only)."""
    from oopao_gb300.closed_loop import ClosedLoop, VonKarmanLayers
    tel, ngs, dm, wfs, _ = system
    m2c, M, gsc = gsc_system
    layers = VonKarmanLayers(tel, r0=0.15, L0=25, windSpeed=(10.,), seed=4)
    a = ClosedLoop(tel, ngs, dm, wfs, M, gain=0.3, layers=layers, gsc=gsc, M2C=m2c, og_start=10 ** 6, max_steps=40)
    a.reset()
    a.run(10, graph=False)
    b = ClosedLoop(tel, ngs, dm, wfs, m2c @ M, gain=0.3, layers=layers, max_steps=40)
    b.reset()
    b.run(10, graph=False)
    assert O.rel_l2(a.coefs.double().cpu().numpy(), b.coefs.double().cpu().numpy()) < 1e-4
