"""GPU parity of the drop-in Pyramid / DeformableMirror against the reference
golden vectors (float64 reference run) and the CPU oracle.

Tolerances (FP32 path): relative L2 <= 1e-5 for frames, raw_data, signal_2D
and signal; valid-pixel maps must be identical.
"""
import contextlib
import io

import numpy as np
import pytest

from oracle import pwfs_oracle as O
from tests import goldens as G

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


def build_system(d):
    import oopao_gb300 as og
    p = d['params']
    kw = {k: v for k, v in p.items() if k not in ('res', 'n_subap', 'modulation', 'light_ratio', 'co', 'sf_radius')}
    with _quiet():
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3, centralObstruction=p['co'])
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'],
                         lightRatio=p['light_ratio'], **kw)
        if 'spatial_filter' in d:
            wfs.spatialFilter = d['spatial_filter']
    return tel, ngs, dm, wfs


def rel(a, b):
    return O.rel_l2(a, b)


@pytest.fixture(scope='module', params=G.CASES)
def system(request):
    d = G.load(request.param)
    return request.param, d, build_system(d)


def test_geometry_and_valid_pixels(system):
    name, d, (tel, ngs, dm, wfs) = system
    assert wfs.resolution == int(d['N'])
    assert wfs.cam.resolution == int(d['cam'])
    assert wfs.nTheta == int(d['n_theta'])
    assert dm.nValidAct == int(d['n_act'])
    np.testing.assert_array_equal(wfs.validI4Q, d['valid_i4q'])
    assert wfs.nSignal == int(d['n_signal'])
    if 'mask' in d:
        # transcendental functions may differ by one ulp between host libms
        np.testing.assert_allclose(wfs.mask, d['mask'], rtol=0, atol=2e-7)
        np.testing.assert_allclose(dm.modes, d['modes'], rtol=1e-14, atol=1e-300)


def test_reference_signal(system):
    name, d, (tel, ngs, dm, wfs) = system
    # a symmetric geometry makes the float64 reference pure round-off (~1e-16);
    # measure the error against the slope scale of an aberrated measurement
    ref = d['reference_2d']
    scale = max(np.linalg.norm(ref), np.linalg.norm(d['dm_signal_2D']))
    err = np.linalg.norm(wfs.referenceSignal_2D - ref) / scale
    assert err < TOL_FP32, err


def test_dm_path(system):
    name, d, (tel, ngs, dm, wfs) = system
    dm.coefs = d['dm_coefs']
    ngs ** tel * dm * wfs
    assert rel(ngs.phase, d['dm_phase']) < 1e-6
    assert rel(wfs.cam.frame, d['dm_frame']) < TOL_FP32
    if 'dm_raw' in d:
        assert rel(wfs.raw_data, d['dm_raw']) < TOL_FP32
    assert rel(wfs.signal_2D, d['dm_signal_2D']) < TOL_FP32
    assert rel(wfs.signal, d['dm_signal']) < TOL_FP32


def test_focal_plane_camera(system):
    """``wfs * wfs.focal_plane_camera`` after the DM measurement: the summed
    |F/N|^2 of the modulation points and the camera's centred crop."""
    name, d, (tel, ngs, dm, wfs) = system
    dm.coefs = d['dm_coefs']
    ngs ** tel * dm * wfs
    assert rel(wfs.focal_plane_image(), d['dm_focal']) < TOL_FP32
    wfs * wfs.focal_plane_camera
    assert wfs.focal_plane_camera.frame.shape == d['dm_focal_cam'].shape
    assert rel(wfs.focal_plane_camera.frame, d['dm_focal_cam']) < TOL_FP32
    # the signal of the measurement is unchanged by the extra propagation
    assert rel(wfs.signal, d['dm_signal']) < TOL_FP32


def test_screen_path(system):
    name, d, (tel, ngs, dm, wfs) = system
    dm.coefs = 0
    ngs ** tel
    wfs.wfs_measure(phase_in=d['screen_phase'])
    assert rel(wfs.cam.frame, d['screen_frame']) < TOL_FP32
    if 'screen_raw' in d:
        assert rel(wfs.raw_data, d['screen_raw']) < TOL_FP32
    assert rel(wfs.signal, d['screen_signal']) < TOL_FP32


@pytest.mark.parametrize('method', ['batched', 'per_mode'])
def test_interaction_matrix(system, method):
    name, d, (tel, ngs, dm, wfs) = system
    if 'im_D' not in d:
        pytest.skip('no interaction matrix in this fixture')
    import oopao_gb300 as og
    calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=d['im_m2c'], stroke=1e-8, nMeasurements=4,
                                 single_pass=True, method=method)
    # stroke 1e-8 m: the column is a difference of O(1) slopes; FP32 cancellation
    # makes 1e-4 the meaningful bound here
    assert rel(calib.D, d['im_D']) < 1e-4
    # the float64 pseudo-inverse of the same matrix matches the reference's SVD
    ref_vault = og.CalibrationVault(d['im_D'])
    assert rel(ref_vault.M, d['im_M']) < 1e-10
    # the optional host eigensolver gives the same reconstructor
    host_vault = og.CalibrationVault(d['im_D'], host_eigensolver=True)
    assert rel(host_vault.M, d['im_M']) < 1e-10
    calib_pp = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=d['im_m2c'], stroke=1e-8, single_pass=False,
                                    method=method)
    assert rel(calib_pp.D, d['im_pp_D']) < 1e-4


def test_batched_phase_cube(system):
    """3-D phase input (all modes x points in one launch) equals per-map calls."""
    name, d, (tel, ngs, dm, wfs) = system
    rng = np.random.default_rng(7)
    res = tel.resolution
    cube = rng.standard_normal((res, res, 3)) * tel.pupil[:, :, None]
    ngs ** tel
    wfs.wfs_measure(phase_in=cube)
    s_batch = wfs.signal.copy()
    assert s_batch.shape == (wfs.nSignal, 3)
    for i in range(3):
        ngs ** tel
        wfs.wfs_measure(phase_in=cube[:, :, i])
        # the slot split over modulation points depends on the batch size, so
        # the FP32 sums are ordered differently: the FP32-path bound applies
        assert rel(s_batch[:, i], wfs.signal) < 1e-5
    # and against the oracle
    wo = G.oracle_pyramid(d)
    _, _, _, s_or = wo.measure(cube)
    assert rel(s_batch, s_or) < TOL_FP32
