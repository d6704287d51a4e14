"""GPU parity on the 40x40 closed-loop optics against the reference's own
Pyramid (golden ``c3``, made by the unmodified reference: 8 m, 240 px, 40x40
pyramid, modulation 5 l/D with 96 points, N = 504, 84x84 camera, 41x41
Gaussian DM), through the drop-in classes ``ngs**tel*dm*wfs``,
``wfs.wfs_measure`` and ``InteractionMatrix``.

Tolerances (FP32 path): relative L2 <= 1e-5 for frames, signal_2D and
signal; identical valid-pixel maps; push-pull IM columns (stroke 1e-8 m, a
difference of O(1) slopes) <= 1e-4 relative Frobenius over all 24 columns;
the tangent IM <= 1e-4 against the reference's float64 derivative.
"""
import contextlib
import io

import numpy as np
import pytest

from oracle import pwfs_oracle as O
from tests import goldens as G

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5


@pytest.fixture(scope='module')
def c3():
    import oopao_gb300 as og
    d = G.load('c3')
    p = d['params']
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'], lightRatio=p['light_ratio'],
                         nTheta_user_defined=p['nTheta_user_defined'], max_batch=16)
    return d, (tel, ngs, dm, wfs)


def test_geometry(c3):
    d, (tel, ngs, dm, wfs) = c3
    assert (wfs.resolution, wfs.cam.resolution, wfs.nTheta) == (504, 84, 96)
    assert dm.nValidAct == int(d['n_act'])
    np.testing.assert_array_equal(wfs.validI4Q, d['valid_i4q'])
    assert wfs.nSignal == int(d['n_signal'])
    np.testing.assert_allclose(dm.modes.sum(axis=0), d['modes_colsum'], rtol=1e-12)
    ref = d['reference_2d']
    scale = max(np.linalg.norm(ref), np.linalg.norm(d['dm_signal_2D']))
    assert np.linalg.norm(wfs.referenceSignal_2D - ref) / scale < TOL_FP32


def test_dm_path_and_focal_camera(c3):
    d, (tel, ngs, dm, wfs) = c3
    dm.coefs = d['dm_coefs']
    ngs ** tel * dm * wfs
    assert O.rel_l2(ngs.phase, d['dm_phase']) < 1e-6
    assert O.rel_l2(wfs.cam.frame, d['dm_frame']) < TOL_FP32
    assert O.rel_l2(wfs.signal_2D, d['dm_signal_2D']) < TOL_FP32
    assert O.rel_l2(wfs.signal, d['dm_signal']) < TOL_FP32
    wfs * wfs.focal_plane_camera
    assert wfs.focal_plane_camera.frame.shape == d['dm_focal_cam'].shape
    assert O.rel_l2(wfs.focal_plane_camera.frame, d['dm_focal_cam']) < TOL_FP32


def test_screen_path(c3):
    d, (tel, ngs, dm, wfs) = c3
    dm.coefs = 0
    ngs ** tel
    wfs.wfs_measure(phase_in=d['screen_phase'])
    assert O.rel_l2(wfs.cam.frame, d['screen_frame']) < TOL_FP32
    assert O.rel_l2(wfs.signal_2D, d['screen_signal_2D']) < TOL_FP32
    assert O.rel_l2(wfs.signal, d['screen_signal']) < TOL_FP32


@pytest.mark.parametrize('method', ['batched', 'per_mode'])
def test_push_pull_interaction_matrix(c3, method):
    d, (tel, ngs, dm, wfs) = c3
    import oopao_gb300 as og
    calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=d['im_m2c'], stroke=1e-8, nMeasurements=1,
                                 single_pass=False, method=method, invert=False)
    assert O.rel_l2(calib.D, d['im_pp_D']) < 1e-4


def test_tangent_interaction_matrix(c3):
    """The interaction matrix from batched tangents (JVPs) against the
    reference's float64 derivative (its own push-pull with a 1e-11 m stroke,
    whose O(stroke^2) truncation is ~1e-9 relative): <= 1e-4 relative
    Frobenius over all 24 columns.  Against the reference's 1e-8 m push-pull
    the distance is that stroke's own truncation, 3.1e-3 between the
    reference's two strokes, so the bound there is 4e-3."""
    d, (tel, ngs, dm, wfs) = c3
    from oopao_gb300.autodiff import jvp_interaction_matrix
    D = jvp_interaction_matrix(ngs, tel, dm, wfs, d['im_m2c']).double().cpu().numpy()
    assert O.rel_l2(D, d['im_fine_D']) < 1e-4
    assert O.rel_l2(D, d['im_pp_D']) < 4e-3
