"""Pin the CPU oracle against golden vectors produced by the unmodified reference.

The reference computes in float64 with pocketfft; the oracle restates the
same algorithm in float64, so agreement is at round-off level (1e-10 relative
is a loose bound; typical agreement is 1e-14).
"""
import numpy as np
import pytest

from oracle import pwfs_oracle as O
from tests import goldens as G

TOL = 1e-10


@pytest.fixture(scope='module', params=G.CASES)
def case(request):
    d = G.load(request.param)
    return request.param, d, G.oracle_pyramid(d)


def test_geometry(case):
    name, d, wfs = case
    p = d['params']
    assert wfs.geom.N == int(d['N'])
    assert wfs.geom.cam == int(d['cam'])
    assert wfs.n_theta == int(d['n_theta'])
    pupil = O.telescope_pupil(p['res'], p['co'])
    np.testing.assert_array_equal(pupil, d['pupil'])
    inten = O.source_intensity(pupil, O.n_photon('V0', 8), 1e-3, 8.0)
    np.testing.assert_array_equal(inten, d['intensity'])
    # exact on the machine that wrote the fixtures; other libms may differ by one ulp
    if 'mask' in d:
        np.testing.assert_allclose(wfs.geom.mask, d['mask'], rtol=0, atol=2e-7)
        np.testing.assert_allclose(wfs.geom.phasor, d['phasor'], rtol=0, atol=1e-14)
        np.testing.assert_allclose(wfs.tt, d['tt'], rtol=2e-7, atol=0)
    else:
        np.testing.assert_allclose(wfs.geom.mask[0], d['mask_row0'], rtol=0, atol=2e-7)
        np.testing.assert_allclose(wfs.geom.mask[:, wfs.geom.N // 2 - 3], d['mask_col_mid'], rtol=0, atol=2e-7)
        assert abs(np.real(wfs.geom.mask).astype(np.float64).sum() - d['mask_real_sum']) < 1e-9
        assert abs(np.imag(wfs.geom.mask).astype(np.float64).sum() - d['mask_imag_sum']) < 1e-9


def test_valid_pixels_and_reference(case):
    name, d, wfs = case
    np.testing.assert_array_equal(wfs.valid_i4q, d['valid_i4q'])
    assert int(wfs.valid_signal.sum()) == int(d['n_signal'])
    # a symmetric pupil gives a reference of pure round-off (~1e-16): compare
    # against the O(1) slope scale instead of its own norm
    ref = d['reference_2d']
    err = np.linalg.norm(wfs.reference_2d - ref) / max(np.linalg.norm(ref), 1e-6 * np.sqrt(ref.size))
    assert err < TOL


def test_dm_modes(case):
    name, d, wfs = case
    p = d['params']
    modes = O.dm_modes(p['res'], 8.0, p['n_subap'], 0.35, p['co'])
    assert modes.shape[1] == int(d['n_act'])
    if 'modes' in d:
        np.testing.assert_allclose(modes, d['modes'], rtol=1e-14, atol=1e-300)
    else:
        np.testing.assert_allclose(modes.sum(axis=0), d['modes_colsum'], rtol=1e-13)
        np.testing.assert_allclose(modes[:, 0], d['modes_col0'], rtol=1e-14, atol=1e-300)


def test_dm_path(case):
    name, d, wfs = case
    p = d['params']
    modes = O.dm_modes(p['res'], 8.0, p['n_subap'], 0.35, p['co'])
    opd = O.dm_opd(modes, d['dm_coefs'], p['res']) * d['pupil']
    phase = opd * 2 * np.pi / float(d['wavelength'])
    assert O.rel_l2(phase, d['dm_phase']) < 1e-13
    raw, frame, s2d, s = wfs.measure(phase)
    if 'dm_raw' in d:
        assert O.rel_l2(raw, d['dm_raw']) < TOL
    assert O.rel_l2(frame, d['dm_frame']) < TOL
    assert O.rel_l2(s2d, d['dm_signal_2D']) < TOL
    assert O.rel_l2(s, d['dm_signal']) < TOL


def test_focal_plane_camera(case):
    """Sum over points of |F/N|^2 (modulation_camera_em) and the focal-plane
    camera frame (its centred crop) of the DM measurement."""
    name, d, wfs = case
    img = O.focal_plane_image(d['dm_phase'], wfs.intensity, wfs.tt, wfs.geom)
    assert O.rel_l2(img, d['dm_focal']) < TOL
    n, m = img.shape[0], d['dm_focal_cam'].shape[0]
    if m <= n:
        crop = img[n // 2 - m // 2:n // 2 + m // 2, n // 2 - m // 2:n // 2 + m // 2]
        assert O.rel_l2(crop, d['dm_focal_cam']) < TOL


def test_screen_path(case):
    name, d, wfs = case
    raw, frame, s2d, s = wfs.measure(d['screen_phase'])
    if 'screen_raw' in d:
        assert O.rel_l2(raw, d['screen_raw']) < TOL
    assert O.rel_l2(frame, d['screen_frame']) < TOL
    assert O.rel_l2(s, d['screen_signal']) < TOL


def test_interaction_matrix(case):
    name, d, wfs = case
    if 'im_D' not in d:
        pytest.skip('no IM in this fixture')
    p = d['params']
    modes = O.dm_modes(p['res'], 8.0, p['n_subap'], 0.35, p['co'])
    D = O.interaction_matrix(wfs, modes, d['im_m2c'], 1e-8, float(d['wavelength']), d['pupil'])
    assert O.rel_l2(D, d['im_D']) < 1e-8
    Dpp = O.interaction_matrix(wfs, modes, d['im_m2c'], 1e-8, float(d['wavelength']), d['pupil'],
                               single_pass=False)
    assert O.rel_l2(Dpp, d['im_pp_D']) < 1e-8
    M, _, _, _ = O.calibration_vault(d['im_D'])
    assert O.rel_l2(M, d['im_M']) < 1e-10
