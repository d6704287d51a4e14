"""Pin the CPU oracle on the 40x40 closed-loop optics (golden ``c3``: 240 px,
40x40 pyramid, modulation 5 l/D with 96 points, N = 504, 84x84 camera, 41x41
DM), produced by the unmodified reference: geometry, valid pixels, reference
slopes, the DM and screen measurements, and push-pull interaction-matrix
columns of the reference's own KL modes.  Agreement is float64 round-off."""
import numpy as np
import pytest

from oracle import pwfs_oracle as O
from tests import goldens as G

TOL = 1e-10


@pytest.fixture(scope='module')
def c3():
    d = G.load('c3')
    return d, G.oracle_pyramid(d)


def test_geometry_valid_pixels_reference(c3):
    d, wfs = c3
    assert (wfs.geom.N, wfs.geom.cam, wfs.n_theta) == (504, 84, 96)
    assert (int(d['N']), int(d['cam']), int(d['n_theta'])) == (504, 84, 96)
    np.testing.assert_array_equal(O.telescope_pupil(240), d['pupil'])
    np.testing.assert_allclose(wfs.geom.mask[0], d['mask_row0'], rtol=0, atol=2e-7)
    np.testing.assert_allclose(wfs.geom.mask[:, 504 // 2 - 3], d['mask_col_mid'], rtol=0, atol=2e-7)
    np.testing.assert_array_equal(wfs.valid_i4q, d['valid_i4q'])
    assert int(wfs.valid_signal.sum()) == int(d['n_signal']) == 2528
    ref = d['reference_2d']
    err = np.linalg.norm(wfs.reference_2d - ref) / max(np.linalg.norm(ref), 1e-6 * np.sqrt(ref.size))
    assert err < TOL


def test_dm_and_screen(c3):
    d, wfs = c3
    modes = O.dm_modes(240, 8.0, 40)
    assert modes.shape[1] == int(d['n_act']) == 1353
    np.testing.assert_allclose(modes.sum(axis=0), d['modes_colsum'], rtol=1e-13)
    phase = O.dm_opd(modes, d['dm_coefs'], 240) * d['pupil'] * 2 * np.pi / float(d['wavelength'])
    assert O.rel_l2(phase, d['dm_phase']) < 1e-13
    _, frame, s2d, s = wfs.measure(phase, workers=8)
    assert O.rel_l2(frame, d['dm_frame']) < TOL
    assert O.rel_l2(s2d, d['dm_signal_2D']) < TOL
    assert O.rel_l2(s, d['dm_signal']) < TOL
    _, frame, s2d, s = wfs.measure(d['screen_phase'], workers=8)
    assert O.rel_l2(frame, d['screen_frame']) < TOL
    assert O.rel_l2(s2d, d['screen_signal_2D']) < TOL
    assert O.rel_l2(s, d['screen_signal']) < TOL


def test_push_pull_columns(c3):
    """Two of the reference's 24 KL push-pull columns (stroke 1e-8 m)."""
    d, wfs = c3
    modes = O.dm_modes(240, 8.0, 40)
    D = O.interaction_matrix(wfs, modes, d['im_m2c'][:, [0, 17]], 1e-8, float(d['wavelength']), d['pupil'],
                             single_pass=False, workers=8)
    assert O.rel_l2(D, d['im_pp_D'][:, [0, 17]]) < 1e-9
