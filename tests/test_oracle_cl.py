"""CPU checks of the oracle's closed loop and science image."""
import numpy as np

from oracle import pwfs_oracle as O


def test_flat_wavefront_strehl_is_100():
    res = 24
    pup = O.telescope_pupil(res)
    inten = O.source_intensity(pup, O.n_photon('V0', 8), 1e-3, 8.0)
    psf = O.science_psf(np.zeros((res, res)), inten, pup, 500e-9)
    assert psf.shape == (2 * res, 2 * res)
    # energy: Parseval with the 1/N normalisation of the field
    assert np.isclose(psf.sum(), inten.sum(), rtol=1e-12)
    assert np.isclose(O.strehl_meter(psf, psf), 100.0)
    x = np.linspace(-1, 1, res)
    xx, yy = np.meshgrid(x, x)
    tilt = xx * 300e-9
    defocus = (xx ** 2 + yy ** 2) * 100e-9
    # the OTF-modulus ratio ignores a pure tilt (a shift of the image)
    assert np.isclose(O.strehl_meter(O.science_psf(tilt, inten, pup, 500e-9), psf), 100.0)
    assert O.strehl_meter(O.science_psf(defocus, inten, pup, 500e-9), psf) < 90.0


def test_oracle_loop_corrects_a_static_dm_shape():
    res, nsub = 24, 4
    pup = O.telescope_pupil(res)
    inten = O.source_intensity(pup, O.n_photon('V0', 8), 1e-3, 8.0)
    w = O.build_pyramid(res, nsub, 3, 0.5, inten)
    modes = O.dm_modes(res, 8.0, nsub)
    D = O.interaction_matrix(w, modes, np.eye(modes.shape[1]), 1e-8, 500e-9, pup, single_pass=False)
    R = np.linalg.pinv(D, rcond=1e-6)   # drops the modes the sensor does not see
    aberr = (modes @ (np.random.default_rng(0).standard_normal(modes.shape[1]) * 20e-9)).reshape(res, res)
    out = O.closed_loop(w, modes, R, lambda t: aberr, pup, 500e-9, 0.5, 25)
    assert out['wfe'][-1] < 0.02 * out['wfe'][0]
    assert out['strehl_le'] > 0
