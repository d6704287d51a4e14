"""Gain-sensing-camera oracle against golden vectors made by the unmodified
reference (``tests/golden/make_golden.py`` cases gsc_*), and the identities
the GPU kernels are built on."""
import json
import os

import numpy as np
import pytest

from oracle import gsc_oracle as G

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.fixture(scope='module', params=['gsc_tiny', 'gsc_small'])
def golden(request):
    z = np.load(os.path.join(HERE, request.param + '.npz'))
    return {k: z[k] for k in z.files}


def test_oracle_matches_reference(golden):
    d = golden
    g = G.OracleGSC(d['mask'], d['basis'])
    g.calibration(d['calib_frame'])
    assert rel(g.IR_calib, d['ir_calib']) < 1e-12
    assert rel(g.sensi_calib, d['sensi_calib']) < 1e-12
    g.compute_optical_gains(d['sky_frame'])
    assert rel(g.IR_sky, d['ir_sky']) < 1e-12
    assert rel(g.og, d['og']) < 1e-12
    p = json.loads(str(d['params']))
    assert g.og.shape == (p['n_modes'],)
    # the screen lowers the gains (a calibrated flat wavefront gives 1)
    assert np.all(d['og'] < 1) and np.all(d['og'] > 0.5)


def test_gains_at_calibration_point_are_one(golden):
    d = golden
    g = G.OracleGSC(d['mask'], d['basis'])
    g.calibration(d['calib_frame'])
    g.compute_optical_gains(d['calib_frame'] * 3.0)   # normalised to unit sum
    np.testing.assert_allclose(g.og, 1.0, rtol=0, atol=1e-12)


@pytest.mark.parametrize('n', [8, 72, 264])
def test_centred_transform_is_signed_fft(n):
    """fftshift(fft2(fftshift(x)))/n == s FFT2(s x)/n and the inverse analogue,
    s = (-1)^(r+c), for even n: the form the kernels evaluate."""
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    r, c = np.indices((n, n))
    s = np.where((r + c) % 2, -1.0, 1.0)
    np.testing.assert_allclose(G.centred_fft2(x), s * np.fft.fft2(s * x) / n, rtol=0, atol=1e-12 * n)
    np.testing.assert_allclose(G.centred_ifft2(x), s * np.fft.ifft2(s * x) * n * n / n, rtol=0, atol=1e-12 * n)


def test_basis_product_is_power_spectrum(golden):
    """fft3(b) * ifft3(b) = |fft3(b)|^2 for a real mode: the GPU keeps it real."""
    d = golden
    n = d['mask'].shape[0]
    bp = G.basis_product(d['basis'][:, :, :3], n)
    ref = np.abs(G.centred_fft2(G.pad_basis(d['basis'][:, :, :3], n), axes=(0, 1))) ** 2
    assert np.abs(bp.imag).max() <= 1e-14 * np.abs(bp.real).max()
    assert rel(bp.real, ref) < 1e-14


def test_padder_rejects_small_output():
    with pytest.raises(ValueError):
        G.pad_basis(np.zeros((8, 8, 1)), 8)
