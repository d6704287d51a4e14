"""CPU checks of the atmosphere: the oracle against the reference's own OPD
sequence (golden, made with the scikit-image warp restated), and the
package's host screen generators against the oracle."""
import json
import os

import numpy as np

from oracle import atm_oracle as A

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'atm_small.npz')


def _golden():
    z = np.load(GOLDEN)
    return {k: z[k] for k in z.files}, json.loads(str(z['params']))


def test_oracle_matches_reference_atmosphere():
    d, p = _golden()
    atm = A.OracleAtmosphere(p['res'], p['diameter'], 1e-3, p['r0'], p['L0'], p['fractionalR0'], p['windSpeed'],
                             p['windDirection'], p['altitude'])
    L = atm.layers[0]
    assert np.abs(L.A - d['A']).max() < 1e-9 * np.abs(d['A']).max()
    assert np.abs(L.B - d['B']).max() < 1e-9 * np.abs(d['B']).max()
    ref = d['opd']
    assert np.linalg.norm(atm.opd - ref[0]) < 1e-12 * np.linalg.norm(ref[0])
    for t in range(p['steps']):
        atm.update()
        assert np.linalg.norm(atm.opd - ref[t + 1]) < 1e-9 * np.linalg.norm(ref[t + 1]), t


def test_oracle_matches_reference_boiling():
    z = np.load(os.path.join(os.path.dirname(GOLDEN), 'atm_boil.npz'))
    p = json.loads(str(z['params']))
    atm = A.OracleAtmosphere(p['res'], p['diameter'], 1e-3, p['r0'], p['L0'], p['fractionalR0'], p['windSpeed'],
                             p['windDirection'], p['altitude'], t_boiling=p['t_boiling'])
    ref = z['opd']
    assert np.linalg.norm(atm.opd - ref[0]) < 1e-12 * np.linalg.norm(ref[0])
    for t in range(p['steps']):
        atm.update()
        assert np.linalg.norm(atm.opd - ref[t + 1]) < 1e-9 * np.linalg.norm(ref[t + 1]), t
    # the still layer changes only through boiling
    assert np.linalg.norm(ref[1] - ref[0]) > 0.05 * np.linalg.norm(ref[0])


def test_package_screens_equal_oracle():
    from oopao_gb300 import atmosphere as P
    for seed in (0, 3):
        a = P.ft_sh_phase_screen(0.15, 25.0, 36, 0.25, seed=seed)
        b = A.ft_sh_phase_screen(0.15, 25.0, 36, 0.25, seed=seed)
        np.testing.assert_array_equal(a, b)
    rng = np.random.default_rng(0)
    z1 = rng.standard_normal(20) + 1j * rng.standard_normal(20)
    z2 = rng.standard_normal(7) + 1j * rng.standard_normal(7)
    np.testing.assert_allclose(P.phase_covariance(z1, z2, 25.0), A.covariance_matrix(z1, z2, 25.0), rtol=1e-14)


def test_cubic_shift_properties():
    img = np.random.default_rng(1).standard_normal((12, 12))
    # integer shifts are exact moves, zero-filled at the edge
    s = A.cubic_shift(img, 1.0, -1.0)
    np.testing.assert_array_equal(s[:-1, 1:], img[1:, :-1])
    # no shift is the identity; a sub-pixel shift stays inside the input range
    np.testing.assert_array_equal(A.cubic_shift(img, 0.0, 0.0), img)
    s = A.cubic_shift(img, 0.3, 0.7)
    assert s.min() >= img.min() and s.max() <= img.max()


def test_boiling_arguments():
    """t_boiling: a scalar for every layer, a list per layer, anything else an
    error; which layers boil and their AR(1) coefficients (host only)."""
    import contextlib
    import io
    import pytest
    import oopao_gb300 as og
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=32, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
    kw = dict(telescope=tel, r0=0.15, L0=25.0, fractionalR0=[0.5, 0.5], windSpeed=[1.0, 2.0],
              windDirection=[0.0, 0.0], altitude=[0.0, 1000.0])
    atm = og.Atmosphere(t_boiling=0.01, **kw)
    assert atm.t_boiling == [0.01, 0.01]
    with pytest.raises(og.OopaoError, match='t_boiling'):
        og.Atmosphere(t_boiling=[0.01], **kw)
    assert og.Atmosphere(**kw).t_boiling == [None, None]
    # frozen: None, non-positive, non-finite, or alpha within 1e-6 of 1
    atm.t_boiling = [None, 1e9]
    assert atm._boil_coefs() == []
    atm.t_boiling = [-1.0, float('inf')]
    assert atm._boil_coefs() == []
    atm.t_boiling = [None, 0.005]
    (i, a, b), = atm._boil_coefs()
    assert i == 1 and a == np.exp(-0.2) and abs(a * a + b * b - 1) < 1e-15
