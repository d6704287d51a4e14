"""Host-only parts of the drop-in API (no GPU): the sensors' full-quadrant
blocks of a given frame, the optical-path printers, the detector's host
binning helpers, the calibration vault's truncation setter."""
import numpy as np


def test_full_quadrant_blocks():
    """grabFullQuadrant of both sensors on even and odd frames: the half size
    n_tot // 2 and the negative starts -n_tot // 2 of the reference
    (OOPAO/Pyramid.py:963-976, OOPAO/BioEdge.py:855-868)."""
    import types
    from oopao_gb300.bioedge import BioEdge
    from oopao_gb300.pyramid import Pyramid
    for n_tot, h in ((44, 22), (45, 22)):
        f = np.arange(n_tot * n_tot, dtype=float).reshape(n_tot, n_tot)
        o = types.SimpleNamespace(cam=types.SimpleNamespace(resolution=n_tot, frame=f))
        lo, hi = slice(None, h), slice(n_tot - (n_tot + 1) // 2, None)
        want_pyr = {3: f[lo, lo], 4: f[lo, hi], 1: f[hi, hi], 2: f[hi, lo]}
        want_be = {4: f[lo, lo], 3: f[lo, hi], 1: f[hi, hi], 2: f[hi, lo]}
        for q in (1, 2, 3, 4):
            np.testing.assert_array_equal(Pyramid.grabFullQuadrant(o, q), want_pyr[q])
            np.testing.assert_array_equal(BioEdge.grabFullQuadrant(o, q), want_be[q])


def test_print_optical_path(capsys):
    """Source and Telescope print_optical_path (OOPAO/Source.py:197-204,
    OOPAO/Telescope.py:575-585) after a host-only relay through the telescope."""
    import oopao_gb300 as og
    tel = og.Telescope(resolution=16, diameter=8.0, samplingTime=1e-3)
    ngs = og.Source(optBand='V0', magnitude=8)
    ngs * tel
    capsys.readouterr()
    ngs.print_optical_path()
    tel.print_optical_path()
    out = capsys.readouterr().out.splitlines()
    assert out == ['NGS(V0) ~~> telescope', 'No light propagated through the telescope']


def test_detector_binning_helpers():
    """Detector.rebin and Detector.set_binning on host arrays
    (OOPAO/Detector.py:174-183): block sums."""
    import oopao_gb300 as og
    cam = og.Detector(8)
    a = np.arange(64, dtype=float).reshape(8, 8)
    want = a.reshape(4, 2, 4, 2).sum(axis=(1, 3))
    np.testing.assert_allclose(cam.rebin(a, (4, 4)), want, rtol=1e-15)
    np.testing.assert_array_equal(cam.set_binning(a, 2), want)
    np.testing.assert_array_equal(cam.set_binning(a, 2, mode='mean'), want / 4)


def test_vault_truncation_setter():
    """CalibrationVault.nTrunc setter (OOPAO/calibration/CalibrationVault.py):
    the truncated inverse and reconstruction from the stored U, s, V on the
    host, against the reference's Mtrunc (nTrunc=1) of the im_offset_tiny
    golden.  The thin SVD is taken in numpy here; the vault's own SVD runs on
    the GPU."""
    import os
    from oopao_gb300.calibration import CalibrationVault
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'im_offset_tiny.npz'))
    for tag in ('pp', 'sp'):
        D = z[tag + '_D_offset']
        U, s, Vh = np.linalg.svd(D, full_matrices=False)
        v = CalibrationVault.__new__(CalibrationVault)
        v.s = v.eigenValues = s
        v.U, v.V = U.T, Vh
        v.nTrunc = 1
        np.testing.assert_allclose(v.Mtrunc, z[tag + '_Mtrunc'], rtol=1e-9, atol=1e-9 * np.abs(v.Mtrunc).max())
        assert v.Dtrunc.shape == D.shape and v.Vtrunc.shape == (len(s) - 1, D.shape[1])
        assert v.cond == s[0] / s[-2]
        # no truncation: the plain pseudo-inverse
        v.nTrunc = 0
        np.testing.assert_allclose(v.Mtrunc, np.linalg.pinv(D), rtol=1e-9, atol=1e-9 * np.abs(v.Mtrunc).max())
