"""Mis-registered DeformableMirror of the drop-in package against golden
vectors made by the unmodified reference (case misreg_tiny): coordinates and
influence functions (host float64, round-off), the frame and slopes of one
DM shape through the mirror (FP32 path, relative L2 <= 1e-5)."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


@pytest.fixture(scope='module')
def golden():
    z = np.load(os.path.join(HERE, 'misreg_tiny.npz'))
    d = {k: z[k] for k in z.files}
    d['params'] = json.loads(str(d['params']))
    return d


@pytest.mark.parametrize('tag', ['rot_shift', 'anamorphosis'])
def test_misregistered_dm(golden, tag):
    import oopao_gb300 as og
    d = golden
    p = d['params']
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'], lightRatio=p['light_ratio'])
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35,
                                 misReg=og.MisRegistration(p['misreg'][tag]))
    np.testing.assert_allclose(dm.coordinates, d[tag + '_coordinates'], rtol=0, atol=1e-12)
    np.testing.assert_allclose(dm.modes, d[tag + '_modes'], rtol=1e-12, atol=1e-300)
    dm.coefs = d['coefs']
    ngs ** tel * dm * wfs
    assert O.rel_l2(wfs.cam.frame, d[tag + '_frame']) < 1e-5
    assert O.rel_l2(wfs.signal, d[tag + '_signal']) < 1e-5
