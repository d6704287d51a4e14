"""Every postProcessing normalisation of the drop-in Pyramid and the detector
binning, against golden vectors made by the unmodified reference (case
modes_tiny: 24 px, 4x4 pyramid, modulation 3, one DM shape).  FP32 path
bound: relative L2 <= 1e-5."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
TOL = 1e-5


@pytest.fixture(scope='module')
def golden():
    z = np.load(os.path.join(HERE, 'modes_tiny.npz'))
    return {k: z[k] for k in z.files}


MODES = ['slopesMaps', 'slopesMaps_incidence_flux', 'slopesMaps_camera_flux', 'fullFrame_camera_flux',
         'fullFrame_incidence_flux', 'fullFrame_sum_flux', 'fullFrame', 'binning2']


@pytest.mark.parametrize('mode', MODES)
def test_postprocessing_and_binning(golden, mode):
    import oopao_gb300 as og
    d = golden
    p = json.loads(str(d['params']))
    kw = dict(binning=2) if mode == 'binning2' else dict(postProcessing=mode)
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'],
                         lightRatio=p['light_ratio'], **kw)
    assert wfs.nSignal == int(d[mode + '_n_signal'])
    dm.coefs = d['coefs']
    ngs ** tel * dm * wfs
    assert np.asarray(wfs.cam.frame).shape == d[mode + '_frame'].shape
    assert O.rel_l2(wfs.cam.frame, d[mode + '_frame']) < TOL
    assert O.rel_l2(wfs.signal_2D, d[mode + '_signal_2D']) < TOL
    assert O.rel_l2(wfs.signal, d[mode + '_signal']) < TOL
