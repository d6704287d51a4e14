"""The drop-in InteractionMatrix with and without a phaseOffset against the
reference's D and Mtrunc (case im_offset_tiny; the reference's offset does
not reach the measured signals).  FP32 path: relative L2 <= 1e-5 (IM columns
<= 1e-4)."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


@pytest.mark.parametrize('tag, single_pass', [('pp', False), ('sp', True)])
def test_im_with_phase_offset(tag, single_pass):
    import oopao_gb300 as og
    z = np.load(os.path.join(HERE, 'im_offset_tiny.npz'))
    d = {k: z[k] for k in z.files}
    p = json.loads(str(d['params']))
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'], lightRatio=p['light_ratio'])
        calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=d['m2c'], stroke=1e-8, nMeasurements=2, nTrunc=1,
                                     phaseOffset=d['offset'], single_pass=single_pass)
    assert O.rel_l2(calib.D, d[tag + '_D_offset']) < 1e-4
    assert O.rel_l2(calib.Mtrunc, d[tag + '_Mtrunc']) < 1e-4
