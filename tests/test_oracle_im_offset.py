"""InteractionMatrix with a phaseOffset, against golden vectors made by the
unmodified reference (case im_offset_tiny: 24 px, 4x4 pyramid, 4 random
modal columns in chunks of 2, push-pull and single pass).  The reference adds
the offset to ngs.phase only after the pull is measured
(OOPAO/calibration/InteractionMatrix.py:126-133), so D is the same with and
without it; the oracle's column rule reproduces both at round-off."""
import json
import os

import numpy as np
import pytest

from oracle import pwfs_oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


@pytest.fixture(scope='module')
def golden():
    z = np.load(os.path.join(HERE, 'im_offset_tiny.npz'))
    d = {k: z[k] for k in z.files}
    d['params'] = json.loads(str(d['params']))
    return d


@pytest.mark.parametrize('tag, single_pass', [('pp', False), ('sp', True)])
def test_offset_leaves_d_unchanged(golden, tag, single_pass):
    d = golden
    p = d['params']
    np.testing.assert_array_equal(d[tag + '_D'], d[tag + '_D_offset'])
    pupil = O.telescope_pupil(p['res'])
    inten = O.source_intensity(pupil, O.n_photon('V0', 8), 1e-3, 8.0)
    wfs = O.build_pyramid(p['res'], p['n_subap'], p['modulation'], p['light_ratio'], inten)
    modes = O.dm_modes(p['res'], 8.0, p['n_subap'])
    D = O.interaction_matrix(wfs, modes, d['m2c'], 1e-8, O.PHOTOMETRY['V0'][0], pupil, single_pass=single_pass)
    assert O.rel_l2(D, d[tag + '_D_offset']) < 1e-9
