"""Pin the Bi-O Edge oracle against golden vectors made by the unmodified
reference (tests/golden/make_golden.py, BIOEDGE_CASES)."""
import json
import os

import numpy as np
import pytest

from oracle import bioedge_oracle as B
from oracle import pwfs_oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = ['bioedge_tiny', 'bioedge_grey']
TOL = 1e-10


def load(name):
    z = np.load(os.path.join(HERE, name + '.npz'))
    d = {k: z[k] for k in z.files}
    d['params'] = json.loads(str(d['params']))
    return d


def oracle_bioedge(d):
    p = d['params']
    return B.build_bioedge(p['res'], p['n_subap'], p['modulation'], p['light_ratio'], d['intensity'],
                           n_pix_separation=p.get('n_pix_separation', 2.), n_theta_user=p.get('nTheta_user_defined'),
                           grey_width=p.get('grey_width', 0.), grey_length=p.get('grey_length', False),
                           quadrants_numbering=p.get('quadrants_numbering', (0, 1, 2, 3)))


@pytest.fixture(scope='module', params=CASES)
def case(request):
    d = load(request.param)
    return d, oracle_bioedge(d)


def test_masks_and_geometry(case):
    d, b = case
    np.testing.assert_allclose(b.masks, d['masks'], rtol=0, atol=1e-14)
    assert b.geom.N == int(d['N']) and b.geom.cam == int(d['cam'])
    assert b.n_theta == int(d['n_theta'])
    np.testing.assert_array_equal(b.valid_i4q, d['valid_i4q'])
    assert O.rel_l2(b.reference_2d, d['reference_2d']) < TOL


def test_dm_and_screen_measurements(case):
    d, b = case
    assert O.rel_l2(b.raw(d['dm_phase']), d['dm_raw']) < TOL
    f, s2d, s = b.measure(d['dm_phase'])
    assert O.rel_l2(f, d['dm_frame']) < TOL
    assert O.rel_l2(s2d, d['dm_signal_2D']) < TOL
    assert O.rel_l2(s, d['dm_signal']) < TOL
    f, s2d, s = b.measure(d['screen_phase'])
    assert O.rel_l2(f, d['screen_frame']) < TOL
    assert O.rel_l2(s, d['screen_signal']) < TOL


def test_focal_plane_camera(case):
    d, b = case
    f = b.focal(d['dm_phase'])
    assert int(d['n_focal_fields']) == 4 * b.tt.shape[0]
    assert O.rel_l2(f, d['dm_focal']) < TOL
    n, m = f.shape[0], d['dm_focal_cam'].shape[0]
    crop = f[n // 2 - m // 2:n // 2 + m // 2, n // 2 - m // 2:n // 2 + m // 2]
    assert O.rel_l2(crop, d['dm_focal_cam']) < TOL


@pytest.mark.parametrize('kw', [dict(), dict(grey_width=1.0, quadrants_numbering=(2, 3, 0, 1)),
                                dict(grey_width=0.5, grey_length=2, sx=[1, 0, -1, 0.5], sy=[0, 1, 0.5, -1]),
                                dict(sx=0.5, sy=-0.25)],
                         ids=['plain', 'grey_numbering', 'grey_length_shifts', 'scalar_shift'])
def test_drop_in_bioedge_masks_match_the_oracle(kw):
    """The drop-in BioEdge's host mask builder against the pinned oracle (no
    GPU needed)."""
    from oopao_gb300.bioedge import bioedge_masks
    res, ns, sep = 32, 4, 2
    edge = sep // 2
    n = int((ns * 2 + sep + edge * 2) * res / ns)
    zp = n / res
    got = np.asarray(bioedge_masks(n, res, ns, zp, **kw))
    want = np.asarray(B.bioedge_masks(res, ns, sep, edge, **kw))
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
