"""Loader for the golden fixtures in tests/golden (written by make_golden.py)."""
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = ['tiny', 'tiny_nocenter', 'tiny_rooftop', 'tiny_nomod', 'small_sep', 'c1', 'tiny_sf', 'tiny_nocenter_sf']


def load(name):
    with np.load(os.path.join(GOLDEN_DIR, name + '.npz')) as z:
        d = {k: z[k] for k in z.files}
    d['params'] = json.loads(str(d['params']))
    return d


def oracle_pyramid(d):
    """Build the oracle sensor with the fixture's construction parameters."""
    from oracle import pwfs_oracle as O
    p = d['params']
    return O.build_pyramid(
        p['res'], p['n_subap'], p['modulation'], p['light_ratio'], d['intensity'],
        n_pix_separation=p.get('n_pix_separation', 2), n_pix_edge=p.get('n_pix_edge'),
        psf_centering=p.get('psfCentering', True), n_theta_user=p.get('nTheta_user_defined'),
        rooftop=p.get('rooftop', 0.0), theta_rotation=p.get('theta_rotation', 0.0),
        spatial_filter=d.get('spatial_filter'))
