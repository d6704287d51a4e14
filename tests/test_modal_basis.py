"""KL modal basis against the reference's compute_KL_basis (golden made by
the unmodified reference).  Tip and tilt (the fitted specific modes) must
match column for column; KL modes of equal modal variance span a space in
which the basis is not unique, so they are compared cluster by cluster
through their projectors in the pupil metric."""
import json
import os
import types

import numpy as np
import pytest

from oracle import pwfs_oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def _system(res, n_subap, r0, L0):
    pupil = O.telescope_pupil(res)
    tel = types.SimpleNamespace(pupil=pupil, resolution=res, D=8.0)
    atm = types.SimpleNamespace(r0=r0, L0=L0)
    dm = types.SimpleNamespace(modes=O.dm_modes(res, 8.0, n_subap), nValidAct=O.dm_modes(res, 8.0, n_subap).shape[1],
                               isM4=False)
    return tel, atm, dm


def _compare(name):
    from oopao_gb300.modal_basis import compute_KL_basis
    z = np.load(os.path.join(HERE, name + '.npz'))
    p = json.loads(str(z['params']))
    tel, atm, dm = _system(p['res'], p['n_subap'], p['r0'], p['L0'])
    m2c = compute_KL_basis(tel, atm, dm)
    ref = z['m2c']
    assert m2c.shape == ref.shape
    ip = tel.pupil.reshape(-1) > 0
    F = dm.modes[ip]
    mine, theirs = F @ m2c, F @ ref
    npup = ip.sum()
    # orthonormal over the pupil (the construction's normalisation)
    gram = mine.T @ mine / npup
    assert np.abs(gram - np.eye(gram.shape[0])).max() < 1e-8
    # tip, tilt: column for column
    for c in range(2):
        assert np.linalg.norm(mine[:, c] - theirs[:, c]) < 1e-6 * np.linalg.norm(theirs[:, c])
    # KL modes: clusters of equal variance, compared by projectors
    var = compute_KL_basis.last_variances
    k0, i = 2, 0
    while i < len(var):
        j = i + 1
        while j < len(var) and abs(var[j] - var[i]) <= 1e-6 * abs(var[i]):
            j += 1
        a, b = mine[:, k0 + i:k0 + j], theirs[:, k0 + i:k0 + j]
        # both sets are orthonormal over the pupil: equal spans <=> all the
        # cosines of the principal angles (singular values of a^T b) are 1
        cos = np.linalg.svd(a.T @ b / npup, compute_uv=False)
        assert np.all(np.abs(cos - 1) < 1e-6), (i, j, cos)
        i = j
    return m2c


def test_kl_basis_tiny():
    _compare('kl_tiny')


def test_kl_basis_20x20():
    _compare('kl_c1')
