"""Pin the oracle's mis-registered DM (actuator coordinates, Gaussian
influence functions, the pyramid measurement through the mirror) against
golden vectors made by the unmodified reference (case misreg_tiny: 24 px,
4x4 pyramid, a rotation + shift and an anamorphosis case).  float64 on both
sides."""
import json
import os

import numpy as np
import pytest

from oracle import pwfs_oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


@pytest.fixture(scope='module')
def golden():
    z = np.load(os.path.join(HERE, 'misreg_tiny.npz'))
    d = {k: z[k] for k in z.files}
    d['params'] = json.loads(str(d['params']))
    return d


@pytest.mark.parametrize('tag', ['rot_shift', 'anamorphosis'])
def test_misregistered_dm(golden, tag):
    d = golden
    p = d['params']
    mr = p['misreg'][tag]
    res, ns = p['res'], p['n_subap']
    u0x, u0y, _ = O.dm_actuator_pixels(res, 8.0, ns, 0.0, mr)
    coords = np.stack([(u0x - res / 2) * 8.0 / res, (u0y - res / 2) * 8.0 / res], axis=1)
    np.testing.assert_allclose(coords, d[tag + '_coordinates'], rtol=0, atol=1e-12)
    modes = O.dm_modes(res, 8.0, ns, 0.35, 0.0, mr)
    np.testing.assert_allclose(modes, d[tag + '_modes'], rtol=1e-12, atol=1e-300)
    pupil = O.telescope_pupil(res)
    inten = O.source_intensity(pupil, O.n_photon('V0', 8), 1e-3, 8.0)
    wfs = O.build_pyramid(res, ns, p['modulation'], p['light_ratio'], inten)
    phase = O.dm_opd(modes, d['coefs'], res) * pupil * 2 * np.pi / O.PHOTOMETRY['V0'][0]
    _, frame, _, s = wfs.measure(phase)
    assert O.rel_l2(frame, d[tag + '_frame']) < 1e-10
    assert O.rel_l2(s, d[tag + '_signal']) < 1e-10


def test_misregistration_object(golden):
    """Name, sum and difference of the drop-in MisRegistration (host only)."""
    from oopao_gb300.mis_registration import MisRegistration
    d = golden
    for tag, mr in d['params']['misreg'].items():
        m = MisRegistration(mr)
        assert m.misRegName == str(d[tag + '_name'])
        assert MisRegistration(m) == m
        z = m - m
        assert all(getattr(z, f) == 0 for f in O.MISREG_FIELDS)
        two = m + m
        assert two.rotationAngle == 2 * mr['rotationAngle']


@pytest.mark.parametrize('tag', ['rot_shift', 'anamorphosis'])
def test_dm_host_geometry(golden, tag):
    """The drop-in DM's host-side grid transform and IF construction (no GPU
    needed) against the reference's coordinates and modes."""
    import types
    from oopao_gb300.deformable_mirror import DeformableMirror as DM
    from oopao_gb300.mis_registration import MisRegistration
    d = golden
    p = d['params']
    res, ns = p['res'], p['n_subap']
    mr = MisRegistration(p['misreg'][tag])
    _, _, valid = O.dm_actuator_pixels(res, 8.0, ns)
    x = np.linspace(-4.0, 4.0, ns + 1)
    X, Y = np.meshgrid(x, x)
    x0, y0 = X.reshape(-1)[valid], Y.reshape(-1)[valid]
    x3, y3 = DM.anamorphosis_coordinates(x0, y0, mr.anamorphosisAngle * np.pi / 180, mr.tangentialScaling,
                                         mr.radialScaling)
    x4, y4 = DM.rotate_coordinates(x3, y3, mr.rotationAngle * np.pi / 180)
    coords = np.stack([x4 - mr.shiftX, y4 - mr.shiftY], axis=1)
    np.testing.assert_allclose(coords, d[tag + '_coordinates'], rtol=0, atol=1e-12)
    fake = types.SimpleNamespace(resolution=res, nActAlongDiameter=ns, mechCoupling=0.35, misReg=mr, sign=1,
                                 flip_lr=False, flip_=False, floating_precision=64)
    u0x = res / 2 + coords[:, 0] * res / 8.0
    u0y = res / 2 + coords[:, 1] * res / 8.0
    modes = DM._gaussian_modes(fake, u0x, u0y)
    np.testing.assert_allclose(modes, d[tag + '_modes'], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize('kw', [dict(), dict(flip_lr=True), dict(flip_=True), dict(flip_lr=True, flip_=True),
                                dict(sign=-1), dict(mr=dict(shiftX=0.1, radialScaling=0.05, tangentialScaling=-0.02))],
                         ids=['plain', 'flip_lr', 'flip', 'both_flips', 'sign', 'shift_scalings'])
def test_separable_factors_rebuild_the_modes(kw):
    """The drop-in DM's separable factors (gx, gy, cell map) reproduce its
    dense float64 Gaussian IFs, and a rotated or anamorphic grid is refused
    (host only)."""
    from oopao_gb300.deformable_mirror import DeformableMirror as DM
    from oopao_gb300.mis_registration import MisRegistration
    res, ns = 48, 8
    mr = MisRegistration(dict(dict.fromkeys(O.MISREG_FIELDS, 0.0), **kw.get('mr', {})))
    def host_dm(**attrs):
        # the DM's host methods on an instance built without a GPU
        d = object.__new__(DM)
        d._modes = None
        d._modes_t_dev = None
        for k, v in attrs.items():
            setattr(d, k, v)
        return d

    attrs = dict(resolution=res, nActAlongDiameter=ns, mechCoupling=0.35, misReg=mr, sign=kw.get('sign', 1),
                 flip_lr=kw.get('flip_lr', False), flip_=kw.get('flip_', False), floating_precision=64)
    u0x, u0y, _ = O.dm_actuator_pixels(res, 8.0, ns, 0.0, mr.__dict__)
    fake = host_dm(**attrs)
    fake.modes = DM._gaussian_modes(fake, u0x, u0y)
    fake32 = host_dm(**dict(attrs, floating_precision=32))
    fake32.modes = DM._gaussian_modes(fake32, u0x, u0y)
    assert fake32.modes.dtype == np.float32 and DM._separable_factors(fake32, u0x, u0y) is not None
    gx, gy, cells = DM._separable_factors(fake, u0x, u0y)
    ny, nx = gy.shape[0], gx.shape[0]
    assert (cells >= 0).sum() == len(u0x)
    coefs = np.random.default_rng(0).standard_normal(len(u0x))
    C = np.zeros(ny * nx)
    C[cells >= 0] = coefs[cells[cells >= 0]]
    opd = gy.astype(np.float64).T @ C.reshape(ny, nx) @ gx.astype(np.float64)
    dense = (fake.modes @ coefs).reshape(res, res)
    assert np.max(np.abs(opd - dense)) < 1e-6 * np.max(np.abs(dense))
    for bad in (dict(rotationAngle=2.0), dict(anamorphosisAngle=20.0)):
        mr2 = MisRegistration(dict(dict.fromkeys(O.MISREG_FIELDS, 0.0), **bad))
        fake.misReg = mr2
        ux, uy, _ = O.dm_actuator_pixels(res, 8.0, ns, 0.0, mr2.__dict__)
        fake.modes = DM._gaussian_modes(fake, ux, uy)
        assert DM._separable_factors(fake, ux, uy) is None
