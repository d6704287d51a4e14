"""Pin the CPU oracle on the Pyramid / Bi-O Edge options against golden
vectors made by the unmodified reference (case options_tiny: 24 px, 4x4
sensor): old_mask (both centrings), apply_shift_wfs (pixels and metres, both
masks), user_modulation_path, delta_theta with extraModulationFactor,
userValidSignal (slopes maps and full frame), the modulation / lightRatio /
delta_Tip / delta_Tilt setters and weight_vector.

Each case is replayed with oracle pieces in the order the reference's
constructor and setters run them: valid pixels from the calibration-
modulation frame, reference slopes re-measured by every call that
recalibrates, and weights applied to single-wavefront measurements only.
float64 on both sides: agreement at round-off (1e-10 relative bound).
"""
import json
import os

import numpy as np
import pytest

from oracle import bioedge_oracle as BO
from oracle import pwfs_oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
TOL = 1e-10
DIAMETER = 8.0


@pytest.fixture(scope='module')
def golden():
    z = np.load(os.path.join(HERE, 'options_tiny.npz'))
    d = {k: z[k] for k in z.files}
    d['params'] = json.loads(str(d['params']))
    return d


def _cases():
    with np.load(os.path.join(HERE, 'options_tiny.npz')) as z:
        return [tuple(c) for c in json.loads(str(z['params']))['cases']]


class _Replay:
    """One sensor of a case, rebuilt from oracle functions."""

    def __init__(self, d, sensor, kw):
        p = d['params']
        self.res, self.ns = p['res'], p['n_subap']
        self.sensor = sensor
        self.mod = kw.get('modulation', p['modulation'])
        self.lr = p['light_ratio']
        self.kw = kw
        self.pupil = O.telescope_pupil(self.res)
        self.inten = O.source_intensity(self.pupil, O.n_photon('V0', 8), 1e-3, DIAMETER)
        self.wavelength = O.PHOTOMETRY['V0'][0]
        self.extra = kw.get('extraModulationFactor', 0)
        self.delta_theta = kw.get('delta_theta', 0.0)
        self.user_path = kw.get('user_modulation_path')
        self.old = kw.get('old_mask', False)
        self.centred = kw.get('psfCentering', True)
        self.full_frame = kw.get('postProcessing', 'slopesMaps')[:9] == 'fullFrame'
        self.tip = self.tilt = 0.0
        self.weights = None
        flat = np.zeros((self.res, self.res))
        if sensor == 'pyramid':
            uv = kw.get('userValidSignal')
            self.user_valid = None if uv is None else d['user_valid_of'][0]
            self.geom = O.pyramid_geometry(self.res, self.ns, psf_centering=self.centred, old_mask=self.old)
            cal = min(50., self.res / 2 - 1)
            cpath, _ = O.modulation_path(cal, None, self.extra, self.delta_theta, user_path=self.user_path)
            self.init_frame = self._frame(flat, O.tt_buffers(cpath, self.geom))
            if self.user_valid is not None:
                self.valid = np.asarray(self.user_valid, dtype=bool)
            elif self.full_frame:
                self.valid = self.init_frame >= self.lr * self.init_frame.max()
            else:
                self.valid, _ = O.valid_pixels(self.init_frame, self.geom, self.lr)
        else:
            self.b = BO.build_bioedge(self.res, self.ns, self.mod, self.lr, self.inten, extra=self.extra,
                                      delta_theta=self.delta_theta)
            self.geom = self.b.geom
        self._set_path()

    # -- reference behaviour --------------------------------------------------
    def _set_path(self):
        self.path, self.n_theta = O.modulation_path(self.mod, None, self.extra, self.delta_theta, self.tip,
                                                    self.tilt, user_path=self.user_path)
        self.tt = O.tt_buffers(self.path, self.geom)
        self._calibrate()

    def _frame(self, phase, tt, weights=None):
        raw = O.wfs_raw(phase, self.inten, tt, self.geom, weight_vector=weights)
        return O.camera_frame(raw, self.geom)

    def _signals(self, frame, ref):
        if self.sensor == 'bioedge':
            return self.b.slopes(frame, reference_2d=ref)
        if self.full_frame:
            s2d, s, _ = O.full_frame(frame, self.valid, ref)
            return s2d, s
        s2d, s, _ = O.slopes_maps(frame, self.geom, self.valid, ref)
        return s2d, s

    def _calibrate(self):
        flat = np.zeros((self.res, self.res))
        if self.sensor == 'bioedge':
            self.b.tt, self.b.n_theta = self.tt, self.n_theta
            self.ref2d, _ = self.b.slopes(self.b.frame(flat), reference_2d=0.0)
            self.b.reference_2d = self.ref2d
            return
        self.ref2d, _ = self._signals(self._frame(flat, self.tt, self.weights), 0.0)

    def apply_shift_wfs(self, sx=0, sy=0, units='pixels'):
        f = 2 if (self.old or self.sensor == 'bioedge') else 1
        factor = f if units == 'pixels' else f / (DIAMETER / self.ns)
        sx4 = [sx] * 4 if np.isscalar(sx) else list(sx)
        sy4 = [sy] * 4 if np.isscalar(sy) else list(sy)
        if self.sensor == 'bioedge':
            self.b.masks = BO.bioedge_masks(self.res, self.ns, sx=sx4, sy=sy4)
        else:
            self.geom = O.pyramid_geometry(self.res, self.ns, psf_centering=self.centred, old_mask=self.old,
                                           sx=[factor * v for v in sx4], sy=[factor * v for v in sy4])
        self._calibrate()

    def set(self, name, val):
        if name == 'modulation':
            self.mod = val
            self._set_path()
        elif name == 'lightRatio':
            self.valid, _ = O.valid_pixels(self.init_frame, self.geom, val)
        elif name == 'delta_Tip':
            self.tip = val
            self._set_path()
        elif name == 'delta_Tilt':
            self.tilt = val
            self._set_path()
        elif name == 'weight_vector':
            assert val == 'ramp'
            self.weights = np.linspace(0.5, 1.5, self.n_theta)
        else:
            raise AssertionError(name)

    def measure(self, phase, single=True):
        if self.sensor == 'bioedge':
            f = self.b.frame(phase)
        else:
            f = self._frame(phase, self.tt, self.weights if single else None)
        s2d, s = self._signals(f, self.ref2d)
        return f, s2d, s


@pytest.mark.parametrize('case', _cases(), ids=lambda c: c[0])
def test_option_case(golden, case):
    name, sensor, kw, calls = case
    d = dict(golden)
    if name + '_user_valid' in d:
        d['user_valid_of'] = [d[name + '_user_valid']]
    r = _Replay(d, sensor, kw)
    for kind, attr, val in calls:
        if kind == 'call':
            getattr(r, attr)(**val)
        else:
            r.set(attr, val)
    assert r.n_theta == int(d[name + '_n_theta'])
    if name + '_modulation_path' in d:
        np.testing.assert_allclose(r.path, d[name + '_modulation_path'], rtol=0, atol=1e-13)
    n_signal = int(r.valid.sum()) if sensor == 'pyramid' and r.full_frame else \
        2 * int((r.valid if sensor == 'pyramid' else r.b.valid_i4q).sum())
    assert n_signal == int(d[name + '_n_signal'])
    modes = O.dm_modes(r.res, DIAMETER, r.ns, 0.35)
    to_phase = 2 * np.pi / r.wavelength
    phase = O.dm_opd(modes, d['coefs'], r.res) * r.pupil * to_phase
    f, s2d, s = r.measure(phase)
    ref = d[name + '_reference_2D']
    assert np.linalg.norm(r.ref2d - ref) / max(np.linalg.norm(ref), 1e-6 * np.sqrt(ref.size)) < TOL
    assert O.rel_l2(f, d[name + '_frame']) < TOL
    assert O.rel_l2(s2d, d[name + '_signal_2D']) < TOL
    assert O.rel_l2(s, d[name + '_signal']) < TOL
    # two DM shapes at once: the reference's 3-D path (unweighted sum)
    cube = O.dm_opd(modes, d['coefs2'], r.res) * r.pupil[..., None] * to_phase
    sig = np.stack([r.measure(cube[..., b], single=False)[2] for b in range(cube.shape[2])], axis=-1)
    assert O.rel_l2(sig, d[name + '_batch_signal']) < TOL


def test_old_mask_against_quadrant_definition():
    """The old mask is piecewise planar: inside each quadrant the phase
    differences along x and y are constant (no golden needed)."""
    m = O.phase_mask_old(24, 4, 2, 1, True)
    n = m.shape[0]
    h = n // 2
    for rows, cols in ((slice(0, h), slice(0, h)), (slice(0, h), slice(h, n)), (slice(h, n), slice(h, n)),
                       (slice(h, n), slice(0, h))):
        q = m[rows, cols]
        assert np.ptp(np.diff(q, axis=1)) < 1e-12
        assert np.ptp(np.diff(q, axis=0)) < 1e-12


@pytest.mark.parametrize('old', [False, True], ids=['faces', 'old_quadrants'])
@pytest.mark.parametrize('centred', [True, False], ids=['4px', '1px'])
def test_drop_in_mask_functions_match_the_oracle(old, centred):
    """The drop-in Pyramid's host mask builders (get_phase_mask,
    get_phase_mask_old) against the pinned oracle, with face shifts, rooftop
    and rotation (no GPU needed)."""
    import types
    from oopao_gb300.pyramid import Pyramid
    res, ns, sep, edge = 24, 4, 2, 1
    sx, sy = [1.0, -0.5, 0.25, 0.0], [0.0, 0.5, -1.0, 0.75]
    fake = types.SimpleNamespace(telescope=types.SimpleNamespace(resolution=res), nSubap=ns, psfCentering=centred,
                                 rooftop=0.0 if old else 0.4, theta_rotation=0.0 if old else 0.05,
                                 n_pix_separation=sep)
    n = int((ns * 2 + sep + edge * 2) * res / ns)
    if old:
        got = Pyramid.get_phase_mask_old(fake, n, ns, sep, edge, psf_centering=centred, sx=sx, sy=sy)
        want = O.phase_mask_old(res, ns, sep, edge, centred, sx, sy)
    else:
        got = Pyramid.get_phase_mask(fake, n, ns, sep, edge, psf_centering=centred, sx=sx, sy=sy)
        want = O.phase_mask(res, ns, sep, edge, centred, fake.rooftop, fake.theta_rotation, sx, sy)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)


@pytest.mark.parametrize('kw', [dict(modulation=3), dict(modulation=2, nTheta_user_defined=12),
                                dict(modulation=3, delta_theta=0.3, extraModulationFactor=1),
                                dict(modulation=3, delta_Tip=0.5, delta_Tilt=-0.25),
                                dict(modulation=0, user_modulation_path=[[1, 0], [0, 1], [-1, 0.5]]),
                                dict(modulation=0)],
                         ids=['default', 'user_ntheta', 'delta_extra', 'tip_tilt', 'user_path', 'no_modulation'])
def test_drop_in_modulation_path_matches_the_oracle(kw):
    """The drop-in Pyramid's modulation setter (host logic, no GPU) against
    the pinned oracle's modulation_path."""
    import types
    from oopao_gb300.pyramid import Pyramid
    p = object.__new__(Pyramid)
    p.telescope = types.SimpleNamespace(resolution=24)
    p.user_modulation_path = kw.get('user_modulation_path')
    p.modulation_length = 2 * np.pi
    p.nTheta_user_defined = kw.get('nTheta_user_defined')
    p.extraModulationFactor = kw.get('extraModulationFactor', 0)
    p.delta_theta = kw.get('delta_theta', 0.0)
    p._delta_Tip = kw.get('delta_Tip', 0.0)
    p._delta_Tilt = kw.get('delta_Tilt', 0.0)
    p.isCalibrated = False
    p._plan = None
    p.modulation = kw['modulation']
    want, n_theta = O.modulation_path(kw['modulation'], kw.get('nTheta_user_defined'), p.extraModulationFactor,
                                      p.delta_theta, p._delta_Tip, p._delta_Tilt, user_path=p.user_modulation_path)
    assert p.nTheta == n_theta
    if want is None:
        assert p.modulation_path is None
    else:
        np.testing.assert_allclose(np.asarray(p.modulation_path, dtype=np.float64), want, rtol=0, atol=1e-14)
