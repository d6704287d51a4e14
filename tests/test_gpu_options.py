"""Constructor options and post-construction calls of the drop-in Pyramid and
BioEdge against golden vectors made by the unmodified reference (case
options_tiny: 24 px, 4x4 sensor): old_mask, apply_shift_wfs, user
modulation paths, delta_theta / extraModulationFactor, userValidSignal, the
modulation / lightRatio / delta_Tip / delta_Tilt setters and weight_vector,
each with one DM shape and a batch of two.  FP32 path bound: relative L2 <=
1e-5."""
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
    z = np.load(os.path.join(HERE, 'options_tiny.npz'))
    d = {k: z[k] for k in z.files}
    d['params'] = json.loads(str(d['params']))
    return d


def _cases():
    with np.load(os.path.join(HERE, 'options_tiny.npz')) as z:
        return [tuple(c) for c in json.loads(str(z['params']))['cases']]


def _build(d, name, sensor, kw):
    import oopao_gb300 as og
    p = d['params']
    kw = dict(kw)
    modulation = kw.pop('modulation', p['modulation'])
    if 'userValidSignal' in kw:
        kw['userValidSignal'] = d[name + '_user_valid']
    cls = og.Pyramid if sensor == 'pyramid' else og.BioEdge
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = cls(nSubap=p['n_subap'], telescope=tel, modulation=modulation, lightRatio=p['light_ratio'], **kw)
    return tel, ngs, dm, wfs


@pytest.mark.parametrize('case', _cases(), ids=lambda c: c[0])
def test_option_case(golden, case):
    name, sensor, kw, calls = case
    d = golden
    tel, ngs, dm, wfs = _build(d, name, sensor, kw)
    with contextlib.redirect_stdout(io.StringIO()):
        for kind, attr, val in calls:
            if kind == 'call':
                getattr(wfs, attr)(**val)
            elif val == 'ramp':
                setattr(wfs, attr, np.linspace(0.5, 1.5, wfs.nTheta))
            else:
                setattr(wfs, attr, val)
    assert wfs.nTheta == int(d[name + '_n_theta'])
    assert int(wfs.nSignal) == int(d[name + '_n_signal'])
    if name + '_modulation_path' in d:
        np.testing.assert_allclose(np.asarray(wfs.modulation_path, dtype=np.float64), d[name + '_modulation_path'],
                                   rtol=0, atol=1e-12)
    ref = d[name + '_reference_2D']
    # a symmetric sensor has reference slopes of pure round-off (old mask
    # centred on one pixel: 3e-15): measure the error against the slope
    # scale of the aberrated measurement
    scale = max(np.linalg.norm(ref), np.linalg.norm(d[name + '_signal_2D']))
    err = np.linalg.norm(np.asarray(wfs.referenceSignal_2D) - ref) / scale
    assert err < TOL, err
    dm.coefs = d['coefs']
    ngs ** tel * dm * wfs
    assert O.rel_l2(wfs.cam.frame, d[name + '_frame']) < TOL
    assert O.rel_l2(wfs.signal_2D, d[name + '_signal_2D']) < TOL
    assert O.rel_l2(wfs.signal, d[name + '_signal']) < TOL
    # a batch of two DM shapes: the reference's 3-D phase path (unweighted)
    dm.coefs = d['coefs2']
    ngs ** tel * dm * wfs
    assert O.rel_l2(wfs.signal, d[name + '_batch_signal']) < TOL
    # the camera keeps the batch's last frame, as the reference's per-mode integration does
    frames = wfs.cam.device_frame
    assert frames.shape[0] == 2 and np.asarray(wfs.cam.frame).shape == frames.shape[1:]
    assert O.rel_l2(wfs.cam.frame, frames[-1].double().cpu().numpy()) == 0


def test_weights_switch_between_single_and_batch(golden):
    """A weighted sensor alternates weighted single measurements with
    unweighted batches; the plan follows each call."""
    d = golden
    tel, ngs, dm, wfs = _build(d, 'weights', 'pyramid', {})
    with contextlib.redirect_stdout(io.StringIO()):
        wfs.weight_vector = np.linspace(0.5, 1.5, wfs.nTheta)
    for _ in range(2):
        dm.coefs = d['coefs']
        ngs ** tel * dm * wfs
        assert O.rel_l2(wfs.signal, d['weights_signal']) < TOL
        dm.coefs = d['coefs2']
        ngs ** tel * dm * wfs
        assert O.rel_l2(wfs.signal, d['weights_batch_signal']) < TOL
    wfs.weight_vector = np.ones(wfs.nTheta + 1)
    dm.coefs = d['coefs']
    import oopao_gb300 as og
    with pytest.raises(og.OopaoError):
        ngs ** tel * dm * wfs


def test_mask_assignment_takes_effect(golden):
    """Assigning wfs.mask (as GSC studies do) changes the next measurement."""
    d = golden
    tel, ngs, dm, wfs = _build(d, 'shift', 'pyramid', {})
    dm.coefs = d['coefs']
    ngs ** tel * dm * wfs
    f0 = np.array(wfs.cam.frame)
    m = np.array(wfs.mask)
    wfs.mask = np.conj(m)
    ngs ** tel * dm * wfs
    assert O.rel_l2(wfs.cam.frame, f0) > 1e-3
    wfs.mask = m
    ngs ** tel * dm * wfs
    assert O.rel_l2(wfs.cam.frame, f0) < 1e-6
