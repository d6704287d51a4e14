"""Infinite-phase-screen atmosphere on the GPU against the reference (golden
OPD sequences, frozen flow and boiling) and the float64 oracle; graph replay against eager updates;
a step outside the planned horizon sets the error flag and moves nothing."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from oracle import atm_oracle as A
from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'atm_small.npz')


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


def _build(res, r0, L0, frac, ws, wd, alt, diameter=8.0, t_boiling=None):
    import oopao_gb300 as og
    with _quiet():
        tel = og.Telescope(resolution=res, diameter=diameter, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        atm = og.Atmosphere(telescope=tel, r0=r0, L0=L0, fractionalR0=frac, windSpeed=ws, windDirection=wd,
                            altitude=alt, t_boiling=t_boiling)
        atm.initializeAtmosphere(tel)
    return tel, ngs, atm


def test_atmosphere_matches_reference_sequence():
    z = np.load(GOLDEN)
    p = json.loads(str(z['params']))
    tel, ngs, atm = _build(p['res'], p['r0'], p['L0'], p['fractionalR0'], p['windSpeed'], p['windDirection'],
                           p['altitude'], p['diameter'])
    A_dev = atm._A.cpu().numpy()
    assert np.abs(A_dev - z['A']).max() < 1e-8 * np.abs(z['A']).max()
    ref = z['opd']
    ngs ** atm * tel
    assert O.rel_l2(ngs.OPD_no_pupil, ref[0]) < 1e-6
    for t in range(p['steps']):
        atm.update()
        ngs ** atm * tel
        assert O.rel_l2(ngs.OPD_no_pupil, ref[t + 1]) < 1e-5, t
    assert atm.status() == 0


def test_boiling_matches_reference_sequence():
    """A still layer that boils, a fast diagonal one that boils and a slow one
    that does not, against the reference's own sequence."""
    z = np.load(os.path.join(os.path.dirname(GOLDEN), 'atm_boil.npz'))
    p = json.loads(str(z['params']))
    tel, ngs, atm = _build(p['res'], p['r0'], p['L0'], p['fractionalR0'], p['windSpeed'], p['windDirection'],
                           p['altitude'], p['diameter'], t_boiling=p['t_boiling'])
    ref = z['opd']
    ngs ** atm * tel
    assert O.rel_l2(ngs.OPD_no_pupil, ref[0]) < 1e-6
    for t in range(p['steps']):
        atm.update()
        ngs ** atm * tel
        assert O.rel_l2(ngs.OPD_no_pupil, ref[t + 1]) < 1e-5, t
    assert atm.status() == 0
    # back to the generated screens and the first seeds: the same sequence again
    atm.reset_state()
    for t in range(3):
        atm.update()
        assert O.rel_l2(atm.OPD, ref[t + 1]) < 1e-5, t


def test_atmosphere_matches_oracle_120px():
    args = dict(r0=0.15, L0=25.0, frac=[0.5, 0.3, 0.2], ws=[10.0, 15.0, 20.0], wd=[0.0, 72.0, 144.0],
                alt=[0.0, 5000.0, 10000.0])
    tel, ngs, atm = _build(120, **args)
    ora = A.OracleAtmosphere(120, 8.0, 1e-3, args['r0'], args['L0'], args['frac'], args['ws'], args['wd'],
                             args['alt'])
    assert O.rel_l2(atm.OPD, ora.opd) < 1e-6
    for t in range(100):
        atm.update()
        ora.update()
        if t % 10 == 9:
            assert O.rel_l2(atm.OPD, ora.opd) < 1e-5, t
    assert atm.status() == 0


@pytest.mark.parametrize('t_boiling', [None, [0.02, None]])
def test_graph_replay_equals_eager_and_horizon_guard(t_boiling):
    """Frozen flow, and a boiling layer whose screens the captured loop draws
    for its whole horizon up front."""
    import torch
    from oopao_gb300.closed_loop import ClosedLoop
    import oopao_gb300 as og
    tel, ngs, atm = _build(40, r0=0.3, L0=25.0, frac=[0.7, 0.3], ws=[30.0, 60.0], wd=[10.0, 200.0],
                           alt=[0.0, 8000.0], t_boiling=t_boiling)
    with _quiet():
        dm = og.DeformableMirror(tel, nSubap=10)
        wfs = og.Pyramid(nSubap=10, telescope=tel, modulation=2, lightRatio=0.5, n_pix_separation=4,
                         n_pix_edge=2, nTheta_user_defined=12)
    R = np.zeros((dm.nValidAct, wfs.nSignal))
    n = 25
    cl = ClosedLoop(tel, ngs, dm, wfs, R, gain=0.0, layers=atm, max_steps=n)
    cl.capture()
    cl.run(n)
    torch.cuda.synchronize()
    opd_graph = atm.OPD.copy()
    wfe_graph = cl.residual_wfe.copy()
    # step t of the loop sees the atmosphere after t + 1 updates, and each
    # step prepares the next one's: after n steps it has been updated n + 1 times
    atm.reset_state()
    for _ in range(n + 1):
        atm.update()
    np.testing.assert_array_equal(atm.OPD, opd_graph)
    assert atm.status() == 0
    # the residual of an open loop is the turbulence itself
    assert np.all(wfe_graph > 0)
    # beyond the planned horizon: flagged, nothing moves, no fault
    cl.run(4)
    torch.cuda.synchronize()
    assert atm.status() == 1
