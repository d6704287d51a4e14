"""Bi-O Edge drop-in against golden vectors made by the unmodified reference:
geometry, valid pixels, reference slopes, a DM measurement through
``ngs**tel*dm*wfs``, a screen through ``wfs_measure`` and push-pull IM
columns, the focal-plane camera.  FP32 path bounds: 1e-5 (frames, signals,
focal-plane frames), 1e-4 (IM columns)."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


@pytest.fixture(scope='module', params=['bioedge_tiny', 'bioedge_grey'])
def system(request):
    import oopao_gb300 as og
    z = np.load(os.path.join(HERE, request.param + '.npz'))
    d = {k: z[k] for k in z.files}
    p = json.loads(str(d['params']))
    kw = {k: v for k, v in p.items() if k not in ('res', 'n_subap', 'modulation', 'light_ratio')}
    with _quiet():
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = og.BioEdge(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'], lightRatio=p['light_ratio'],
                         **kw)
    return d, tel, ngs, dm, wfs


def test_geometry_and_calibration(system):
    d, tel, ngs, dm, wfs = system
    assert wfs.resolution == int(d['N']) and wfs.cam.resolution == int(d['cam'])
    assert wfs.nTheta == int(d['n_theta'])
    for m, g in zip(wfs.mask, d['masks']):
        np.testing.assert_allclose(m, g, rtol=0, atol=1e-14)
    np.testing.assert_array_equal(wfs.validI4Q, d['valid_i4q'])
    assert wfs.nSignal == int(d['n_signal'])
    assert O.rel_l2(wfs.referenceSignal_2D, d['reference_2d']) < 1e-5


def test_dm_measurement(system):
    d, tel, ngs, dm, wfs = system
    dm.coefs = d['dm_coefs']
    ngs ** tel * dm * wfs
    assert O.rel_l2(wfs.raw_data, d['dm_raw']) < 1e-5
    assert O.rel_l2(wfs.cam.frame, d['dm_frame']) < 1e-5
    assert O.rel_l2(wfs.signal_2D, d['dm_signal_2D']) < 1e-5
    assert O.rel_l2(wfs.signal, d['dm_signal']) < 1e-5


def test_focal_plane_camera(system):
    """wfs * wfs.focal_plane_camera after the DM measurement: the reference's
    sum over its list of four fields per modulation point, cropped to the
    camera; the zoom of get_modulation_frame follows it."""
    d, tel, ngs, dm, wfs = system
    dm.coefs = d['dm_coefs']
    ngs ** tel * dm * wfs
    with _quiet():
        wfs * wfs.focal_plane_camera
    assert O.rel_l2(wfs.focal_plane_camera.frame, d['dm_focal_cam']) < 1e-5
    # radius 8 lambda/D: a crop inside both cases' camera frames (72 of N=72, 80 of N=128)
    n_trunc = int(wfs.resolution / 2 - 8 * wfs.zeroPaddingFactor)
    ref = d['dm_focal_cam'][n_trunc:-n_trunc, n_trunc:-n_trunc]
    assert ref.size > 0
    assert O.rel_l2(wfs.get_modulation_frame(radius=8), ref / ref.max()) < 1e-5


def test_screen_measurement(system):
    d, tel, ngs, dm, wfs = system
    dm.coefs = 0
    ngs ** tel
    wfs.wfs_measure(phase_in=d['screen_phase'])
    assert O.rel_l2(wfs.cam.frame, d['screen_frame']) < 1e-5
    assert O.rel_l2(wfs.signal, d['screen_signal']) < 1e-5


def test_interaction_matrix(system):
    import oopao_gb300 as og
    d, tel, ngs, dm, wfs = system
    with _quiet():
        calib = og.InteractionMatrix(ngs, tel, dm, wfs, d['im_m2c'], 1e-8, single_pass=False, invert=False)
    assert O.rel_l2(np.asarray(calib.D), d['im_pp_D']) < 1e-4


def test_shared_forward_matches_per_mask_plans(system):
    """One plan with the four masks (forward transforms shared) gives the
    frames of four single-mask plans.  bioedge_tiny (N = 72) takes the
    shared path; bioedge_grey (N = 128, two stage-B butterflies per thread)
    keeps one plan per mask; both are checked against the goldens above."""
    import torch
    from oopao_gb300 import _native as N
    from oopao_gb300.pyramid import _Plan
    d, tel, ngs, dm, wfs = system
    plans = wfs.plans
    assert wfs._shared_forward == (wfs.resolution == 72)
    rng = np.random.default_rng(9)
    opd = torch.as_tensor(rng.standard_normal((3, tel.resolution, tel.resolution)) * 50e-9, dtype=torch.float32,
                          device='cuda')
    scale = 2 * np.pi / ngs.wavelength
    ngs ** tel
    frame, raw = wfs._measure_frames(opd, scale, want_raw=True)
    cam, n = wfs._cam_eff, wfs.resolution
    half = 0.5 * np.asarray(ngs.intensity, dtype=np.float64)
    for q, m in enumerate(wfs.mask):
        p = _Plan(tel.resolution, n, cam, m, wfs.modulation_path, 1.0, True)
        p.set_amplitude(half, None)
        nb = p.workspace_bytes(3)
        ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
        tile = torch.empty((3, cam, cam), device='cuda')
        rt = torch.empty((3, n, n), device='cuda')
        N.call('oopao_pwfs_measure', p.h, N.ptr(opd), float(scale), 3, N.ptr(tile), N.ptr(rt), N.ptr(ws), nb,
               N.stream_handle())
        i, j = divmod(q, 2)
        ft = frame[:, i * cam:(i + 1) * cam, j * cam:(j + 1) * cam].double().cpu().numpy()
        rr = raw[:, i * n:(i + 1) * n, j * n:(j + 1) * n].double().cpu().numpy()
        assert O.rel_l2(ft, tile.double().cpu().numpy()) < 1e-6, q
        assert O.rel_l2(rr, rt.double().cpu().numpy()) < 1e-6, q


def test_one_axis_path_matches_three_passes(system):
    """The Bi-O Edge masks vary along one focal-plane axis each, so their plans
    take the one-axis path (filtered lines of that axis, |line|^2 summed over
    the points that share the other axis' phasor, no column transform):
    frames and raw data equal those of the three-pass path to float32
    round-off, for a batch with and without per-point weights."""
    import torch
    from oopao_gb300 import _native as N
    d, tel, ngs, dm, wfs = system
    plans = wfs.plans
    assert all(N.call('oopao_pwfs_separable', p.h) == 2 for p in plans)
    rng = np.random.default_rng(12)
    opd = torch.as_tensor(rng.standard_normal((3, tel.resolution, tel.resolution)) * 50e-9, dtype=torch.float32,
                          device='cuda')
    scale = 2 * np.pi / ngs.wavelength
    ngs ** tel
    for weights in (None, rng.uniform(0.5, 1.5, wfs.nTheta)):
        # weights apply to a single wavefront (a 2-D OPD), as in the reference
        wfs._weight_vector = weights
        o = opd[0] if weights is not None else opd
        f1, r1 = wfs._measure_frames(o, scale, want_raw=True)
        f1b, _ = wfs._measure_frames(o, scale, want_raw=False)
        for p in plans:
            N.call('oopao_pwfs_set_separable', p.h, 0)
        try:
            f3, r3 = wfs._measure_frames(o, scale, want_raw=True)
        finally:
            for p in plans:
                N.call('oopao_pwfs_set_separable', p.h, 1)
        assert O.rel_l2(f1.double().cpu().numpy(), f3.double().cpu().numpy()) < 2e-6
        assert O.rel_l2(f1b.double().cpu().numpy(), f3.double().cpu().numpy()) < 2e-6
        assert O.rel_l2(r1.double().cpu().numpy(), r3.double().cpu().numpy()) < 2e-6
    wfs._weight_vector = None
