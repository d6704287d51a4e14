"""GPU parity through the C ABI itself (ctypes on include/oopao_gb300.h):
propagation + binning against the float64 oracle, both kernel variants at
every compile-time FFT size, signal processing and the DM projection.

Tolerances: FP32 path, relative L2 <= 1e-5 against float64."""
import ctypes

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope='module')
def lib():
    import torch
    from oopao_gb300 import _native as N
    torch.cuda.init()
    return N


def make_plan(N, res, n, cam, mask, path, psf_centering=True, amp=None):
    h = ctypes.c_void_p()
    m = np.ascontiguousarray(mask, dtype=np.complex64)
    p = None if path is None else np.ascontiguousarray(path, dtype=np.float64)
    N.call('oopao_pwfs_plan_create', ctypes.byref(h), res, n, cam, 1 if path is None else len(path),
           m, p, 1.0, int(psf_centering))
    if amp is not None:
        a = np.ascontiguousarray(amp, dtype=np.float32)
        N.call('oopao_pwfs_set_amplitude', h, a)
    return h


def measure(N, h, opd, n, cam, scale=1.0, want_raw=True):
    import torch
    B = opd.shape[0]
    x = torch.as_tensor(np.ascontiguousarray(opd, dtype=np.float32), device='cuda')
    frame = torch.empty((B, cam, cam), device='cuda')
    raw = torch.empty((B, n, n), device='cuda') if want_raw else None
    nb = N.load().oopao_pwfs_workspace_bytes(h, B)
    ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
    N.call('oopao_pwfs_measure', h, N.ptr(x), scale, B, N.ptr(frame), N.ptr(raw), N.ptr(ws), nb,
           N.stream_handle())
    torch.cuda.synchronize()
    return frame.double().cpu().numpy(), None if raw is None else raw.double().cpu().numpy()


def oracle_raw(phase, inten, tt, geom):
    return O.wfs_raw(np.moveaxis(phase, 0, -1), inten, tt, geom)


@pytest.mark.parametrize('res,nsub,sep,mod,k', [(24, 4, 2, 3, 12), (120, 20, 2, 3, 48), (40, 10, 4, 2, 8)])
def test_measure_matches_oracle(lib, res, nsub, sep, mod, k):
    N = lib
    geom = O.pyramid_geometry(res, nsub, sep)
    path, K = O.modulation_path(mod, k)
    tt = O.tt_buffers(path, geom)
    pupil = O.telescope_pupil(res)
    inten = O.source_intensity(pupil, O.n_photon('V0', 8), 1e-3, 8.0)
    amp = np.sqrt(inten / K)
    rng = np.random.default_rng(res)
    phase = rng.standard_normal((3, res, res)) * pupil
    h = make_plan(N, res, geom.N, geom.cam, geom.mask, path, amp=amp)
    try:
        frame, raw = measure(N, h, phase, geom.N, geom.cam)
        ref = oracle_raw(phase, inten, tt, geom)
        for b in range(3):
            assert O.rel_l2(raw[b], ref[b]) < TOL
            assert O.rel_l2(frame[b], O.camera_frame(ref[b], geom)) < TOL
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


@pytest.mark.parametrize('n,res,cam', [(72, 24, 12), (96, 32, 16), (112, 40, 28), (128, 32, 16),
                                       (240, 120, 40), (264, 120, 44), (480, 240, 80), (504, 240, 84),
                                       (1920, 480, 320)])
def test_variants_agree(lib, n, res, cam):
    """Compile-time two-stage passes == generic runtime-planned passes."""
    N = lib
    rng = np.random.default_rng(n)
    mask = np.exp(1j * rng.uniform(-np.pi, np.pi, (n, n))).astype(np.complex64)
    path = rng.uniform(-3, 3, (6, 2))
    amp = rng.uniform(0.5, 1.5, (res, res))
    h = make_plan(N, res, n, cam, mask, path, amp=amp)
    try:
        nv = N.load().oopao_pwfs_num_variants(h)
        assert nv >= 1
        assert 1 <= N.load().oopao_pwfs_get_variant(h) <= nv    # starts on a compiled plan
        phase = rng.standard_normal((2, res, res))
        N.call('oopao_pwfs_set_variant', h, 0)
        f0, r0 = measure(N, h, phase, n, cam)
        f0b, _ = measure(N, h, phase, n, cam, want_raw=False)
        for v in range(1, nv + 1):
            N.call('oopao_pwfs_set_variant', h, v)
            f1, r1 = measure(N, h, phase, n, cam)
            assert O.rel_l2(r1, r0) < 2e-6, v
            assert O.rel_l2(f1, f0) < 2e-6, v
            # binned path (no raw_data requested) agrees as well
            f1b, _ = measure(N, h, phase, n, cam, want_raw=False)
            assert O.rel_l2(f1b, f0b) < 2e-6, v
            # no bounded wait of the variant's kernels timed out
            code = np.ones(1, np.int32)
            N.call('oopao_pwfs_device_status', h, code)
            assert code[0] == 0, v
        assert N.load().oopao_pwfs_set_variant(h, nv + 1) == 2
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


def test_variant_against_float64_fft(lib):
    """The 504-point plan against a float64 numpy evaluation (no golden at this size)."""
    N = lib
    n, res, cam = 504, 240, 84
    rng = np.random.default_rng(3)
    mask = np.exp(1j * rng.uniform(-np.pi, np.pi, (n, n))).astype(np.complex64)
    path = rng.uniform(-5, 5, (4, 2))
    amp = rng.uniform(0.5, 1.5, (res, res))
    h = make_plan(N, res, n, cam, mask, path, amp=amp)
    try:
        phase = rng.standard_normal((1, res, res))
        _, raw = measure(N, h, phase, n, cam)
        geom = O.PyramidGeometry(res=res, n_subap=40, n_pix_separation=2, n_pix_edge=1, psf_centering=True,
                                 N=n, cam=cam, center=n // 2, mask=mask, phasor=None, tip=None, tilt=None)
        xx, yy = np.meshgrid(np.arange(n), np.arange(n))
        geom.phasor = np.exp(-(1j * np.pi * (n + 1) / n) * (xx + yy))
        t = np.linspace(-np.pi, np.pi, res)
        tip, tilt = np.meshgrid(t, t)
        tt = np.stack([px * tip + py * tilt for px, py in path])
        ref = O.wfs_raw(phase[0], amp ** 2 * len(path), tt, geom)
        assert O.rel_l2(raw[0], ref) < TOL
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


@pytest.mark.parametrize('mode', ['slopesMaps', 'fullFrame'])
def test_signal_processing(lib, mode):
    import torch
    N = lib
    geom = O.pyramid_geometry(120, 20, 2)
    h = make_plan(N, 120, geom.N, geom.cam, geom.mask, np.zeros((4, 2)))
    try:
        rng = np.random.default_rng(5)
        frames = rng.uniform(0.5, 2.0, (3, geom.cam, geom.cam))
        valid, _ = O.valid_pixels(frames[0], geom, 0.9)
        ref2d = rng.standard_normal((40, 20)) * 0.01
        nq = 20
        # grabQuadrant origins for cam 44, 20 subapertures, separation 2
        org = np.array([[1, 1], [1, 23], [23, 23], [23, 1]], dtype=np.int32).reshape(-1)
        for q in range(4):
            np.testing.assert_array_equal(
                O.grab_quadrant(frames[0], q + 1, geom),
                frames[0][org[2 * q]:org[2 * q] + nq, org[2 * q + 1]:org[2 * q + 1] + nq])
        if mode == 'slopesMaps':
            v8 = np.ascontiguousarray(valid, dtype=np.uint8)
            r32 = np.ascontiguousarray(ref2d, dtype=np.float32)
            N.call('oopao_pwfs_set_signal_processing', h, 0, nq, org, v8, r32, 1.0, 0.0)
            n2d = 2 * nq * nq
        else:
            vs = frames[0] >= 0.9 * frames[0].max()
            v8 = np.ascontiguousarray(vs, dtype=np.uint8)
            N.call('oopao_pwfs_set_signal_processing', h, 3, 0, None, v8, None, 1.0, 0.0)
            n2d = geom.cam ** 2
        ns = N.load().oopao_pwfs_n_signal(h)
        f = torch.as_tensor(frames.astype(np.float32), device='cuda')
        s2 = torch.empty((3, n2d), device='cuda')
        sg = torch.empty((3, ns), device='cuda')
        N.call('oopao_pwfs_signal', h, N.ptr(f), 3, N.ptr(s2), N.ptr(sg), None, N.stream_handle())
        torch.cuda.synchronize()
        for b in range(3):
            if mode == 'slopesMaps':
                m2, s, _ = O.slopes_maps(frames[b], geom, valid, ref2d)
            else:
                m2, s, _ = O.full_frame(frames[b], vs)
            assert O.rel_l2(s2[b].double().cpu().numpy().reshape(m2.shape), m2) < TOL
            assert O.rel_l2(sg[b].double().cpu().numpy(), s) < TOL
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


@pytest.mark.parametrize('batch', [1, 3, 8, 20, 300])
def test_dm_projection(lib, batch):
    import torch
    N = lib
    modes = O.dm_modes(120, 8.0, 20)
    rng = np.random.default_rng(batch)
    coefs = rng.standard_normal((modes.shape[1], batch))
    mt = torch.as_tensor(np.ascontiguousarray(modes.T, dtype=np.float32), device='cuda')
    c = torch.as_tensor(coefs.astype(np.float32), device='cuda')
    out = torch.empty((batch, 120 * 120), device='cuda')
    N.call('oopao_dm_opd_f32', N.ptr(mt), N.ptr(c), modes.shape[1], 120 * 120, batch, 2.0, N.ptr(out),
           N.stream_handle())
    torch.cuda.synchronize()
    ref = (modes @ coefs).T * 2.0
    assert O.rel_l2(out.double().cpu().numpy(), ref) < 1e-6


def test_invalid_arguments_are_rejected(lib):
    N = lib
    h = make_plan(N, 24, 72, 12, np.ones((72, 72), np.complex64), np.zeros((4, 2)))
    try:
        st = N.load().oopao_pwfs_measure(h, None, 1.0, 1, None, None, None, 0, None)
        assert st == 1
        assert N.load().oopao_pwfs_set_variant(h, -1) == 1
        assert N.load().oopao_pwfs_set_variant(h, 7) == 2
        # workspace smaller than one item
        import torch
        x = torch.zeros((1, 24, 24), device='cuda')
        fr = torch.empty((1, 12, 12), device='cuda')
        ws = torch.empty(16, dtype=torch.uint8, device='cuda')
        st = N.load().oopao_pwfs_measure(h, N.ptr(x), 1.0, 1, N.ptr(fr), None, N.ptr(ws), 16, None)
        assert st == 4
    finally:
        N.load().oopao_pwfs_plan_destroy(h)
