"""The two-pass propagation for masks that factorise per axis, through the C
ABI: the reference geometry's four-face mask factorises and takes the two
passes; a rooftop mask or a random mask does not.  Two-pass frames, raw
data, weighted sums and tangents against the three-pass path of the same
plan (float32 round-off, <= 2e-6 relative L2) and against the float64
oracle (<= 1e-5)."""
import ctypes

import numpy as np
import pytest

from oracle import pwfs_oracle as O
from tests.test_gpu_cabi import make_plan, measure, oracle_raw

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_PATHS = 2e-6


@pytest.fixture(scope='module')
def lib():
    import torch
    from oopao_gb300 import _native as N
    torch.cuda.init()
    return N


def sensor(N, res, nsub, mod, k, **geom_kw):
    geom = O.pyramid_geometry(res, nsub, 2, **geom_kw)
    path, K = O.modulation_path(mod, k)
    tt = O.tt_buffers(path, geom)
    pupil = O.telescope_pupil(res)
    inten = O.source_intensity(pupil, O.n_photon('V0', 8), 1e-3, 8.0)
    h = make_plan(N, res, geom.N, geom.cam, geom.mask, path, amp=np.sqrt(inten / K))
    return h, geom, tt, inten, pupil


@pytest.mark.parametrize('res,nsub,mod,k', [(24, 4, 3, 12), (120, 20, 3, 48), (240, 40, 5, 96)])
def test_two_pass_matches_three_pass_and_oracle(lib, res, nsub, mod, k):
    N = lib
    h, geom, tt, inten, pupil = sensor(N, res, nsub, mod, k)
    try:
        assert N.call('oopao_pwfs_separable', h) == 1
        rng = np.random.default_rng(res + 1)
        phase = rng.standard_normal((3, res, res)) * pupil
        f2, r2 = measure(N, h, phase, geom.N, geom.cam)
        f2b, _ = measure(N, h, phase, geom.N, geom.cam, want_raw=False)
        N.call('oopao_pwfs_set_separable', h, 0)
        assert N.call('oopao_pwfs_separable', h) == 0
        f3, r3 = measure(N, h, phase, geom.N, geom.cam)
        assert O.rel_l2(r2, r3) < TOL_PATHS
        assert O.rel_l2(f2, f3) < TOL_PATHS
        assert O.rel_l2(f2b, f3) < TOL_PATHS
        if res <= 120:
            ref = oracle_raw(phase, inten, tt, geom)
            for b in range(3):
                assert O.rel_l2(r2[b], ref[b]) < TOL
                assert O.rel_l2(f2b[b], O.camera_frame(ref[b], geom)) < TOL
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


def test_weighted_sum(lib):
    N = lib
    h, geom, tt, inten, pupil = sensor(N, 120, 20, 3, 48)
    try:
        w = np.random.default_rng(2).uniform(0.2, 2.0, 48).astype(np.float32)
        N.call('oopao_pwfs_set_weights', h, w)
        phase = np.random.default_rng(3).standard_normal((2, 120, 120)) * pupil
        f2, _ = measure(N, h, phase, geom.N, geom.cam, want_raw=False)
        N.call('oopao_pwfs_set_separable', h, 0)
        f3, _ = measure(N, h, phase, geom.N, geom.cam, want_raw=False)
        assert O.rel_l2(f2, f3) < TOL_PATHS
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


@pytest.mark.parametrize('kw', [dict(rooftop=0.5), dict(theta_rotation=0.3), dict(sx=(0.5, 0, 0, 0))])
def test_non_factorising_masks_take_three_passes(lib, kw):
    N = lib
    h, geom, tt, inten, pupil = sensor(N, 24, 4, 3, 12, **kw)
    try:
        assert N.call('oopao_pwfs_separable', h) == 0
        phase = np.random.default_rng(4).standard_normal((1, 24, 24)) * pupil
        _, raw = measure(N, h, phase, geom.N, geom.cam)
        assert O.rel_l2(raw[0], oracle_raw(phase, inten, tt, geom)[0]) < TOL
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


def jvp(N, h, opd0, dopd, cam):
    import torch
    B = dopd.shape[0]
    x0 = torch.as_tensor(np.ascontiguousarray(opd0, dtype=np.float32), device='cuda')
    dx = torch.as_tensor(np.ascontiguousarray(dopd, dtype=np.float32), device='cuda')
    out = torch.empty((B, cam, cam), device='cuda')
    nb = N.load().oopao_pwfs_ad_workspace_bytes(h, B)
    ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
    N.call('oopao_pwfs_jvp', h, N.ptr(x0), 1, N.ptr(dx), 1.0, B, N.ptr(out), N.ptr(ws), nb, N.stream_handle())
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


@pytest.mark.parametrize('res,nsub,mod,k', [(24, 4, 3, 12), (120, 20, 3, 48)])
def test_two_pass_tangent(lib, res, nsub, mod, k):
    """Two-pass JVP against the three-pass JVP and a float64 central
    difference of the oracle's camera frame."""
    N = lib
    h, geom, tt, inten, pupil = sensor(N, res, nsub, mod, k)
    try:
        rng = np.random.default_rng(7)
        opd0 = rng.standard_normal((1, res, res)) * pupil
        dopd = rng.standard_normal((3, res, res)) * pupil
        d2 = jvp(N, h, opd0, dopd, geom.cam)
        N.call('oopao_pwfs_set_separable', h, 0)
        d3 = jvp(N, h, opd0, dopd, geom.cam)
        assert O.rel_l2(d2, d3) < 1e-5
        eps = 1e-4
        for b in range(2):
            fp = O.camera_frame(oracle_raw(opd0 + eps * dopd[b:b + 1], inten, tt, geom)[0], geom)
            fm = O.camera_frame(oracle_raw(opd0 - eps * dopd[b:b + 1], inten, tt, geom)[0], geom)
            assert O.rel_l2(d2[b], (fp - fm) / (2 * eps)) < 1e-4
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


def vjp(N, h, opd, fbar):
    import torch
    B = opd.shape[0]
    x = torch.as_tensor(np.ascontiguousarray(opd, dtype=np.float32), device='cuda')
    fb = torch.as_tensor(np.ascontiguousarray(fbar, dtype=np.float32), device='cuda')
    out = torch.empty_like(x)
    nb = N.load().oopao_pwfs_ad_workspace_bytes(h, B)
    ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
    N.call('oopao_pwfs_vjp', h, N.ptr(x), N.ptr(fb), 1.0, B, N.ptr(out), N.ptr(ws), nb, N.stream_handle())
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


@pytest.mark.parametrize('res,nsub,mod,k', [(24, 4, 3, 12), (120, 20, 3, 48), (240, 40, 5, 96)])
def test_two_pass_adjoint(lib, res, nsub, mod, k):
    """Two-pass VJP against the three-pass VJP, and the dot-product identity
    <J dphi, fbar> = <dphi, J^T fbar> with the two-pass JVP (per item)."""
    N = lib
    h, geom, tt, inten, pupil = sensor(N, res, nsub, mod, k)
    try:
        rng = np.random.default_rng(11)
        opd = rng.standard_normal((2, res, res)) * pupil
        fbar = rng.standard_normal((2, geom.cam, geom.cam))
        a2 = vjp(N, h, opd, fbar)
        dphi = rng.standard_normal((1, res, res)) * pupil
        jv = jvp(N, h, opd[:1], dphi, geom.cam)
        lhs = float((jv[0] * fbar[0]).sum())
        rhs = float((dphi[0] * a2[0]).sum())
        assert abs(lhs - rhs) / abs(lhs) < 1e-4
        N.call('oopao_pwfs_set_separable', h, 0)
        a3 = vjp(N, h, opd, fbar)
        assert O.rel_l2(a2, a3) < 1e-5
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


@pytest.mark.parametrize('res,nsub,mod,k', [(120, 20, 3, 48), (240, 40, 5, 96)])
def test_every_two_pass_plan(lib, res, nsub, mod, k):
    """Every compile-time two-pass plan of the size (radix orders, columns per
    CTA, shared or separate exchange buffers) and a spread of slot counts give
    the three-pass frames."""
    N = lib
    h, geom, tt, inten, pupil = sensor(N, res, nsub, mod, k)
    try:
        phase = np.random.default_rng(13).standard_normal((2, res, res)) * pupil
        N.call('oopao_pwfs_set_separable', h, 0)
        f3, _ = measure(N, h, phase, geom.N, geom.cam, want_raw=False)
        for sp in range(1, N.call('oopao_pwfs_num_separable', h) + 1):
            N.call('oopao_pwfs_set_separable', h, sp)
            assert N.call('oopao_pwfs_separable', h) == 1
            for ks in (0, 1, 3, k // 2):
                N.call('oopao_pwfs_set_launch', h, 0, 0, 0, ks)
                f2, _ = measure(N, h, phase, geom.N, geom.cam, want_raw=False)
                assert O.rel_l2(f2, f3) < TOL_PATHS, (sp, ks)
            N.call('oopao_pwfs_set_launch', h, 0, 0, 0, 0)
    finally:
        N.load().oopao_pwfs_plan_destroy(h)
