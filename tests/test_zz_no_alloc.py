"""The allocation-free measurement entry point (oopao_pwfs_measure_noalloc).

Callers that cannot allocate device memory while they measure — a real-time
control loop that forbids allocation once running, or a host framework that
owns the GPU allocator — use this entry point: its scratch is a fixed 64 MiB
array inside the library.  These tests call it through the C ABI and compare
it with the workspace-taking oopao_pwfs_measure on the same inputs, for two
calls in a row (the shared scratch keeps the previous call's contents, which
must not leak into the next result).  The file sorts last so that a run that
stops at the first failure has run every other test first; it also passes
alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5  # same FP32 tolerance as the other parity tests


@pytest.fixture(scope='module')
def native():
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from oopao_gb300 import _native as N
    torch.cuda.init()
    return N


def _plan(N, res, nsub, mod, k, sep=2):
    geom = O.pyramid_geometry(res, nsub, sep)
    path, K = O.modulation_path(mod, k)
    pupil = O.telescope_pupil(res)
    inten = O.source_intensity(pupil, O.n_photon('V0', 8), 1e-3, 8.0)
    h = ctypes.c_void_p()
    mask = np.ascontiguousarray(geom.mask, dtype=np.complex64)
    p = np.ascontiguousarray(path, dtype=np.float64)
    N.call('oopao_pwfs_plan_create', ctypes.byref(h), res, geom.N, geom.cam, K, mask, p, 1.0, 1)
    amp = np.ascontiguousarray(np.sqrt(inten / K), dtype=np.float32)
    N.call('oopao_pwfs_set_amplitude', h, amp)
    return h, geom, pupil


def _with_workspace(N, h, x, frame, raw):
    import torch
    nb = N.load().oopao_pwfs_workspace_bytes(h, x.shape[0])
    ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
    N.call('oopao_pwfs_measure', h, N.ptr(x), 1.0, x.shape[0], N.ptr(frame), N.ptr(raw), N.ptr(ws), nb,
           N.stream_handle())


def test_noalloc_matches_workspace_entry_point(native):
    import torch
    N = native
    h, geom, pupil = _plan(N, 120, 20, 3, 48)
    try:
        rng = np.random.default_rng(11)
        for call in range(2):
            phase = rng.standard_normal((3, 120, 120)) * pupil * (1.0 + call)
            x = torch.as_tensor(phase.astype(np.float32), device='cuda')
            f_ref = torch.empty((3, geom.cam, geom.cam), device='cuda')
            _with_workspace(N, h, x, f_ref, None)
            f_na = torch.full((3, geom.cam, geom.cam), float('nan'), device='cuda')
            N.call('oopao_pwfs_measure_noalloc', h, N.ptr(x), 1.0, 3, N.ptr(f_na), None, N.stream_handle())
            torch.cuda.synchronize()
            a, b = f_na.double().cpu().numpy(), f_ref.double().cpu().numpy()
            assert np.isfinite(a).all()
            assert O.rel_l2(a, b) < TOL, (call, O.rel_l2(a, b))
            # with raw_data requested (un-binned partial sums in the same scratch)
            r_ref = torch.empty((1, geom.N, geom.N), device='cuda')
            f1 = torch.empty((1, geom.cam, geom.cam), device='cuda')
            _with_workspace(N, h, x[:1].contiguous(), f1, r_ref)
            r_na = torch.full((1, geom.N, geom.N), float('nan'), device='cuda')
            f2 = torch.empty((1, geom.cam, geom.cam), device='cuda')
            N.call('oopao_pwfs_measure_noalloc', h, N.ptr(x[:1].contiguous()), 1.0, 1, N.ptr(f2), N.ptr(r_na),
                   N.stream_handle())
            torch.cuda.synchronize()
            assert O.rel_l2(r_na.double().cpu().numpy(), r_ref.double().cpu().numpy()) < TOL
            assert O.rel_l2(f2.double().cpu().numpy(), f1.double().cpu().numpy()) < TOL
    finally:
        N.load().oopao_pwfs_plan_destroy(h)


def test_noalloc_rejects_plans_beyond_its_scratch(native):
    """An FFT grid whose smallest pass exceeds 64 MiB returns OOPAO_ERR_WORKSPACE
    without launching anything."""
    import torch
    N = native
    res, n, cam, k = 480, 1920, 320, 4
    h = ctypes.c_void_p()
    mask = np.ones((n, n), np.complex64)
    path = np.zeros((k, 2))
    N.call('oopao_pwfs_plan_create', ctypes.byref(h), res, n, cam, k, mask, path, 1.0, 1)
    try:
        x = torch.zeros((1, res, res), device='cuda')
        f = torch.empty((1, cam, cam), device='cuda')
        st = N.load().oopao_pwfs_measure_noalloc(h, N.ptr(x), 1.0, 1, N.ptr(f), None, N.stream_handle())
        assert st == 4
        assert b'allocation-free scratch' in N.load().oopao_last_error()
    finally:
        N.load().oopao_pwfs_plan_destroy(h)
