"""Benchmark: PWFS frames/s of the batched interaction-matrix build.

Workload (N=1): the "batched calibration" configuration — 8 m pupil, 120 px
(6 px/subaperture), 20x20 pyramid (N=264 FFT grid, 44x44 camera),
modulation 3 lambda/D with 48 points, 21x21 Gaussian-IF DM (357 valid
actuators, coupling 0.35), 300 KL modes, push-pull +-1e-8 m RMS,
float32 commands, FP64 SVD reconstructor keeping 280 modes.  One step = one
push-pull interaction matrix = 600 PWFS frames (each frame = 48 modulation
points).

  value: frames/s with the mode basis and IFs resident on the GPU
         (DM GEMM -> batched propagation -> signals, no host copies)
  e2e:   frames/s through the public call
         InteractionMatrix(ngs, tel, dm, wfs, M2C, stroke, single_pass=False,
         nTrunc=20) with M2C in host memory and the CalibrationVault
         returned to host memory

``--impl reference`` times the float64 CPU oracle port of the reference
algorithm on the host cores on a bounded sample of the same workload.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import contextlib
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RES, NSUB, MOD, NTHETA, NMODES, STROKE, NTRUNC = 120, 20, 3, 48, 300, 1e-8, 20
WORKLOAD = ('batched push-pull interaction matrix: 8 m, 120 px, 20x20 PWFS (N=264, cam 44), '
            'modulation 3 l/D x 48 points, 21x21 Gaussian DM (357 act), 300 KL modes, '
            '+-1e-8 m RMS, FP64 SVD 280 modes')


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


_KL_CACHE = {}


def kl_like_basis(modes, pupil, n_modes, diameter=8.0, r0=0.15, L0=25.0):
    """KL modal basis M2C [n_act, n_modes] of the DM, computed as the
    reference's compute_KL_basis does (oopao_gb300.modal_basis: tip/tilt
    fitted, seed basis, diagonalisation of the von Karman HHt; piston
    removed), truncated to the first n_modes.  Modes are orthonormal over the
    pupil (1 m RMS per unit coefficient).  Cached per DM geometry."""
    import types
    from oopao_gb300.modal_basis import compute_KL_basis
    key = (modes.shape, pupil.shape, float(np.asarray(modes).sum()), diameter, r0, L0)
    if key not in _KL_CACHE:
        tel = types.SimpleNamespace(pupil=pupil, resolution=pupil.shape[0], D=diameter)
        atm = types.SimpleNamespace(r0=r0, L0=L0)
        dm = types.SimpleNamespace(modes=modes, nValidAct=modes.shape[1], isM4=False)
        _KL_CACHE[key] = compute_KL_basis(tel, atm, dm)
    return np.ascontiguousarray(_KL_CACHE[key][:, :n_modes])


KL_FIXTURE = os.path.join(ROOT, 'tests', 'golden', 'kl_c1.npz')
ERR_COLS = 32


def reference_kl_c1(n_modes):
    """The first `n_modes` columns of the reference's own KL basis of the
    21x21 Gaussian DM on the 120 px, 8 m pupil (compute_KL_basis with lim
    1e-3, piston removed; stored by tests/golden/make_golden.py): 357 x
    n_modes float64, orthonormal over the pupil (1 m RMS per unit
    coefficient).  Both arms of the headline use it."""
    with np.load(KL_FIXTURE) as z:
        return np.ascontiguousarray(z['m2c'][:, :n_modes])


def err_columns(n_modes, n=ERR_COLS, seed=1234):
    """Seeded, sorted subset of `n` interaction-matrix columns on which the
    float64 oracle is run (all columns when there are at most `n`)."""
    if n_modes <= n:
        return list(range(n_modes))
    return sorted(int(c) for c in np.random.default_rng(seed).choice(n_modes, n, replace=False))


def oracle_im(res, nsub, mod, ntheta, m2c, stroke, cols, threads=None):
    """Float64 oracle push-pull columns `cols` of M2C at `stroke` (the
    reference's InteractionMatrix column rule) and its run time."""
    from oracle import pwfs_oracle as O
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    pup = O.telescope_pupil(res)
    inten = O.source_intensity(pup, O.n_photon('V0', 8), 1e-3, 8.0)
    ow = O.build_pyramid(res, nsub, mod, 0.5, inten, n_theta_user=ntheta, workers=threads)
    D = O.interaction_matrix(ow, O.dm_modes(res, 8.0, nsub), m2c[:, cols], stroke, O.PHOTOMETRY['V0'][0], pup,
                             single_pass=False, workers=threads)
    return D, time.perf_counter() - t0


def rel_fro(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def build_system(dev_index, res=RES, nsub=NSUB, mod=MOD, ntheta=NTHETA, max_batch=100, if_dtype='fp32'):
    import oopao_gb300 as og
    with _quiet():
        tel = og.Telescope(resolution=res, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=nsub, mechCoupling=0.35, if_dtype=if_dtype)
        wfs = og.Pyramid(nSubap=nsub, telescope=tel, modulation=mod, lightRatio=0.5,
                         nTheta_user_defined=ntheta, max_batch=max_batch)
    return tel, ngs, dm, wfs


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def im_comparison(tel, ngs, dm, wfs, m2c, n_per_mode, with_error=True):
    """Interaction-matrix build times of one system: the plain per-mode
    push-pull GPU path (operator path ngs**tel*dm*wfs per mode; its time is
    measured on the first `n_per_mode` modes and scaled linearly to all
    modes), the batched push-pull path and the batched tangent (JVP) path.
    Errors are relative Frobenius norms over ERR_COLS seeded columns (named
    in the output): the batched push-pull matrix against the float64 oracle
    at the same stroke, the tangent matrix against a float64 derivative (the
    oracle's push-pull at 1e-12 m)."""
    from oopao_gb300.calibration import InteractionMatrix
    from oopao_gb300.autodiff import jvp_interaction_matrix
    n_modes = m2c.shape[1]
    InteractionMatrix(ngs, tel, dm, wfs, m2c[:, :2], STROKE, single_pass=False, method='per_mode', invert=False)
    _, t_pm = _timed(lambda: InteractionMatrix(ngs, tel, dm, wfs, m2c[:, :n_per_mode], STROKE, single_pass=False,
                                               method='per_mode', invert=False))
    InteractionMatrix(ngs, tel, dm, wfs, m2c[:, :8], STROKE, single_pass=False, method='batched', invert=False)
    Db, t_b = _timed(lambda: InteractionMatrix(ngs, tel, dm, wfs, m2c, STROKE, single_pass=False,
                                               method='batched', invert=False))
    jvp_interaction_matrix(ngs, tel, dm, wfs, m2c[:, :8])
    D, t_j = _timed(lambda: jvp_interaction_matrix(ngs, tel, dm, wfs, m2c))
    out = {'modes': n_modes, 'per_mode_push_pull_ms': t_pm / n_per_mode * n_modes * 1000.0,
           'per_mode_push_pull_note': 'measured on %d modes, scaled linearly to %d' % (n_per_mode, n_modes),
           'per_mode_timed_modes': n_per_mode, 'batched_push_pull_ms': t_b * 1000.0, 'jvp_ms': t_j * 1000.0}
    out['jvp_speedup_vs_per_mode_push_pull'] = out['per_mode_push_pull_ms'] / out['jvp_ms']
    out['batched_speedup_vs_per_mode_push_pull'] = out['per_mode_push_pull_ms'] / out['batched_push_pull_ms']
    if with_error:
        res, nsub, k = tel.resolution, int(round(dm.nActAlongDiameter)), wfs.nTheta
        cols = err_columns(n_modes)
        Dd, t1 = oracle_im(res, nsub, wfs.modulation, k, m2c, 1e-12, cols)
        Dp, t2 = oracle_im(res, nsub, wfs.modulation, k, m2c, STROKE, cols)
        out['error_columns'] = cols
        out['jvp_rel_fro_err_vs_fp64_derivative'] = rel_fro(D[:, cols].double().cpu().numpy(), Dd)
        out['batched_rel_fro_err_vs_fp64_push_pull'] = rel_fro(np.asarray(Db.D)[:, cols], Dp)
        out['oracle_seconds'] = t1 + t2
    return out


def cl_rate(n_steps=2000, n_oracle=20):
    """Graph-replayed closed-loop steps/s on the 40x40 configuration: 240 px,
    N=504, modulation 5 l/D x 96 points, 41x41 DM, 3-layer infinite phase
    screens (r0 0.12 m, L0 30 m, 0/5/10 km, 10/15/20 m/s, updated on the GPU
    inside the captured step), 1000-mode KL integrator (gain 0.4,
    delay 1, reconstructor M2C @ M from the JVP interaction matrix and its
    full FP64 pseudo-inverse); BF16 tensor-core IF projection with FP32
    accumulation.  Reports the replay rate and the residual of the loop, and
    the error against the float64 oracle loop (same reconstructor, the
    float64 restatement of the same seeded infinite screens) over the first
    `n_oracle` frames: slopes of every frame, residual WFE trajectory,
    long-exposure PSF and Strehl ratio, final commands."""
    import torch
    from oopao_gb300.autodiff import jvp_interaction_matrix
    from oopao_gb300.calibration import CalibrationVault
    from oopao_gb300 import Atmosphere
    from oopao_gb300.closed_loop import ClosedLoop
    from oopao_gb300 import autotune
    tel, ngs, dm, wfs = build_system(0, 240, 40, 5, 96, max_batch=16, if_dtype='bf16')
    m2c = kl_like_basis(dm.modes, tel.pupil, 1000, r0=0.12, L0=30.0)
    D = jvp_interaction_matrix(ngs, tel, dm, wfs, m2c).double().cpu().numpy()
    with _quiet():
        R = m2c @ np.asarray(CalibrationVault(D).M)
    autotune.tune_pyramid(wfs, batch=1)
    with _quiet():
        atm = Atmosphere(telescope=tel, r0=0.12, L0=30, fractionalR0=[1 / 3, 1 / 3, 1 / 3],
                         windSpeed=[10., 15., 20.], windDirection=[0., 72., 144.], altitude=[0., 5000., 10000.])
        atm.initializeAtmosphere(tel)

    def timed_loop(nvtx=None):
        cl = ClosedLoop(tel, ngs, dm, wfs, R, gain=0.4, layers=atm, max_steps=n_steps + 30)
        cl.capture()
        cl.run(20)
        torch.cuda.synchronize()
        cl.reset()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if nvtx:
            torch.cuda.nvtx.range_push(nvtx)
        e0.record()
        cl.run(n_steps)
        e1.record()
        if nvtx:
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n_steps, cl.residual_wfe

    # the DM's default projection (separable Gaussian IFs), then the dense
    # BF16 tensor-core GEMV over the same IFs for comparison
    path = dm.projection_path()
    ms, wfe = timed_loop('cl_steps')
    dm.separable_projection = False
    ms_dense, wfe_dense = timed_loop('cl_steps_dense_dm')
    dm.separable_projection = path == 'separable'
    oracle = cl_oracle_error(tel, ngs, dm, wfs, R, atm, n_oracle,
                             (0.12, 30.0, [1 / 3, 1 / 3, 1 / 3], [10., 15., 20.], [0., 72., 144.],
                              [0., 5000., 10000.]))
    return {'config': '40x40 PWFS, 240 px, N=504, 96 points, 41x41 DM (%d act), 3 infinite-screen layers, '
                      '1000 KL modes'
                      % dm.nValidAct, 'fp64_oracle': oracle,
            'steps': n_steps, 'us_per_step': ms * 1000.0, 'khz': 1.0 / ms,
            'graph': True, 'variant': int(N_variant(wfs)), 'dm': path,
            'us_per_step_dense_bf16_dm': ms_dense * 1000.0,
            'wfe_rel_diff_dense_vs_default': float(np.linalg.norm(wfe_dense - wfe) / np.linalg.norm(wfe)),
            'tc_status': dm.tensor_core_status(), 'wfe_first_nm': float(wfe[0] * 1e9),
            'wfe_mean_last_500_nm': float(wfe[-500:].mean() * 1e9)}


def cl_oracle_error(tel, ngs, dm, wfs, R, atm, n_oracle, atm_params, gain=0.4):
    """Run `n_oracle` eager steps of the GPU loop (science PSF on) and the
    float64 oracle loop on the same reconstructor and the float64
    restatement of the same seeded atmosphere; relative L2 errors of the
    per-frame slopes, the residual WFE trajectory, the long-exposure PSF, the
    final commands and the Strehl ratio."""
    import torch
    from oopao_gb300.closed_loop import ClosedLoop
    from oracle import atm_oracle as A
    from oracle import pwfs_oracle as O
    res, nsub = tel.resolution, int(round(dm.nActAlongDiameter))
    cl = ClosedLoop(tel, ngs, dm, wfs, R, gain=gain, layers=atm, max_steps=n_oracle + 10, science=True)
    sig = []
    for _ in range(n_oracle):
        cl.step()
        sig.append(cl.s[0].double().cpu().numpy())
    torch.cuda.synchronize()
    wfe, psf, sr = cl.residual_wfe, cl.long_exposure_psf(), cl.long_exposure_strehl()
    coefs = cl.coefs.double().cpu().numpy()
    del cl
    t0 = time.perf_counter()
    pup = O.telescope_pupil(res)
    inten = O.source_intensity(pup, O.n_photon('V0', 8), 1e-3, 8.0)
    ow = O.build_pyramid(res, nsub, wfs.modulation, 0.5, inten, n_theta_user=wfs.nTheta, workers=os.cpu_count())
    r0, L0, fr, ws, wd, alt = atm_params
    ora = A.OracleAtmosphere(res, tel.D, 1e-3, r0, L0, fr, ws, wd, alt)

    def turbulence(t):
        ora.update()            # step t sees the atmosphere after t + 1 updates
        return ora.opd

    ref = O.closed_loop(ow, O.dm_modes(res, tel.D, nsub), np.asarray(R, np.float64), turbulence, pup,
                        ngs.wavelength, gain, n_oracle, workers=os.cpu_count(), record_signals=True)
    sig = np.stack(sig)
    per_frame = [O.rel_l2(sig[t], ref['signals'][t]) for t in range(n_oracle)]
    return {'frames': n_oracle, 'oracle_seconds': time.perf_counter() - t0,
            'signal_rel_l2': O.rel_l2(sig, ref['signals']), 'signal_rel_l2_max_frame': max(per_frame),
            'wfe_rel_l2': O.rel_l2(wfe, ref['wfe']), 'psf_le_rel_l2': O.rel_l2(psf, ref['psf_le']),
            'commands_rel_l2': O.rel_l2(coefs, ref['coefs']),
            'strehl_le_pct': sr, 'oracle_strehl_le_pct': ref['strehl_le'],
            'strehl_rel_err': abs(sr - ref['strehl_le']) / ref['strehl_le'],
            'wfe_nm_first_last': [float(wfe[0] * 1e9), float(wfe[-1] * 1e9)]}


def cl_strehl(n_steps=500, n_oracle=100):
    """Plain closed loop on the 20x20 configuration: 8 m, 120 px, modulation
    3 l/D x 48 points, 21x21 DM, one infinite-screen von Karman layer (r0
    0.15 m at 500 nm, L0 25 m, 10 m/s, the reference's seeds), 300-mode KL
    integrator (gain 0.4, delay 1,
    reconstructor M2C @ M from the batched IM and its full FP64 pseudo-inverse,
    as the reference tutorial builds it), `n_steps` frames at 1 kHz with the
    science PSF summed on the GPU.
    The float64 oracle runs the first `n_oracle` frames of the same loop with
    the same reconstructor; the error of the residual WFE trajectory, of the
    long-exposure PSF and of its Strehl ratio over those frames is reported."""
    import torch
    from oopao_gb300.calibration import InteractionMatrix
    from oopao_gb300 import Atmosphere
    from oopao_gb300.closed_loop import ClosedLoop
    from oracle import atm_oracle as A
    from oracle import pwfs_oracle as O
    tel, ngs, dm, wfs = build_system(0)
    m2c = kl_like_basis(dm.modes, tel.pupil, NMODES)
    with _quiet():
        calib = InteractionMatrix(ngs, tel, dm, wfs, m2c, STROKE, single_pass=False)
        layers = Atmosphere(telescope=tel, r0=0.15, L0=25, fractionalR0=[1.0], windSpeed=[10.], windDirection=[0.],
                            altitude=[0.])
        layers.initializeAtmosphere(tel)
    R = m2c @ np.asarray(calib.M)
    out = {'config': '20x20 PWFS, 120 px, N=264, 48 points, 21x21 DM, 1 layer r0 0.15 m, 300-mode integrator '
                     'gain 0.4, %d frames' % n_steps}
    for science in (False, True):
        cl = ClosedLoop(tel, ngs, dm, wfs, R, gain=0.4, layers=layers, max_steps=n_steps + 10, science=science)
        cl.capture()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        cl.run(n_oracle)
        e1.record()
        torch.cuda.synchronize()
        key = 'with_science_psf' if science else 'wfs_only'
        out['us_per_step_' + key] = e0.elapsed_time(e1) / n_oracle * 1000.0
    wfe100, psf100, sr100 = cl.residual_wfe, cl.long_exposure_psf(), cl.long_exposure_strehl()
    cl.run(n_steps - n_oracle)
    torch.cuda.synchronize()
    wfe = cl.residual_wfe
    out.update({'strehl_le_pct': cl.long_exposure_strehl(), 'wfe_first_nm': float(wfe[0] * 1e9),
                'wfe_mean_last_100_nm': float(wfe[-100:].mean() * 1e9)})
    pup = O.telescope_pupil(RES)
    inten = O.source_intensity(pup, O.n_photon('V0', 8), 1e-3, 8.0)
    ow = O.build_pyramid(RES, NSUB, MOD, 0.5, inten, n_theta_user=NTHETA, workers=os.cpu_count())
    t0 = time.perf_counter()
    ora = A.OracleAtmosphere(RES, 8.0, 1e-3, 0.15, 25.0, [1.0], [10.0], [0.0], [0.0])

    def turbulence(t):
        ora.update()            # step t sees the atmosphere after t + 1 updates
        return ora.opd

    ref = O.closed_loop(ow, O.dm_modes(RES, 8.0, NSUB), R.astype(np.float64), turbulence, pup,
                        ngs.wavelength, 0.4, n_oracle, workers=os.cpu_count())
    out['oracle'] = {'frames': n_oracle, 'seconds': time.perf_counter() - t0,
                     'strehl_le_pct': ref['strehl_le'], 'gpu_strehl_le_pct': sr100,
                     'strehl_rel_err': abs(sr100 - ref['strehl_le']) / ref['strehl_le'],
                     'psf_le_rel_l2': O.rel_l2(psf100, ref['psf_le']),
                     'wfe_rel_l2': O.rel_l2(wfe100, ref['wfe'])}
    return out


def large_config(n_modes=4000, chunk=16, oracle_cols=4, n_loop=200):
    """39 m, 480 px, 80x80 pyramid (N=1920, 320x320 camera, modulation 4 l/D
    x 128 points), 81x81 Gaussian DM: frames/s of the autotuned plan at batch
    1 and 4; a 4000-mode interaction matrix built by batched tangents (JVPs)
    around the flat wavefront, whose operating-point fields G_k of the 128
    points are computed once and kept (3.8 GB, the checkpoint every tangent
    reads); and the graph-replayed closed-loop step with 35 infinite-screen
    layers (r0 0.157 m, L0 25 m).  The modes are seeded random commands of
    the 81x81 DM (smooth DM shapes, 10 nm RMS): a KL basis at this size needs
    the dense 9.6 GB IF matrix.  Error: `oracle_cols` columns against a
    float64 central difference (+-1e-3 rad RMS) of the float64 oracle.  The
    loop's reconstructor is a zero matrix of the right size (5209 x 10048):
    the MVM runs in full, the timing does not depend on its values."""
    import torch
    import oopao_gb300 as og
    from oopao_gb300 import autodiff as AD
    from oopao_gb300 import autotune
    from oopao_gb300.closed_loop import ClosedLoop
    with _quiet():
        tel = og.Telescope(resolution=480, diameter=39.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        wfs = og.Pyramid(nSubap=80, telescope=tel, modulation=4, lightRatio=0.5, n_pix_separation=80, n_pix_edge=40,
                         nTheta_user_defined=128, max_batch=chunk)
        t0 = time.perf_counter()
        dm = og.DeformableMirror(tel, nSubap=80, mechCoupling=0.35)
        dm_build_s = time.perf_counter() - t0
    ngs ** tel
    wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
    out = {'config': '39 m, 480 px, 80x80 PWFS, N=1920, cam 320, modulation 4 l/D x 128 points, 81x81 DM',
           'n_signal': wfs.nSignal, 'n_act': dm.nValidAct, 'dm_build_s': dm_build_s,
           'dm_projection': dm.projection_path()}
    g = torch.Generator(device='cuda').manual_seed(0)
    for B in (1, 4):
        tune = autotune.tune_pyramid(wfs, batch=B)
        opd = torch.randn((B, 480, 480), device='cuda', generator=g) * 50e-9
        wfs._measure_frames(opd, 2 * np.pi / ngs.wavelength)
        _, t = _timed(lambda: [wfs._measure_frames(opd, 2 * np.pi / ngs.wavelength) for _ in range(3)])
        out['frames_per_s_batch%d' % B] = 3 * B / t
        out['variant_batch%d' % B] = tune['variant']
    # ---- 4000-mode IM from batched tangents
    autotune.tune_pyramid(wfs, batch=chunk)
    cmd = torch.randn((dm.nValidAct, n_modes), device='cuda', generator=g)
    pup = torch.as_tensor(tel.pupil, dtype=torch.float32, device='cuda') > 0
    rms = torch.stack([dm.opd_device(cmd[:, i:i + 64].contiguous())[:, pup].std(dim=1)
                       for i in range(0, 256, 64)]).mean()
    cmd *= 10e-9 / rms
    opd0 = torch.zeros((1, 480, 480), device='cuda')
    frame0 = AD.frames(wfs, opd0)

    def build_im():
        cols = []
        for b0 in range(0, n_modes, chunk):
            dopd = dm.opd_device(cmd[:, b0:b0 + chunk].contiguous())
            _, ds = AD.signal_jvp(wfs, frame0, AD.frame_jvp(wfs, opd0, dopd))
            cols.append(ds)
        return torch.cat(cols).T

    build_im()  # warm-up (plans, workspaces)
    D, t_im = _timed(build_im)
    out['im_modes'] = n_modes
    out['im_build_s'] = t_im
    out['im_tangents_per_s'] = n_modes / t_im
    out['im_chunk'] = chunk
    out['checkpoint_bytes'] = 128 * 1920 * 1920 * 8
    # float64 oracle derivative of the camera frame along a few modes
    if oracle_cols:
        from oracle import pwfs_oracle as O
        workers = os.cpu_count() or 1
        t0 = time.perf_counter()
        geom = O.pyramid_geometry(480, 80, 80, n_pix_edge=40)
        path, K = O.modulation_path(4, 128)
        tt = O.tt_buffers(path, geom)
        inten = O.source_intensity(O.telescope_pupil(480), O.n_photon('V0', 8), 1e-3, 39.0)
        scale = 2 * np.pi / ngs.wavelength
        errs = []
        cols = [int(c) for c in np.random.default_rng(7).choice(n_modes, oracle_cols, replace=False)]
        for c in cols:
            dopd = dm.opd_device(cmd[:, c:c + 1].contiguous())
            got = AD.frame_jvp(wfs, opd0, dopd)[0].double().cpu().numpy()
            dphi = dopd[0].double().cpu().numpy() * scale * tel.pupil
            h = 1e-3 / np.sqrt((dphi[tel.pupil > 0] ** 2).mean())
            fp = O.camera_frame(O.wfs_raw(h * dphi, inten, tt, geom, workers=workers), geom)
            fm = O.camera_frame(O.wfs_raw(-h * dphi, inten, tt, geom, workers=workers), geom)
            ref = (fp - fm) / (2 * h)
            errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
        out['im_frame_derivative_rel_err_vs_fp64_oracle'] = {
            'columns': cols, 'rel_l2': errs, 'oracle_seconds': time.perf_counter() - t0,
            'reference': 'float64 oracle camera frames, central difference +-1e-3 rad RMS'}
    del D, cmd
    # ---- 35-layer closed-loop step
    with _quiet():
        atm = og.Atmosphere(telescope=tel, r0=0.157, L0=25, fractionalR0=[1 / 35] * 35,
                            windSpeed=list(np.linspace(5., 30., 35)), windDirection=list(np.linspace(0., 340., 35)),
                            altitude=list(np.linspace(0., 20000., 35)))
        atm.initializeAtmosphere(tel)
    autotune.tune_pyramid(wfs, batch=1)
    R = np.zeros((dm.nValidAct, wfs.nSignal), dtype=np.float32)
    cl = ClosedLoop(tel, ngs, dm, wfs, R, gain=0.4, layers=atm, max_steps=n_loop + 30)
    cl.capture()
    cl.run(10)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    cl.run(n_loop)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n_loop
    out['cl_35_layers'] = {'steps': n_loop, 'us_per_step': ms * 1e3, 'hz': 1e3 / ms, 'graph': True,
                           'layers': 35, 'atm_status': atm.status(),
                           'reconstructor': 'zero matrix %dx%d (timing only)' % R.shape}
    return out


def config4_leg(n_modes=500, n_screens=64, n_steps=200, sigma=50e-9, n_fd=4, seed=0):
    """Differentiable PWFS on the 40x40 optics (240 px, N=504, 96 points,
    41x41 DM): the loss ||signal(M2C x) - target||^2 over the first 500 KL
    modes, 64 seeded modal screens with coefficients ~N(0, 50 nm) (the modes
    are 1 m RMS per unit coefficient), the targets measured through the same
    sensor.  Reports the hand-written adjoint gradient against central finite
    differences (step 1e-3 rad RMS of phase along seeded unit directions, every
    screen) and against the gradient of the push-pull interaction matrix
    (2 D^T (s - t), stroke 1e-8 m) at the flat operating point, then the time
    per step of 200 batched gradient-descent (Adam) steps and the loss and
    modal error before and after."""
    import torch
    import oopao_gb300 as og
    from oopao_gb300 import autodiff as AD
    from oopao_gb300 import autotune
    tel, ngs, dm, wfs = build_system(0, 240, 40, 5, 96, max_batch=n_screens)
    m2c = kl_like_basis(dm.modes, tel.pupil, n_modes, r0=0.12, L0=30.0)
    autotune.tune_pyramid(wfs, batch=n_screens)
    ngs ** tel
    truth = np.stack([np.random.default_rng(seed + s).standard_normal(n_modes) for s in range(n_screens)], axis=1)
    truth *= sigma
    dev = wfs._dev
    m = torch.as_tensor(m2c, dtype=torch.float32, device=dev)
    with torch.no_grad():
        targets = AD.dm_signal(wfs, dm, m @ torch.as_tensor(truth, dtype=torch.float32, device=dev))
    x0 = np.zeros_like(truth)
    loss0, g = AD.modal_loss_grad(wfs, dm, m2c, x0, targets)
    g = g.double().cpu().numpy()
    # adjoint against central differences of the loss
    rng = np.random.default_rng(seed + 1000)
    h = 1e-3 * ngs.wavelength / (2 * np.pi)
    fd_err = []
    for _ in range(n_fd):
        u = rng.standard_normal(truth.shape)
        u /= np.linalg.norm(u, axis=0)
        lp = AD.modal_loss(wfs, dm, m2c, x0 + h * u, targets).cpu().numpy()
        lm = AD.modal_loss(wfs, dm, m2c, x0 - h * u, targets).cpu().numpy()
        fd = (lp - lm) / (2 * h)
        ad = (g * u).sum(axis=0)
        fd_err.append(float(np.max(np.abs(fd - ad)) / np.max(np.abs(ad))))
    # adjoint against the push-pull interaction matrix at the flat point
    with _quiet():
        calib = og.InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=1, single_pass=False,
                                     invert=False)
    with torch.no_grad():
        s0 = AD.dm_signal(wfs, dm, torch.zeros((dm.nValidAct, 1), device=dev))
    r = s0.double().cpu().numpy()[0][:, None] - targets.double().cpu().numpy().T
    g_pp = 2 * np.asarray(calib.D).T @ r
    pp_err = float(np.linalg.norm(g - g_pp) / np.linalg.norm(g_pp))
    # batched gradient descent
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x, hist = AD.modal_gradient_descent(wfs, dm, m2c, targets, n_iter=n_steps, lr=0.2 * sigma)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    xe = x.double().cpu().numpy()
    # the same estimation in the sensor's linear range: the screens scaled to
    # 50 nm RMS in total (coefficients ~N(0, 50 nm / sqrt(500)))
    lin = truth / np.sqrt(n_modes)
    with torch.no_grad():
        t_lin = AD.dm_signal(wfs, dm, m @ torch.as_tensor(lin, dtype=torch.float32, device=dev))
    x_lin, h_lin = AD.modal_gradient_descent(wfs, dm, m2c, t_lin, n_iter=n_steps // 2,
                                             lr=0.2 * sigma / np.sqrt(n_modes))
    lin_err = float(np.linalg.norm(x_lin.double().cpu().numpy() - lin) / np.linalg.norm(lin))
    return {'config': '40x40 PWFS, 240 px, N=504, 96 points, 41x41 DM, %d KL modes, %d seeded modal screens, '
                      'coefficients ~N(0, %g nm)' % (n_modes, n_screens, sigma * 1e9),
            'linear_range': {'coefficients': 'N(0, %.2f nm): 50 nm RMS wavefronts' % (sigma * 1e9 / np.sqrt(n_modes)),
                             'gd_steps': n_steps // 2, 'loss_first': h_lin[0], 'loss_last': h_lin[-1],
                             'modal_rel_err_last': lin_err},
            'adjoint_vs_fd_1e-3rad_max_rel_err': max(fd_err), 'fd_directions': n_fd,
            'adjoint_vs_push_pull_im_rel_err': pp_err,
            'gd_steps': n_steps, 'gd_ms_per_step': el * 1000.0 / n_steps, 'optimizer': 'Adam, lr 0.2 sigma',
            'loss_first': hist[0], 'loss_last': hist[-1], 'loss_at_step_50': hist[min(49, len(hist) - 1)],
            'modal_rel_err_first': 1.0, 'modal_rel_err_last': float(np.linalg.norm(xe - truth) / np.linalg.norm(truth)),
            'wavefront_rms_nm_truth': float(np.sqrt((truth ** 2).sum(axis=0)).mean() * 1e9)}


def dm_projection(peaks):
    """DM influence-function projection OPD = modes @ coefs at the 20x20,
    40x40 and 80x80 sizes: FP32 CUDA-core path vs BF16 tcgen05 path vs the
    FP32-accuracy tcgen05 path (three TF32 products, batches from 16), per
    batch, and the separable projection of Gaussian IFs on the same actuator
    grid ('separable': factors [n_side+1][res], the DM's default path).
    Modes and factors are seeded device-random (timing does not depend on
    the values).  Dense FLOPs 2*n_pix*n_act*B; IF bytes are the bytes of the
    IF matrix one call streams (FP32 [n_act][n_pix] or BF16
    [n_pix][n_act_pad])."""
    import torch
    from oopao_gb300 import _native as N
    lib = N.load()
    st = N.stream_handle()
    out = {}
    for name, n_side, n_act in (('20x20', 120, 357), ('40x40', 240, 1353), ('80x80', 480, 5209)):
        n_pix = n_side * n_side
        n_pad = (n_act + 63) // 64 * 64
        g = torch.Generator(device='cuda').manual_seed(0)
        mt = torch.randn((n_act, n_pix), device='cuda', generator=g)
        mb = torch.empty((n_pix, n_pad), dtype=torch.bfloat16, device='cuda')
        N.call('oopao_dm_modes_bf16', mt, n_act, n_pix, n_pad, mb, st)
        n_pad32 = (n_act + 31) // 32 * 32
        m2 = torch.empty((2, n_pix, n_pad32), dtype=torch.float32, device='cuda')
        N.call('oopao_dm_modes_tf32x2', mt, n_act, n_pix, n_pad32, m2, st)
        n_grid = int(name.split('x')[0]) + 1
        gxs = torch.randn((n_grid, n_side), device='cuda', generator=g)
        gys = torch.randn((n_grid, n_side), device='cuda', generator=g)
        cells = torch.full((n_grid * n_grid,), -1, dtype=torch.int32, device='cuda')
        cells[:n_act] = torch.arange(n_act, dtype=torch.int32, device='cuda')
        rows = []
        for B in (1, 16, 64, 300):
            c = torch.randn((n_act, B), device='cuda', generator=g)
            o = torch.empty((B, n_pix), device='cuda')
            nb = lib.oopao_dm_bf16_workspace_bytes(n_pad, B)
            ws = torch.zeros(nb, dtype=torch.uint8, device='cuda')
            nbs = lib.oopao_dm_sep_workspace_bytes(n_grid, n_side, B)
            wss = torch.zeros(nbs, dtype=torch.uint8, device='cuda')
            nbt = lib.oopao_dm_tf32_workspace_bytes(n_pad32, B)
            wst = torch.zeros(nbt, dtype=torch.uint8, device='cuda')
            runs = {'fp32': lambda: N.call('oopao_dm_opd_acc_f32', mt, c, n_act, n_pix, B, 1.0, None, o, st),
                    'bf16_tc': lambda: N.call('oopao_dm_opd_bf16', mb, n_pad, c, n_act, n_pix, B, 1.0, None, o, ws,
                                              nb, st),
                    'separable': lambda: N.call('oopao_dm_opd_sep_f32', gxs, gys, cells, n_grid, n_grid, c, n_act,
                                                n_side, B, 1.0, None, o, wss, nbs, st)}
            if B >= 16:
                runs['tf32x3_tc'] = lambda: N.call('oopao_dm_opd_tf32x3', m2, n_pad32, c, n_act, n_pix, B, 1.0, None,
                                                   o, wst, nbt, st)
            row = {'batch': B}
            for key, fn in runs.items():
                reps = 20
                for _ in range(3):
                    fn()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    fn()
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                if key == 'separable':
                    row[key] = {'ms': ms, 'dense_equivalent_tflops': 2.0 * n_pix * n_act * B / ms / 1e9,
                                'tflops': 2.0 * n_grid * n_side * (n_grid + n_side) * B / ms / 1e9}
                    continue
                if_bytes = {'fp32': n_pix * n_act * 4, 'bf16_tc': n_pix * n_pad * 2,
                            'tf32x3_tc': 2 * n_pix * n_pad32 * 4}[key]
                row[key] = {'ms': ms, 'tflops': 2.0 * n_pix * n_act * B / ms / 1e9,
                            'if_gbs': if_bytes / ms / 1e6}
                if key == 'bf16_tc' and peaks.get('bf16_tflops'):
                    row[key]['tensor_frac_of_measured_bf16'] = row[key]['tflops'] / peaks['bf16_tflops']
                if peaks.get('hbm_gbs'):
                    row[key]['hbm_frac_of_measured'] = row[key]['if_gbs'] / peaks['hbm_gbs']
            row['tc_error_word'] = int(ws[:4].view(torch.int32).item()) | int(wst[:4].view(torch.int32).item())
            rows.append(row)
        out[name] = {'n_pix': n_pix, 'n_act': n_act, 'if_bf16_mb': n_pix * n_pad * 2 / 1e6,
                     'l2_resident': n_pix * n_pad * 2 < 120e6, 'rows': rows}
        del mt, mb, m2
        torch.cuda.empty_cache()
    return out


def gsc_leg(peaks):
    """Gain-sensing camera: optical gains per focal-plane frame at the 20x20
    (N=264, 300 modes) and 40x40 (N=504, 1000 modes) pyramid sizes, batch 1
    and 16, through oopao_gsc_optical_gains (seven launches: frame sums,
    two 2-D transforms, contraction with the basis product, sums over
    chunks).  The basis product (modes x N^2 float32) is streamed once per
    call; `bp_gbs` is its bytes over the whole call's time, a lower bound on
    the contraction's bandwidth.  The float64 oracle (numpy, the reference's
    algorithm) is timed on one frame at 20x20."""
    import torch
    from oopao_gb300 import GainSensingCamera
    from oopao_gb300 import _native as N
    from oracle import gsc_oracle as G
    from oracle import pwfs_oracle as O
    out = {}
    for name, res, nsub, n_modes in (('20x20', 120, 20, 300), ('40x40', 240, 40, 1000)):
        geom = O.pyramid_geometry(res, nsub, 2)
        n = geom.N
        rng = np.random.default_rng(0)
        basis = rng.standard_normal((res, res, n_modes)).astype(np.float32) * 1e-8
        r = np.hypot(*np.meshgrid(np.arange(n) - n / 2, np.arange(n) - n / 2))
        frame = (np.exp(-(r / 10.0) ** 2) + 1e-3).astype(np.float32)
        gsc = GainSensingCamera(np.asarray(geom.mask, np.complex64), basis)
        _, t_cal = _timed(lambda: gsc.calibration(frame))
        lib = N.load()
        st = N.stream_handle()
        rows = []
        for B in (1, 16):
            f = torch.as_tensor(np.broadcast_to(frame, (B, n, n)).copy(), device='cuda')
            og = torch.empty((B, n_modes), dtype=torch.float64, device='cuda')
            nb = lib.oopao_gsc_workspace_bytes(gsc._plan, B)
            ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
            fn = lambda: N.call('oopao_gsc_optical_gains', gsc._plan, f, B, og, None, None, ws, nb, st)
            for _ in range(3):
                fn()
            reps = 20
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            bp_bytes = n_modes * n * n * 4
            row = {'batch': B, 'ms': ms, 'frames_per_s': B / ms * 1e3, 'bp_gbs': bp_bytes / ms / 1e6,
                   'og_at_calibration_point_max_dev': float((og - 1).abs().max())}
            if peaks.get('hbm_gbs'):
                row['bp_hbm_frac_of_measured'] = row['bp_gbs'] / peaks['hbm_gbs']
            rows.append(row)
        entry = {'N': n, 'modes': n_modes, 'basis_product_mb': n_modes * n * n * 4 / 1e6,
                 'calibration_s': t_cal, 'rows': rows}
        if name == '20x20':
            ref = G.OracleGSC(geom.mask, basis.astype(np.float64))
            ref.calibration(frame.astype(np.float64))
            t0 = time.perf_counter()
            ref.compute_optical_gains(frame.astype(np.float64))
            entry['oracle_cpu_ms_per_frame'] = (time.perf_counter() - t0) * 1e3
        out[name] = entry
        del gsc
        torch.cuda.empty_cache()
    return out


def cl_gsc(n_steps=500, og_start=30):
    """The reference's GSC tutorial loop on the 20x20 configuration: 300-mode
    KL modal reconstructor (push-pull IM, full FP64 pseudo-inverse), one
    infinite-screen layer (r0 0.10 m, L0 25 m, 10 m/s), gain 0.4, frame delay
    2; a GainSensingCamera on the 300 KL modes (basis = tel.OPD of the modes),
    calibrated on the flat-wavefront focal-plane frame; from step `og_start`
    the commands are M2C @ diag(1/og) @ M @ s.  Every step also forms the
    full-resolution focal-plane frame and its optical gains (captured in the
    same CUDA graph).  Reports us per step and the long-exposure Strehl with
    and without the compensation on the same turbulence."""
    import torch
    import oopao_gb300 as og
    from oopao_gb300.calibration import InteractionMatrix
    from oopao_gb300.closed_loop import ClosedLoop
    tel, ngs, dm, wfs = build_system(0)
    m2c = kl_like_basis(dm.modes, tel.pupil, NMODES)
    with _quiet():
        calib = InteractionMatrix(ngs, tel, dm, wfs, m2c, STROKE, single_pass=False)
        dm.coefs = m2c
        ngs ** tel * dm
        basis = np.array(tel.OPD)
        dm.coefs = 0
        gsc = og.GainSensingCamera(wfs.mask, basis)
        wfs.focal_plane_camera.resolution = wfs.nRes
        ngs ** tel * wfs
        wfs * wfs.focal_plane_camera
        wfs.focal_plane_camera * gsc
        atm = og.Atmosphere(telescope=tel, r0=0.10, L0=25, fractionalR0=[1.0], windSpeed=[10.], windDirection=[0.],
                            altitude=[0.])
        atm.initializeAtmosphere(tel)
    M = np.asarray(calib.M)
    out = {'config': '20x20 PWFS, 300 KL modes, 1 layer r0 0.10 m, gain 0.4, delay 2, %d frames, OG compensation '
                     'from frame %d' % (n_steps, og_start)}
    for key, start in (('with_og', og_start), ('without_og', 10 ** 9)):
        cl = ClosedLoop(tel, ngs, dm, wfs, M, gain=0.4, frame_delay=2, layers=atm, max_steps=n_steps + 10,
                        science=True, gsc=gsc, M2C=m2c, og_start=start)
        cl.capture()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        cl.run(n_steps)
        e1.record()
        torch.cuda.synchronize()
        ogv = cl.og[0].cpu().numpy()
        out[key] = {'us_per_step': e0.elapsed_time(e1) / n_steps * 1e3,
                    'strehl_le_pct': cl.long_exposure_strehl(),
                    'wfe_mean_last_100_nm': float(cl.residual_wfe[-100:].mean() * 1e9),
                    'og_first_modes': [float(v) for v in ogv[:5]], 'og_mean': float(ogv.mean())}
        del cl
    return out


def _event_ms(fn, reps, warm=3):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def next_rows_leg():
    """The components either side of the path, each against its float64 CPU
    counterpart (the oracle, i.e. the reference's algorithm in numpy):

    * BioEdge on the 20x20 configuration (120 px, N=264, 48 points, 4 Fourier
      masks): frames/s at batch 100 of random screens; oracle s per frame.
    * Atmosphere update (infinite screens, frozen flow, on the GPU): us per
      update for 1 layer at 120 px (10 m/s), 3 layers at 240 px (0/5/10 km,
      10/15/20 m/s) and 35 layers at 480 px (the 39 m configuration's
      profile size); oracle ms per update at 120 px and 240 px.
    * KL modal basis (compute_KL_basis, HHt on the GPU): seconds for the
      21x21 (357 actuators) and 41x41 (1353 actuators) DMs."""
    import types
    import torch
    import oopao_gb300 as og
    from oopao_gb300.modal_basis import compute_KL_basis
    from oracle import atm_oracle as A
    from oracle import bioedge_oracle as BO
    from oracle import pwfs_oracle as O
    out = {}
    # ---- BioEdge
    with _quiet():
        tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        wfs = og.BioEdge(nSubap=20, telescope=tel, modulation=3, lightRatio=0.5, nTheta_user_defined=48,
                         max_batch=100)
    ngs ** tel
    g = torch.Generator(device='cuda').manual_seed(0)
    opd = torch.randn((100, 120, 120), device='cuda', generator=g) * 50e-9
    scale = 2 * np.pi / ngs.wavelength
    ms = _event_ms(lambda: wfs._measure_frames(opd, scale), 5)
    inten = O.source_intensity(O.telescope_pupil(120), O.n_photon('V0', 8), 1e-3, 8.0)
    ob = BO.build_bioedge(120, 20, 3, 0.5, inten, n_theta_user=48)
    ph = np.random.default_rng(1).standard_normal((120, 120)) * 0.3
    t0 = time.perf_counter()
    ob.frame(ph)
    t_or = time.perf_counter() - t0
    out['bioedge_20x20'] = {'frames_per_s': 100 / ms * 1e3, 'ms_per_100_frames': ms, 'masks': 4,
                            'oracle_s_per_frame': t_or, 'speedup_vs_oracle': t_or / (ms / 100 / 1e3)}
    del wfs
    # ---- Atmosphere
    rows = []
    cases = (('1 layer, 120 px', 120, 8.0, [1.0], [10.], [0.], [0.]),
             ('3 layers, 240 px', 240, 8.0, [1 / 3] * 3, [10., 15., 20.], [0., 72., 144.], [0., 5000., 10000.]),
             ('35 layers, 480 px', 480, 39.0, [1 / 35] * 35, list(np.linspace(5., 30., 35)),
              list(np.linspace(0., 340., 35)), list(np.linspace(0., 20000., 35))))
    for name, res, D, fr, ws, wd, alt in cases:
        with _quiet():
            t = og.Telescope(resolution=res, diameter=D, samplingTime=1e-3)
            s = og.Source(optBand='V0', magnitude=8)
            s * t
            atm = og.Atmosphere(telescope=t, r0=0.15, L0=25, fractionalR0=fr, windSpeed=ws, windDirection=wd,
                                altitude=alt)
            atm.initializeAtmosphere(t)
        atm.prepare(260)
        us = _event_ms(atm.update, 200, warm=10) * 1e3
        row = {'case': name, 'us_per_update': us, 'status': atm.status()}
        if res <= 240:
            oa = A.OracleAtmosphere(res, D, 1e-3, 0.15, 25.0, fr, ws, wd, alt)
            oa.update()
            t0 = time.perf_counter()
            for _ in range(5):
                oa.update()
            row['oracle_ms_per_update'] = (time.perf_counter() - t0) / 5 * 1e3
        rows.append(row)
        del atm
    out['atmosphere'] = rows
    # ---- KL basis
    kl = []
    for nsub, res in ((20, 120), (40, 240)):
        pupil = O.telescope_pupil(res)
        modes = O.dm_modes(res, 8.0, nsub)
        tel_ = types.SimpleNamespace(pupil=pupil, resolution=res, D=8.0)
        atm_ = types.SimpleNamespace(r0=0.15, L0=25.0)
        dm_ = types.SimpleNamespace(modes=modes, nValidAct=modes.shape[1], isM4=False)
        t0 = time.perf_counter()
        m2c = compute_KL_basis(tel_, atm_, dm_)
        torch.cuda.synchronize()
        kl.append({'dm': '%dx%d' % (nsub + 1, nsub + 1), 'actuators': modes.shape[1], 'modes': m2c.shape[1],
                   'seconds': time.perf_counter() - t0})
    out['kl_basis'] = kl
    torch.cuda.empty_cache()
    return out


def N_variant(wfs):
    from oopao_gb300 import _native as N
    return N.load().oopao_pwfs_get_variant(wfs.plan.h)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.Q, '--format=csv,noheader,nounits',
                 '-lms', '200'], stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(',')]
                if len(f) >= 9:
                    rows.append(f)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unavailable'], 'samples': 0}
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == 'active'})
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows)}


def load_peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        d = json.load(open(p))
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def load_traffic(kernel):
    """DRAM bytes per (mode, point) unit from a committed ncu summary, or None."""
    p = os.path.join(ROOT, 'profiles', 'traffic.json')
    try:
        d = json.load(open(p))
        return d[kernel]
    except Exception:
        return None


def kernel_bytes(kernel, res, n, cam, units, items, launches):
    """Algorithmic (compulsory) DRAM bytes of a kernel summed over the timed
    region: `units` (item, modulation point) pairs over `items` frames in
    `launches` launches.  Per unit (complex64 intermediates): the row pass
    writes res x N, the column pass reads res x N and writes N x N, the
    row-inverse pass reads N x N; per item: the OPD (4 res^2) and the camera
    frame (4 cam^2); per launch: tables (amplitude 4 res^2, mask 8 N^2)."""
    if kernel == 'pwfs_rows_fwd':
        return units * 8 * res * n + items * 4 * res * res + launches * 4 * res * res
    if kernel == 'pwfs_cols':
        return units * (8 * res * n + 8 * n * n) + launches * 8 * n * n
    if kernel == 'pwfs_rows_inv':
        return units * 8 * n * n + items * 4 * cam * cam
    return items * 4 * cam * cam


KERNELS = ['pwfs_rows_fwd', 'pwfs_cols', 'pwfs_rows_inv', 'pwfs_bin']
# stages of the two-pass path (masks that factorise per axis): 0 field + filtered
# rows, 1 filtered columns with the |G|^2 sum and binning, 3 fixed-order slot sum
KERNELS_SEP = ['pwfs_srows', 'pwfs_scols', 'unused', 'pwfs_reduce_binned']


def kernel_bytes_sep(kernel, res, n, cam, ng, units, items, ksplit):
    """Algorithmic DRAM bytes of the two-pass kernels over the timed region:
    `units` (item, point) pairs, `items` frames, `ng` row-transform groups.
    Row stage: OPD in (4 res^2), field out and back in (16 res^2), filtered
    rows out (8 res N per group).  Column stage: the filtered rows of a point
    read once per point (8 res N) and binned slot partials out (4 cam^2 per
    slot).  Reduce: the slot partials in, the frame out."""
    if kernel == 'pwfs_srows':
        return items * (4 * res * res + 16 * res * res + ng * 8 * res * n)
    if kernel == 'pwfs_scols':
        return units * 8 * res * n + items * ksplit * 4 * cam * cam
    return items * (ksplit + 1) * 4 * cam * cam


def fft_flops(kernel, res, n, ng, units, items):
    """Nominal FFT flops (5 N log2 N per length-N complex transform) of the
    two-pass kernels: per group and pupil row a forward and an inverse row
    transform; per (item, point) N forward and N inverse column transforms."""
    per = 5.0 * n * np.log2(n)
    if kernel == 'pwfs_srows':
        return items * ng * res * 2 * per
    if kernel == 'pwfs_scols':
        return units * n * 2 * per
    return 0.0


def fp32_peak_tflops(sm_mhz):
    """FP32 CUDA-core peak at the sampled SM clock: SMs x 128 lanes x 2 flops."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12


def headline_config():
    """`config` of the headline JSON line, the same for both arms."""
    return {'workload': WORKLOAD, 'modes': NMODES, 'frames_per_im': 2 * NMODES, 'modulation_points': NTHETA,
            'fft_grid': 264, 'camera': 44, 'stroke_m': STROKE,
            'basis': "the reference's KL basis of the 21x21 DM (tests/golden/kl_c1.npz), first %d modes" % NMODES,
            'l2': 'intermediates (>=2.4 GB per launch) exceed L2; no flush needed'}


def cpu_oracle_rate(m2c, budget_s=12.0, min_frames=4, threads=None, modes_per_step=None, seed=7):
    """Oracle (float64 numpy/scipy port of the reference) push-pull frames/s on
    the host cores for a bounded sample of the workload: seeded columns of
    the same M2C, two frames each.  Either runs for `budget_s` seconds or, with
    `modes_per_step`, exactly that many modes.  Returns
    (frames/s, frames, seconds, threads)."""
    from oracle import pwfs_oracle as O
    threads = threads or os.cpu_count() or 1
    inten = O.source_intensity(O.telescope_pupil(RES), O.n_photon('V0', 8), 1e-3, 8.0)
    wfs = O.build_pyramid(RES, NSUB, MOD, 0.5, inten, n_theta_user=NTHETA, workers=threads)
    modes = O.dm_modes(RES, 8.0, NSUB)
    pupil = O.telescope_pupil(RES)
    lam = O.PHOTOMETRY['V0'][0]
    order = np.random.default_rng(seed).permutation(m2c.shape[1])
    frames, t0, m = 0, time.perf_counter(), 0
    while True:
        c = int(order[m % len(order)])
        O.interaction_matrix(wfs, modes, m2c[:, c:c + 1], STROKE, lam, pupil, single_pass=False,
                             workers=threads)
        frames += 2
        m += 1
        el = time.perf_counter() - t0
        if modes_per_step is not None:
            if m >= modes_per_step:
                break
        elif frames >= min_frames and el >= budget_s:
            break
    return frames / el, frames, el, threads


REF_MODES_PER_STEP = 8


def run_reference(args):
    """Reference arm: the float64 oracle port of the reference's push-pull
    interaction-matrix loop on the host cores.  One step = REF_MODES_PER_STEP
    seeded modes of the same 300-mode KL basis (2 frames each), timed whole;
    `value` = frames over the K timed steps / their wall time."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    m2c = reference_kl_c1(NMODES)
    times, frames = [], 0
    for i in range(args.warmup + args.steps):
        r, fr, el, thr = cpu_oracle_rate(m2c, threads=threads, modes_per_step=REF_MODES_PER_STEP, seed=100 + i)
        if i >= args.warmup:
            times.append(el)
            frames += fr
    total = sum(times)
    v = frames / total
    line = {
        'metric': 'PWFS frames/s (batched IM build)', 'value': v, 'unit': 'frames/s',
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1000.0 * total / args.steps, 'frames_per_step': 2 * REF_MODES_PER_STEP,
        'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference',
        'config': headline_config(),
        'cpu_baseline': {'value': v, 'unit': 'frames/s', 'cores': threads, 'kind': 'port',
                         'sample': 'per step: %d seeded push-pull modes (%d frames) of the %d-mode basis, '
                                   'float64 oracle, scipy.fft workers=%d'
                                   % (REF_MODES_PER_STEP, 2 * REF_MODES_PER_STEP, NMODES, threads)},
        'e2e': {'value': v, 'unit': 'frames/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group('nccl')
    from oopao_gb300 import _native as N
    from oopao_gb300.calibration import InteractionMatrix, _signals_batched
    # every mode of one sign in one launch sequence (measured: 68.5k frames/s
    # against 66.6k in chunks of 100)
    tel, ngs, dm, wfs = build_system(local, max_batch=NMODES)
    m2c = reference_kl_c1(NMODES)
    dev = wfs._dev
    m2c_dev = torch.as_tensor(m2c.astype(np.float32), device=dev)
    n, cam, k = wfs.resolution, wfs._cam_eff, wfs.nTheta
    plan = wfs.plan
    ksplit = 8 if k >= 8 else k
    scale = 2 * np.pi / ngs.wavelength
    ngs ** tel
    wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())

    def device_step():
        sp_all, sm_all = [], []
        for b0 in range(0, NMODES, wfs.max_batch):
            cb = m2c_dev[:, b0:b0 + wfs.max_batch] * STROKE
            for sgn, acc in ((1.0, sp_all), (-1.0, sm_all)):
                opd = dm.opd_device((cb * sgn).contiguous())
                frame, _ = wfs._measure_frames(opd, scale)
                _, sig = wfs._signals(frame)
                acc.append(sig)
        sp, sm = torch.cat(sp_all), torch.cat(sm_all)
        return (0.5 * (sp - sm) / STROKE).T

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    from oopao_gb300 import autotune
    tune = autotune.tune_pyramid(wfs, batch=wfs.max_batch)
    for _ in range(args.warmup):
        device_step()
    barrier()
    stream = torch.cuda.current_stream()
    N.call('oopao_pwfs_set_profiling', plan.h, 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = N.load().oopao_launch_count()
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            D = device_step()
        e1.record(stream)
        barrier()
    launches = N.load().oopao_launch_count() - n0
    ms_step = e0.elapsed_time(e1) / args.steps
    ms = (N.c_double * 4)()
    cnt = (N.c_int * 4)()
    N.call('oopao_pwfs_profile_read', plan.h, ms, cnt)
    N.call('oopao_pwfs_set_profiling', plan.h, 0)
    clocks = clk.summary()
    if world > 1:
        t = torch.tensor([ms_step], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    frames_step = 2 * NMODES
    value = frames_step * world / (ms_step / 1000.0)

    # ---- roofline of the dominant kernel
    two_pass = N.call('oopao_pwfs_separable', plan.h) == 1
    names = KERNELS_SEP if two_pass else KERNELS
    totals = {names[i]: ms[i] for i in range(4) if cnt[i]}
    top = max(totals, key=totals.get)
    ti = names.index(top)
    items = frames_step * args.steps
    units = items * k
    nl = cnt[ti]
    fp32 = None
    if two_pass:
        info = np.zeros(4, np.int32)
        N.call('oopao_pwfs_pass_info', plan.h, wfs.max_batch, info)
        ng, ks = int(info[1]), int(info[2])
        byts = kernel_bytes_sep(top, RES, n, cam, ng, units, items, ks)
        flops = fft_flops(top, RES, n, ng, units, items)
        sm_mhz = (clocks or {}).get('sm_mhz') or 2070.0
        fpk = fp32_peak_tflops(sm_mhz)
        ach_tf = flops / (totals[top] / 1000.0) / 1e12
        fp32 = {'achieved_tflops': ach_tf, 'peak_tflops': fpk, 'frac': ach_tf / fpk,
                'peak_kind': 'nominal (SMs x 128 FP32 lanes x 2 x sampled SM clock)',
                'flops': 'nominal FFT flops, 5 N log2 N per length-N transform'}
        # the per-point bytes of the three-pass formulation, 8 (2 res N + 2 N^2):
        # the bandwidth a bandwidth-bound three-pass pipeline would need for
        # this frame rate
        three_pass_gbs = units * 8 * (2 * RES * n + 2 * n * n) / (sum(totals.values()) / 1000.0) / 1e9
    else:
        byts = kernel_bytes(top, RES, n, cam, units, items, nl)
    achieved = byts / (totals[top] / 1000.0) / 1e9
    peak, peak_kind = load_peaks()
    variant = int(N_variant(wfs))
    # per-variant capture when the variant's kernel differs (persistent column pass)
    tr = load_traffic('%s@v%d' % (top, variant)) or load_traffic(top)
    traffic = None
    if tr is not None and 'dram_bytes_per_unit' in tr:
        # committed ncu capture: DRAM bytes per (item, point) unit, scaled to one launch here
        traffic = float(tr['dram_bytes_per_unit']) * units / max(nl, 1)
    elif tr is not None and 'dram_bytes_per_group_item' in tr and two_pass:
        # the row pass: per (item, row-transform group)
        traffic = float(tr['dram_bytes_per_group_item']) * items * ng / max(nl, 1)
    share = totals[top] / max(sum(totals.values()), 1e-12)

    # ---- end to end through the public API (host M2C in, host vault out)
    ngs ** tel
    for _ in range(max(1, args.warmup // 2)):
        InteractionMatrix(ngs, tel, dm, wfs, m2c, STROKE, single_pass=False, nTrunc=NTRUNC)
    barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, args.steps // 2)
    for _ in range(e2e_steps):
        calib = InteractionMatrix(ngs, tel, dm, wfs, m2c, STROKE, single_pass=False, nTrunc=NTRUNC)
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    ns = wfs.nSignal
    # host -> device: commands (float32), D for the float64 vault
    h2d = m2c.size * 4 + ns * NMODES * 8
    # device -> host: D (float64), the vault's U, s, V, D, M, Mtrunc, Dtrunc and its condition check
    d2h = ns * NMODES * 8 + (5 * ns * NMODES + NMODES + NMODES * NMODES + 2) * 8
    e2e = {'value': frames_step * world / e2e_s, 'unit': 'frames/s', 'h2d_bytes_per_step': int(h2d),
           'd2h_bytes_per_step': int(d2h), 'im_build_ms': e2e_s * 1000.0,
           'api': 'InteractionMatrix(..., single_pass=False, nTrunc=20)'}

    # ---- reported CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        r, frames, el, thr = cpu_oracle_rate(m2c)
        cpu = {'value': r, 'unit': 'frames/s', 'cores': thr, 'kind': 'port',
               'sample': '%d push-pull frames (%d seeded modes of the same basis) in %.1f s, float64 oracle, '
                         'scipy.fft workers=%d' % (frames, frames // 2, el, thr)}

    # accuracy of this step's IM against the float64 oracle on seeded columns
    err = None
    if rank == 0 and not args.no_cpu:
        cols = err_columns(NMODES)
        Dref, t_or = oracle_im(RES, NSUB, MOD, NTHETA, m2c, STROKE, cols)
        err = {'rel_fro': rel_fro(D[:, cols].double().cpu().numpy(), Dref), 'columns': cols,
               'oracle_seconds': t_or}

    extra = {}
    if rank == 0 and world == 1 and not args.no_extra:
        extra['im_c1_300'] = im_comparison(tel, ngs, dm, wfs, m2c, n_per_mode=30)
        tel3, ngs3, dm3, wfs3 = build_system(0, 240, 40, 5, 96, max_batch=16)
        autotune.tune_pyramid(wfs3, batch=16)
        m2c3 = kl_like_basis(dm3.modes, tel3.pupil, 1000, r0=0.12, L0=30.0)
        extra['im_c3_1000'] = im_comparison(tel3, ngs3, dm3, wfs3, m2c3, n_per_mode=10)
        del tel3, ngs3, dm3, wfs3
        extra['cl_step'] = cl_rate()
        extra['cl_strehl_20x20'] = cl_strehl()
        extra['config4_differentiable'] = config4_leg()
        extra['large_80x80'] = large_config()
        try:
            pk = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
        except Exception:
            pk = {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0}
        extra['dm_projection'] = dm_projection(pk)
        extra['gsc'] = gsc_leg(pk)
        extra['next_rows'] = next_rows_leg()
        extra['cl_gsc_20x20'] = cl_gsc()

    if rank == 0:
        line = {
            'metric': 'PWFS frames/s (batched IM build)', 'value': value, 'unit': 'frames/s',
            'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_step,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded KL basis, Gaussian IFs)',
            'frames_per_step': frames_step, 'batch_per_launch': wfs.max_batch,
            'config': headline_config(),
            'im_rel_fro_err_vs_fp64_oracle': err,
            'roofline': {'bound': 'hbm', 'kernel': top, 'variant': variant, 'two_pass': two_pass,
                         'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                         'peak_kind': peak_kind, 'traffic': traffic, 'kernel_share': share,
                         'kernel_ms': totals,
                         'launches': {names[i]: cnt[i] for i in range(4) if cnt[i]},
                         'fp32': fp32,
                         'limiter': ('FP32 issue: the column pass moves %.0f%% of the HBM peak and runs its FFTs '
                                     'from registers and shared memory' % (100 * achieved / peak))
                         if two_pass else None,
                         'three_pass_equivalent_gbs': three_pass_gbs if two_pass else None},
            'e2e': e2e,
            'gpu_launches': int(launches),
            'clocks': clocks,
            'cpu_baseline': cpu,
            'autotune': {'variant': tune['variant'], 'ms_per_variant': tune['ms'],
                         'two_pass': tune.get('two_pass')},
        }
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


CASES = {'pwfs20': (120, 20, 3, 48), 'pwfs40': (240, 40, 5, 96)}


def run_case(args):
    """Small fixed workload for profiler captures (prints one JSON line, not a
    bench line).  pwfs20 / pwfs40: `--reps` batched PWFS measurements of
    `--batch` seeded random OPDs on the 20x20 / 40x40 configuration with the
    autotuned kernel variant; dm40: `--reps` BF16 tensor-core and FP32 IF
    projections of `--batch` coefficient vectors on the 40x40 DM.  The
    measured loop is the NVTX range 'case' (ncu --nvtx --nvtx-include case/)."""
    import torch
    from oopao_gb300 import _native as N
    from oopao_gb300 import autotune
    torch.cuda.set_device(0)
    g = torch.Generator(device='cuda').manual_seed(0)
    t0 = time.perf_counter()
    if args.case in CASES:
        res, nsub, mod, nth = CASES[args.case]
        tel, ngs, dm, wfs = build_system(0, res, nsub, mod, nth, max_batch=args.batch)
        if args.variant >= 0:
            N.call('oopao_pwfs_set_variant', wfs.plan.h, args.variant)
            tune = {'variant': args.variant}
        else:
            tune = autotune.tune_pyramid(wfs, batch=args.batch)
        if args.three_pass:
            N.call('oopao_pwfs_set_separable', wfs.plan.h, 0)
        ngs ** tel
        wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
        opd = torch.randn((args.batch, res, res), device='cuda', generator=g) * 50e-9
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push('case')
        for _ in range(args.reps):
            frame, _ = wfs._measure_frames(opd, 2 * np.pi / ngs.wavelength)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out = {'case': args.case, 'batch': args.batch, 'reps': args.reps, 'variant': tune['variant'],
               'two_pass': N.call('oopao_pwfs_separable', wfs.plan.h) == 1,
               'frame_sum': float(frame.double().sum().item())}
    elif args.case == 'dm40':
        tel, ngs, dm, wfs = None, None, None, None
        with _quiet():
            import oopao_gb300 as og
            tel = og.Telescope(resolution=240, diameter=8.0, samplingTime=1e-3)
            dm = og.DeformableMirror(tel, nSubap=40, if_dtype='bf16')
        # profile the dense tensor-core GEMM, not the separable default
        dm.separable_projection = False
        c = torch.randn((dm.nValidAct, args.batch), device='cuda', generator=g) * 50e-9
        o = torch.empty((args.batch, 240, 240), device='cuda')
        # the same IFs in FP32 for the FP32-accuracy tensor-core path
        pad32 = (dm.nValidAct + 31) // 32 * 32
        m2 = torch.empty((2, 240 * 240, pad32), device='cuda')
        N.call('oopao_dm_modes_tf32x2', dm._modes_t, dm.nValidAct, 240 * 240, pad32, m2, N.stream_handle())
        nbt = N.load().oopao_dm_tf32_workspace_bytes(pad32, args.batch)
        wst = torch.zeros(nbt, dtype=torch.uint8, device='cuda')
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push('case')
        for _ in range(args.reps):
            dm.opd_device(c, out=o)
            N.call('oopao_dm_opd_acc_f32', dm._modes_t, c, dm.nValidAct, 240 * 240, args.batch, 1.0, None, o,
                   N.stream_handle())
            N.call('oopao_dm_opd_tf32x3', m2, pad32, c, dm.nValidAct, 240 * 240, args.batch, 1.0, None, o, wst, nbt,
                   N.stream_handle())
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out = {'case': args.case, 'batch': args.batch, 'reps': args.reps, 'tc_status': dm.tensor_core_status(),
               'tf32_status': int(wst[:4].view(torch.int32).item())}
    elif args.case == 'jvp40':
        # tangent passes of the 40x40 sensor: --batch modal tangents at the
        # flat operating point through oopao_pwfs_jvp (the storing column
        # pass of G_k, then the tangent row and column passes of the batch)
        from oopao_gb300 import autodiff as AD
        res, nsub, mod, nth = CASES['pwfs40']
        tel, ngs, dm, wfs = build_system(0, res, nsub, mod, nth, max_batch=args.batch)
        ngs ** tel
        wfs.plan.set_amplitude(ngs.intensity, wfs._amplitude_key())
        c = torch.randn((dm.nValidAct, args.batch), device='cuda', generator=g) * 1e-8
        dopd = dm.opd_device(c)
        opd0 = torch.zeros((1, res, res), device='cuda')
        AD.frame_jvp(wfs, opd0, dopd)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push('case')
        for _ in range(args.reps):
            df = AD.frame_jvp(wfs, opd0, dopd)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out = {'case': args.case, 'batch': args.batch, 'reps': args.reps,
               'dframe_norm': float(df.double().norm().item())}
    elif args.case == 'bioedge20':
        # Bi-O Edge 20x20 (120 px, N=264, 48 points, four knife-edge masks):
        # --reps measurements of --batch seeded OPDs through the one-axis path
        import oopao_gb300 as og
        with _quiet():
            tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
            ngs = og.Source(optBand='V0', magnitude=8)
            ngs * tel
            wfs = og.BioEdge(nSubap=20, telescope=tel, modulation=3, lightRatio=0.5, nTheta_user_defined=48,
                             max_batch=args.batch)
        ngs ** tel
        opd = torch.randn((args.batch, 120, 120), device='cuda', generator=g) * 50e-9
        scale = 2 * np.pi / ngs.wavelength
        frame, _ = wfs._measure_frames(opd, scale)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push('case')
        for _ in range(args.reps):
            frame, _ = wfs._measure_frames(opd, scale)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out = {'case': args.case, 'batch': args.batch, 'reps': args.reps,
               'path': N.call('oopao_pwfs_separable', wfs.plan.h), 'frame_sum': float(frame.double().sum().item())}
    elif args.case == 'clgsc':
        out = {'case': args.case, 'cl_gsc_20x20': cl_gsc()}
    elif args.case == 'cl':
        out = {'case': args.case, 'cl_step': cl_rate()}
    elif args.case == 'c5':
        out = {'case': args.case, 'large_80x80': large_config()}
    elif args.case == 'c4':
        out = {'case': args.case, 'config4_differentiable': config4_leg()}
    elif args.case == 'dmproj':
        try:
            pk = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
        except Exception:
            pk = {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0}
        out = {'case': args.case, 'dm_projection': dm_projection(pk)}
    elif args.case == 'next':
        out = {'case': args.case, 'next_rows': next_rows_leg()}
    elif args.case == 'gsc':
        hbm, _ = load_peaks()
        out = {'case': args.case, 'gsc': gsc_leg({'hbm_gbs': hbm})}
    else:
        raise SystemExit('unknown case %s' % args.case)
    out['seconds'] = time.perf_counter() - t0
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline and accuracy legs')
    ap.add_argument('--no-extra', action='store_true',
                    help='skip the interaction-matrix comparisons and the closed-loop rate')
    ap.add_argument('--case', default=None, help='run a small profiling workload (%s, dm40, jvp40, bioedge20, gsc, next, clgsc, cl, c4, c5, dmproj) instead'
                    % ', '.join(CASES))
    ap.add_argument('--batch', type=int, default=16)
    ap.add_argument('--reps', type=int, default=3)
    ap.add_argument('--variant', type=int, default=-1, help='kernel variant for --case (-1: autotune)')
    ap.add_argument('--three-pass', action='store_true',
                    help='pwfs20/pwfs40 cases: force the three-pass propagation (masks that do not factorise)')
    args = ap.parse_args()
    if args.case:
        import __graft_entry__
        __graft_entry__.build()
        run_case(args)
    elif args.impl == 'reference':
        run_reference(args)
    else:
        import __graft_entry__
        __graft_entry__.build()
        run_ours(args)


if __name__ == '__main__':
    main()
