"""The device camera (oopao_gb300.Detector) against the unmodified reference
Detector (tests/golden/detector_tiny.npz): integration over loop steps, full
well, CCD/CMOS gain, ADC with and without full well, unsigned casts, log
scale, background map and hardware binning, step by step and as one batch;
the noise stages (photon, readout, dark current, EMCCD, background) by their
moments; a pyramid whose camera integrates over two loop steps."""
import contextlib
import io

import numpy as np
import pytest
import torch

from tests.goldens import load

pytestmark = pytest.mark.gpu


def _frames_close(ours, ref, tag):
    """float32 frames against the reference's float64: relative 1e-6, except
    that a quantised pixel whose value sits on an integer edge may truncate
    one level apart."""
    ours = np.asarray(ours, dtype=np.float64)
    assert ours.shape == ref.shape, tag
    diff = np.abs(ours - ref)
    bad = diff > 1e-6 * np.maximum(np.abs(ref), 1.0)
    if bad.any():
        assert diff[bad].max() <= 1.0 + 1e-6 and bad.mean() < 2e-3, (tag, diff.max(), bad.sum())


def test_readout_chain_matches_reference():
    from oopao_gb300.detector import Detector
    g = load('detector_tiny')
    dt = float(g['dt'])
    frames = torch.as_tensor(g['frames'], dtype=torch.float32, device='cuda')
    for tag, kw in g['params']['cases'].items():
        kw = dict(kw)
        if tag == 'log_bg':
            kw['backgroundMap'] = g['bg']
        with contextlib.redirect_stdout(io.StringIO()):
            cam = Detector(12, **kw)
            steps = [cam._integrate_device(frames[i][None], dt=dt, wfs=False)[0] for i in range(frames.shape[0])]
        _frames_close(torch.stack(steps).cpu().numpy(), g[tag], tag + ' step by step')
        with contextlib.redirect_stdout(io.StringIO()):
            cam = Detector(12, **kw)
            batch = cam._integrate_device(frames, dt=dt, wfs=False)
        _frames_close(batch.cpu().numpy(), g[tag], tag + ' batch')
        _frames_close(cam.frame, g[tag][-1], tag + ' frame')
    # the camera never writes into the frames it is given
    np.testing.assert_array_equal(frames.cpu().numpy(), g['frames'].astype(np.float32))


def test_saturation_reports():
    from oopao_gb300.detector import Detector
    g = load('detector_tiny')
    f = torch.as_tensor(g['frames'][:1], dtype=torch.float32, device='cuda')
    with contextlib.redirect_stdout(io.StringIO()) as out:
        cam = Detector(12, FWC=20000)
        cam._integrate_device(f, wfs=False)
    assert 'saturating' in out.getvalue()
    assert cam.saturation == pytest.approx(100 * g['frames'][0].max() / 20000, rel=1e-6)
    assert float(cam.frame.max()) == 20000.0


def _gen(seed):
    return torch.Generator(device='cuda').manual_seed(seed)


def test_noise_moments():
    """Moments of each noise stage over 16 frames of 64 x 64 pixels (65536
    draws): means within 5 standard errors, variances within 5%."""
    from oopao_gb300.detector import Detector
    shape = (16, 64, 64)
    n = np.prod(shape)

    def check(frames, mean, var):
        x = frames.double().cpu().numpy()
        assert abs(x.mean() - mean) < 5 * np.sqrt(var / n), (x.mean(), mean)
        assert abs(x.var() / var - 1) < 0.05, (x.var(), var)

    lam = torch.full(shape, 100.0, device='cuda')
    cam = Detector(64, photonNoise=True)
    cam.generator = _gen(1)
    check(cam._integrate_device(lam, wfs=False), 100.0, 100.0)

    cam = Detector(64, readoutNoise=3.0)
    cam.generator = _gen(2)
    # round(N(0, 9)) adds the rounding's 1/12
    check(cam._integrate_device(torch.zeros(shape, device='cuda'), wfs=False), 0.0, 9.0 + 1 / 12)

    cam = Detector(64, darkCurrent=2000.0, integrationTime=5e-3)
    cam.generator = _gen(3)
    reads = torch.stack([cam._integrate_device(torch.zeros((5, 64, 64), device='cuda'), dt=1e-3, wfs=False)[-1]
                         for _ in range(16)])
    check(reads, 10.0, 10.0)
    assert cam.dark_shot_noise == pytest.approx(np.sqrt(10.0))

    cam = Detector(64, sensor='EMCCD', gain=10)
    cam.generator = _gen(4)
    # Poisson(50) amplified by the gain
    check(cam._integrate_device(torch.full(shape, 50.0, device='cuda'), wfs=False), 500.0, 100 * 50.0)

    cam = Detector(64, backgroundFlux=np.full((64, 64), 20.0))
    cam.backgroundNoise = True
    cam.generator = _gen(5)
    check(cam._integrate_device(torch.full(shape, 7.0, device='cuda'), wfs=False), 27.0, 20.0)

    cam = Detector(64, photonNoise=True, QE=0.5, gain=4)
    cam.generator = _gen(6)
    # QE after the photon draw, gain after the readout: 4 * 0.5 * Poisson(100)
    check(cam._integrate_device(lam, wfs=False), 200.0, 4.0 * 100.0)


def test_pyramid_camera_integrates_two_steps():
    """A pyramid whose camera integrates over two loop steps: after the first
    step the camera still shows the last frame read out, after the second the
    sum of both steps' frames; the signals follow the camera frame."""
    import oopao_gb300 as og
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=24, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=4)
        wfs = og.Pyramid(nSubap=4, telescope=tel, modulation=3, lightRatio=0.5)
    rng = np.random.default_rng(21)
    ca, cb = rng.standard_normal((2, dm.nValidAct)) * 40e-9
    frames = []
    for c in (ca, cb):
        dm.coefs = c
        ngs ** tel * dm * wfs
        frames.append(wfs.cam.frame.copy())
    wfs.cam.integrationTime = 2 * tel.samplingTime
    dm.coefs = ca
    ngs ** tel * dm * wfs
    np.testing.assert_array_equal(wfs.cam.frame, frames[1])
    dm.coefs = cb
    ngs ** tel * dm * wfs
    np.testing.assert_allclose(wfs.cam.frame, frames[0] + frames[1], rtol=1e-6, atol=1e-6 * frames[0].max())
    # the signals are those of the integrated frame
    fsum = torch.as_tensor(frames[0] + frames[1], dtype=torch.float32, device=wfs._dev)[None]
    _, sig = wfs._signals(fsum)
    np.testing.assert_allclose(wfs.signal, sig[0].double().cpu().numpy(), rtol=1e-5, atol=1e-6)


def test_adc_wide_words_against_oracle():
    """32-bit ADC with a full well, and a 32-bit ADC without: the top level
    2^32 - 1 and the unsigned conversion stay in range (no wrap to 0 of the
    saturated pixels), against the float64 oracle."""
    from oopao_gb300.detector import Detector
    from oracle import detector_oracle as D
    g = load('detector_tiny')
    frames = g['frames'][:2]
    for kw in (dict(bits=32, FWC=20000), dict(bits=32), dict(bits=16, FWC=20000, gain=3)):
        with contextlib.redirect_stdout(io.StringIO()):
            cam = Detector(12, **kw)
            got = cam._integrate_device(torch.as_tensor(frames, dtype=torch.float32, device='cuda'), wfs=False)
        ref = np.array([D.readout(f, **kw) for f in frames])
        assert np.abs(got.double().cpu().numpy() - ref).max() <= 1e-6 * np.abs(ref).max() + 1.0, kw
        assert got.min().item() >= 0
