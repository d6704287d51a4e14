"""GainSensingCamera on the GPU against golden vectors made by the unmodified
reference (cases gsc_*) and against the float64 oracle at the 20x20 pyramid
size (N = 264).  FP32 path bound: relative L2 <= 1e-5 for the impulse
responses, the sensitivities and the optical gains."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from oracle import gsc_oracle as G
from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
TOL = 1e-5


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.fixture(scope='module', params=['gsc_tiny', 'gsc_small'])
def golden(request):
    z = np.load(os.path.join(HERE, request.param + '.npz'))
    return {k: z[k] for k in z.files}


def test_against_golden_frames(golden):
    from oopao_gb300 import GainSensingCamera
    d = golden
    gsc = GainSensingCamera(d['mask'], d['basis'])
    assert gsc.tag == 'GSC' and gsc.n_modes == d['basis'].shape[-1]
    gsc.calibration(d['calib_frame'])
    assert gsc.calibration_ready
    np.testing.assert_array_equal(gsc.og, 1.0)
    assert rel(gsc.IR_calib, d['ir_calib']) < TOL
    assert rel(gsc.sensi_calib, d['sensi_calib']) < TOL
    n = d['mask'].shape[0]
    assert rel(gsc.basis_product, G.basis_product(d['basis'], n).real) < TOL
    gsc.compute_optical_gains(d['sky_frame'])
    assert rel(gsc.IR_sky, d['ir_sky']) < TOL
    assert rel(gsc.og, d['og']) < TOL
    gsc.reset_calibration()
    assert not gsc.calibration_ready
    np.testing.assert_array_equal(gsc.og, 1.0)


def test_tutorial_flow(golden):
    """The reference tutorial's sequence with the drop-in objects: basis from
    tel.OPD of a DM mode set, full-resolution focal-plane camera, camera * gsc
    to calibrate and then to compute the gains."""
    import oopao_gb300 as og
    d = golden
    p = json.loads(str(d['params']))
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=p['res'], diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=p['n_subap'], mechCoupling=0.35)
        wfs = og.Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'],
                         lightRatio=p['light_ratio'])
    dm.coefs = d['m2c']
    ngs ** tel * dm
    basis = np.array(tel.OPD)
    assert basis.shape == d['basis'].shape
    assert rel(basis, d['basis']) < 1e-6
    dm.coefs = 0
    gsc = og.GainSensingCamera(mask=wfs.mask, basis=basis)
    wfs.focal_plane_camera.resolution = wfs.nRes
    ngs ** tel * wfs
    wfs * wfs.focal_plane_camera
    assert rel(wfs.focal_plane_camera.frame, d['calib_frame']) < TOL
    wfs.focal_plane_camera * gsc
    assert gsc.calibration_ready and gsc.detector_properties is not None
    ngs ** tel
    tel.OPD_no_pupil = d['sky_opd']
    tel * wfs
    wfs * wfs.focal_plane_camera
    assert rel(wfs.focal_plane_camera.frame, d['sky_frame']) < TOL
    wfs.focal_plane_camera * gsc
    assert rel(gsc.og, d['og']) < TOL


@pytest.fixture(scope='module')
def c1_case():
    """20x20 pyramid mask (N = 264), 48 random smooth modes on 120 px, a
    calibration frame and five other positive frames."""
    geom = O.pyramid_geometry(120, 20, 2)
    n = geom.N
    rng = np.random.default_rng(11)
    k = np.fft.fftfreq(120)
    kx, ky = np.meshgrid(k, k)
    filt = 1.0 / (1.0 + (kx ** 2 + ky ** 2) * 400.0)
    basis = np.stack([np.real(np.fft.ifft2(filt * np.fft.fft2(rng.standard_normal((120, 120)))))
                      for _ in range(48)], axis=-1) * 1e-7
    r = np.hypot(*np.meshgrid(np.arange(n) - n / 2, np.arange(n) - n / 2))
    base = np.exp(-(r / 12.0) ** 2) + 1e-3
    frames = np.stack([base * rng.uniform(0.5, 1.5, (n, n)) for _ in range(6)])
    return np.asarray(geom.mask, dtype=np.complex64), basis, frames


def test_batch_against_oracle(c1_case):
    from oopao_gb300 import GainSensingCamera
    mask, basis, frames = c1_case
    gsc = GainSensingCamera(mask, basis)
    gsc.calibration(frames[0])
    ref = G.OracleGSC(mask, basis)
    ref.calibration(frames[0])
    assert rel(gsc.sensi_calib, ref.sensi_calib) < TOL
    gsc.compute_optical_gains(frames[1:])
    assert gsc.og_batch.shape == (5, 48)
    for b in range(5):
        ref.compute_optical_gains(frames[1 + b])
        assert rel(gsc.og_batch[b], ref.og) < TOL, b
    # one frame at a time gives the gains of the batch (only the summation
    # order of the contraction differs)
    batch_og = gsc.og_batch.copy()
    gsc.compute_optical_gains(frames[3])
    assert rel(gsc.og, batch_og[2]) < 1e-6


def test_device_frames_stay_on_device(c1_case):
    import torch
    from oopao_gb300 import GainSensingCamera
    mask, basis, frames = c1_case
    gsc = GainSensingCamera(mask, basis)
    f = torch.as_tensor(frames.astype(np.float32), device='cuda')
    gsc.calibration(f[0])
    gsc.compute_optical_gains(f[1:3])
    assert gsc.device_og.is_cuda and gsc.device_og.shape == (2, 48)
    ref = G.OracleGSC(mask, basis)
    ref.calibration(frames[0].astype(np.float32).astype(np.float64))
    ref.compute_optical_gains(frames[2].astype(np.float32).astype(np.float64))
    assert rel(gsc.og, ref.og) < TOL


def test_errors(c1_case):
    from oopao_gb300 import GainSensingCamera
    from oopao_gb300.tools import OopaoError
    mask, basis, frames = c1_case
    gsc = GainSensingCamera(mask, basis)
    with pytest.raises(OopaoError):
        gsc.compute_optical_gains(frames[1])
    with pytest.raises(OopaoError):
        gsc.calibration(frames[0][:100, :100])
    with pytest.raises(OopaoError):
        GainSensingCamera(mask, basis[:119, :119])
    with pytest.raises(OopaoError):
        GainSensingCamera(mask, np.zeros((300, 300, 2)))
