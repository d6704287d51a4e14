"""The autotuner: its choices change launch shapes only, never results.

* tune_pyramid on a factorising mask times the two-pass plans and slot
  counts and leaves the sensor on the winner; frames before and after agree
  to float32 round-off (<= 2e-6 relative L2) and the cached choice is
  re-applied without timing.
* tune_dm picks the separable / BF16 tensor-core cut-over and the GEMM's
  batch tile per batch; projections before and after agree within the BF16
  IF rounding (<= 2e-3 relative L2 against float64)."""
import contextlib
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


@pytest.fixture
def cache(tmp_path, monkeypatch):
    p = tmp_path / 'autotune.json'
    monkeypatch.setenv('OOPAO_GB300_AUTOTUNE_CACHE', str(p))
    return p


def test_tune_pyramid_two_pass(cache):
    import torch
    import oopao_gb300 as og
    from oopao_gb300 import _native as N
    from oopao_gb300 import autotune
    with _quiet():
        tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        wfs = og.Pyramid(nSubap=20, telescope=tel, modulation=3, lightRatio=0.5, nTheta_user_defined=48,
                         max_batch=8)
    ngs ** tel
    scale = 2 * np.pi / ngs.wavelength
    opd = torch.randn((8, 120, 120), device='cuda', generator=torch.Generator(device='cuda').manual_seed(1)) * 5e-8
    f0, _ = wfs._measure_frames(opd, scale)
    f0 = f0.double().cpu()
    entry = autotune.tune_pyramid(wfs, batch=8)
    assert 'two_pass' in entry and entry['two_pass']['plan'] >= 1
    assert N.call('oopao_pwfs_separable', wfs.plan.h) == 1
    f1, _ = wfs._measure_frames(opd, scale)
    assert float((f1.double().cpu() - f0).norm() / f0.norm()) < 2e-6
    assert cache.exists()
    again = autotune.tune_pyramid(wfs, batch=8)
    assert again['two_pass'] == entry['two_pass']


def test_tune_dm(cache):
    import torch
    import oopao_gb300 as og
    from oopao_gb300 import autotune
    with _quiet():
        tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
        dm = og.DeformableMirror(tel, nSubap=20, mechCoupling=0.35, if_dtype='bf16')
    ms = autotune.tune_dm(dm, batches=(1, 16, 64))
    assert set(ms) == {1, 16, 64}
    assert all(t in (0, 64, 128) for _, t in dm.tc_tile_rule)
    modes = np.asarray(dm.modes)
    for B in (1, 16, 40, 64, 100):
        c = np.random.default_rng(B).standard_normal((dm.nValidAct, B)) * 1e-8
        got = dm.opd_device(torch.as_tensor(c, dtype=torch.float32, device='cuda')).double().cpu().numpy()
        ref = (modes @ c).T.reshape(B, 120, 120)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 2e-3, (B, dm.projection_path(B))


def test_tune_dm_tf32_cut_over(cache):
    """FP32 IFs that do not factorise (a rotated grid): the tuner times the
    CUDA-core FP32 GEMM against the FP32-accuracy tensor-core GEMM and sets
    the batch from which the latter runs; every batch stays at FP32 accuracy."""
    import torch
    import oopao_gb300 as og
    from oopao_gb300 import autotune
    with _quiet():
        tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
        mr = og.MisRegistration({'rotationAngle': 2.0, 'shiftX': 0.0, 'shiftY': 0.0, 'anamorphosisAngle': 0,
                                 'tangentialScaling': 0, 'radialScaling': 0})
        dm = og.DeformableMirror(tel, nSubap=20, misReg=mr)
    ms = autotune.tune_dm(dm, batches=(1, 16, 64, 300))
    assert all({'fp32', 'tf32'} <= set(r) for r in ms.values())
    assert dm.tf32_min_batch is None or dm.tf32_min_batch in (1, 16, 64, 300)
    modes = np.asarray(dm.modes)
    for B in (1, 16, 300):
        c = np.random.default_rng(B).standard_normal((dm.nValidAct, B)) * 1e-8
        got = dm.opd_device(torch.as_tensor(c, dtype=torch.float32, device='cuda')).double().cpu().numpy()
        ref = (modes @ c).T.reshape(B, 120, 120)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 2e-6, (B, dm.projection_path(B))
