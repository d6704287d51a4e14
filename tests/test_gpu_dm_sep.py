"""Separable DM projection (Gaussian IFs on a Cartesian grid factorise as
gx(x) gy(y)) against the float64 dense product modes @ coefs, for single
shapes, small and large batches, an incoming OPD (the relay's accumulate),
flips and mis-registrations.  FP32 path: relative L2 <= 1e-6."""
import contextlib
import io

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dm(res=120, nsub=20, **kw):
    import oopao_gb300 as og
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=res, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=nsub, mechCoupling=0.35, **kw)
    return tel, dm


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


@pytest.mark.parametrize('kw', [dict(), dict(flip_lr=True), dict(flip=True, sign=-1), dict(if_dtype='bf16'),
                                dict(actuator_selection=0.2)],
                         ids=['plain', 'flip_lr', 'flip_sign', 'bf16_ifs', 'std_selection'])
@pytest.mark.parametrize('batch', [1, 3, 300])
def test_separable_projection(kw, batch):
    tel, dm = _dm(**kw)
    assert dm.projection_path() == 'separable'
    # factorising IFs take the separable projection at every batch (the
    # tiled FP32 GEMM beats the BF16 tensor-core one); a BF16-IF mirror keeps
    # the tensor-core path for batches above its cut-over
    path = dm.projection_path(batch)
    assert path == ('bf16' if kw.get('if_dtype') == 'bf16' and batch > dm.separable_max_batch else 'separable')
    tol = 2e-3 if path == 'bf16' else 1e-6
    rng = np.random.default_rng(batch)
    coefs = rng.standard_normal((dm.nValidAct, batch)) * 1e-7
    ref = (dm.modes @ coefs).T.reshape(batch, tel.resolution, tel.resolution)
    c = torch.as_tensor(coefs, dtype=torch.float32, device='cuda')
    out = dm.opd_device(c).cpu().double().numpy()
    assert _rel(out, ref) < tol
    base = torch.as_tensor(rng.standard_normal((batch, tel.resolution, tel.resolution)) * 1e-7,
                           dtype=torch.float32, device='cuda')
    out2 = dm.opd_device(c, base=base).cpu().double().numpy()
    assert _rel(out2, ref + base.cpu().double().numpy()) < tol


def test_dense_and_separable_agree_through_the_relay():
    import oopao_gb300 as og
    tel, dm = _dm()
    coefs = np.random.default_rng(5).standard_normal(dm.nValidAct) * 1e-7
    dm.coefs = coefs
    a = np.array(dm.OPD)
    dm.separable_projection = False
    assert dm.projection_path() == 'fp32'
    dm.coefs = coefs
    b = np.array(dm.OPD)
    assert _rel(a, b) < 1e-6
    assert _rel(a, (dm.modes @ coefs).reshape(tel.resolution, tel.resolution)) < 1e-6


@pytest.mark.parametrize('mr, path', [(dict(shiftX=0.05, shiftY=-0.1, radialScaling=0.03), 'separable'),
                                      (dict(rotationAngle=1.0), 'fp32'),
                                      (dict(anamorphosisAngle=15.0, tangentialScaling=0.02), 'fp32')])
def test_misregistered_projection_path(mr, path):
    import oopao_gb300 as og
    full = dict(rotationAngle=0.0, shiftX=0.0, shiftY=0.0, anamorphosisAngle=0.0, tangentialScaling=0.0,
                radialScaling=0.0)
    full.update(mr)
    tel, dm = _dm(misReg=og.MisRegistration(full))
    assert dm.projection_path() == path
    coefs = np.random.default_rng(2).standard_normal((dm.nValidAct, 4)) * 1e-7
    out = dm.opd_device(torch.as_tensor(coefs, dtype=torch.float32, device='cuda')).cpu().double().numpy()
    ref = (dm.modes @ coefs).T.reshape(4, tel.resolution, tel.resolution)
    assert _rel(out, ref) < 1e-6


@pytest.mark.parametrize('nx, ny, batch', [(12, 9, 2), (150, 60, 2), (300, 70, 3), (150, 60, 40), (12, 9, 17)],
                         ids=['one_launch', 'one_launch_96k', 'two_launches', 'tiled_96k', 'tiled'])
def test_separable_cabi(nx, ny, batch):
    """oopao_dm_opd_sep_f32 on synthetic factors: a grid whose coefficient map
    fits in shared memory (one launch) and one that does not (two), with
    empty grid cells, against the float64 product."""
    from oopao_gb300 import _native as N
    res, n_act = 64, None
    rng = np.random.default_rng(nx)
    gx = rng.standard_normal((nx, res)).astype(np.float32)
    gy = rng.standard_normal((ny, res)).astype(np.float32)
    cells = np.full(nx * ny, -1, np.int32)
    used = rng.choice(nx * ny, size=(nx * ny) * 3 // 4, replace=False)
    n_act = len(used)
    cells[used] = rng.permutation(n_act).astype(np.int32)
    coefs = rng.standard_normal((n_act, batch)).astype(np.float32)
    C = np.zeros((batch, ny * nx))
    C[:, used] = coefs[cells[used]].T
    ref = np.einsum('jy,bji,ix->byx', gy.astype(np.float64), C.reshape(batch, ny, nx), gx.astype(np.float64))
    dev = lambda a: torch.as_tensor(a, device='cuda')
    out = torch.empty((batch, res, res), dtype=torch.float32, device='cuda')
    nb = N.load().oopao_dm_sep_workspace_bytes(ny, res, batch)
    ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
    g_x, g_y, c_d, k_d = dev(gx), dev(gy), dev(cells), dev(coefs)
    N.call('oopao_dm_opd_sep_f32', g_x, g_y, c_d, nx, ny, k_d, n_act, res, batch, 1.0, None, out, ws, nb,
           N.stream_handle())
    assert _rel(out.cpu().double().numpy(), ref) < 1e-5
