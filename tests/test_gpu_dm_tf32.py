"""FP32-accuracy influence-function projection on the tensor cores (tcgen05
kind::tf32, three products of TF32 values and FP32 remainders).

Through the C ABI against the float64 product of the FP32 operands (relative
L2 <= 2e-6, the FP32 path bound being 1e-5), with and without a base OPD,
across batch tiles (16, 64, 65, 300 columns) and both pixel-tile edges; through
the drop-in DeformableMirror with IFs that do not factorise (a rotated grid),
whose large batches take this path, against the same DM's CUDA-core FP32
path and against float64."""
import contextlib
import io

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def modes():
    return O.dm_modes(120, 8.0, 20)


def _project(modes, coefs, scale, base=None):
    import torch
    from oopao_gb300 import _native as N
    n_pix, n_act = modes.shape
    pad = (n_act + 31) // 32 * 32
    batch = coefs.shape[1]
    mt = torch.as_tensor(np.ascontiguousarray(modes.T, dtype=np.float32), device='cuda')
    m2 = torch.empty((2, n_pix, pad), dtype=torch.float32, device='cuda')
    N.call('oopao_dm_modes_tf32x2', mt, n_act, n_pix, pad, m2, N.stream_handle())
    c = torch.as_tensor(coefs, device='cuda')
    b = None if base is None else torch.as_tensor(base, device='cuda')
    out = torch.full((batch, n_pix), float('nan'), device='cuda')
    nb = N.load().oopao_dm_tf32_workspace_bytes(pad, batch)
    ws = torch.zeros(nb, dtype=torch.uint8, device='cuda')
    N.call('oopao_dm_opd_tf32x3', m2, pad, c, n_act, n_pix, batch, scale, b, out, ws, nb, N.stream_handle())
    torch.cuda.synchronize()
    assert int(ws[:4].view(torch.int32).item()) == 0
    return out.double().cpu().numpy(), m2


@pytest.mark.parametrize('batch', [16, 64, 65, 300])
def test_tf32x3_projection(modes, batch):
    rng = np.random.default_rng(100 + batch)
    coefs = rng.standard_normal((modes.shape[1], batch)).astype(np.float32)
    got, m2 = _project(modes, coefs, 0.5)
    assert np.isfinite(got).all()
    # the split is exact: hi + lo reproduces the FP32 IFs
    m = m2.double().cpu().numpy()
    np.testing.assert_array_equal((m[0] + m[1])[:, :modes.shape[1]], modes.astype(np.float32))
    exact = (modes.astype(np.float32).astype(np.float64) @ coefs.astype(np.float64)).T * 0.5
    assert O.rel_l2(got, exact) < 2e-6


def test_tf32x3_projection_with_base(modes):
    rng = np.random.default_rng(7)
    coefs = rng.standard_normal((modes.shape[1], 130)).astype(np.float32)
    base = rng.standard_normal((130, modes.shape[0])).astype(np.float32)
    got, _ = _project(modes, coefs, 1.0, base)
    exact = (modes.astype(np.float32).astype(np.float64) @ coefs.astype(np.float64)).T + base
    assert O.rel_l2(got, exact) < 2e-6


def test_rotated_dm_large_batch_on_tensor_cores():
    import torch
    import oopao_gb300 as og
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
        mr = og.MisRegistration({'rotationAngle': 2.0, 'shiftX': 0.0, 'shiftY': 0.0, 'anamorphosisAngle': 0,
                                 'tangentialScaling': 0, 'radialScaling': 0})
        dm = og.DeformableMirror(tel, nSubap=20, misReg=mr)
    assert dm.projection_path(1) == 'fp32' and dm.projection_path(300) == 'tf32'
    rng = np.random.default_rng(3)
    c = torch.as_tensor(rng.standard_normal((dm.nValidAct, 300)).astype(np.float32) * 1e-7, device='cuda')
    tc = dm.opd_device(c).double().cpu().numpy()
    assert dm.tensor_core_status() == 0
    dm.tf32_min_batch = None
    assert dm.projection_path(300) == 'fp32'
    cuda_cores = dm.opd_device(c).double().cpu().numpy()
    exact = (np.asarray(dm.modes, dtype=np.float32).astype(np.float64) @ c.double().cpu().numpy()).T
    exact = exact.reshape(tc.shape)
    assert O.rel_l2(tc, exact) < 2e-6 and O.rel_l2(cuda_cores, exact) < 2e-6
    assert O.rel_l2(tc, cuda_cores) < 2e-6
