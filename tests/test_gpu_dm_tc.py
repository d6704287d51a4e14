"""BF16 tensor-core (tcgen05) influence-function projection.

Exactness of the MMA pipeline is checked against a float64 product of the
same BF16 operands (BF16 IFs, coefficients as hi + lo BF16 terms; only the
FP32 accumulation differs: <= 1e-5); the BF16 path as a whole against the
float64 projection (<= 2e-3), and the pyramid signal of a BF16 DM against
the FP32 one (<= 2e-3, the BF16 IF path tolerance)."""
import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu


def bf16_round(a):
    import torch
    return torch.as_tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).to(torch.float64).numpy()


def bf16_split(c):
    """hi + lo with hi = bf16(c), lo = bf16(c - hi), as the kernel stores them."""
    c = np.asarray(c, dtype=np.float32)
    hi = bf16_round(c)
    lo = bf16_round(c - hi.astype(np.float32))
    return hi + lo


@pytest.fixture(scope='module')
def modes():
    return O.dm_modes(120, 8.0, 20)


@pytest.mark.parametrize('batch', [1, 3, 64, 65, 300])
def test_tc_projection(modes, batch):
    import torch
    from oopao_gb300 import _native as N
    n_pix, n_act = modes.shape
    n_pad = (n_act + 63) // 64 * 64
    mt = torch.as_tensor(np.ascontiguousarray(modes.T, dtype=np.float32), device='cuda')
    mb = torch.empty((n_pix, n_pad), dtype=torch.bfloat16, device='cuda')
    N.call('oopao_dm_modes_bf16', mt, n_act, n_pix, n_pad, mb, N.stream_handle())
    rng = np.random.default_rng(batch)
    coefs = rng.standard_normal((n_act, batch)).astype(np.float32)
    c = torch.as_tensor(coefs, device='cuda')
    out = torch.full((batch, n_pix), float('nan'), device='cuda')
    nb = N.load().oopao_dm_bf16_workspace_bytes(n_pad, batch)
    ws = torch.zeros(nb, dtype=torch.uint8, device='cuda')
    N.call('oopao_dm_opd_bf16', mb, n_pad, c, n_act, n_pix, batch, 0.5, None, out, ws, nb, N.stream_handle())
    torch.cuda.synchronize()
    assert int(ws[:4].view(torch.int32).item()) == 0
    got = out.double().cpu().numpy()
    assert np.isfinite(got).all()
    exact_bf16 = (bf16_round(modes) @ bf16_split(coefs)).T * 0.5
    assert O.rel_l2(got, exact_bf16) < 1e-5
    full = (modes @ coefs.astype(np.float64)).T * 0.5
    assert O.rel_l2(got, full) < 2e-3


def test_tc_projection_with_base(modes):
    import torch
    from oopao_gb300 import _native as N
    n_pix, n_act = modes.shape
    n_pad = (n_act + 63) // 64 * 64
    mt = torch.as_tensor(np.ascontiguousarray(modes.T, dtype=np.float32), device='cuda')
    mb = torch.empty((n_pix, n_pad), dtype=torch.bfloat16, device='cuda')
    N.call('oopao_dm_modes_bf16', mt, n_act, n_pix, n_pad, mb, N.stream_handle())
    coefs = np.random.default_rng(9).standard_normal((n_act, 2)).astype(np.float32)
    base = np.random.default_rng(10).standard_normal((2, n_pix)).astype(np.float32)
    c = torch.as_tensor(coefs, device='cuda')
    b = torch.as_tensor(base, device='cuda')
    out = torch.empty((2, n_pix), device='cuda')
    nb = N.load().oopao_dm_bf16_workspace_bytes(n_pad, 2)
    ws = torch.zeros(nb, dtype=torch.uint8, device='cuda')
    N.call('oopao_dm_opd_bf16', mb, n_pad, c, n_act, n_pix, 2, 1.0, b, out, ws, nb, N.stream_handle())
    torch.cuda.synchronize()
    ref = (bf16_round(modes) @ bf16_split(coefs)).T + base
    assert O.rel_l2(out.double().cpu().numpy(), ref) < 1e-5


def test_bf16_dm_signal_within_tolerance():
    """The BF16 tensor-core IF path against the reference's own Pyramid
    (golden c1: a DM shape's signal and push-pull IM columns of three modes,
    made by the unmodified reference in float64): the BF16 IF bound, 2e-3
    relative L2."""
    import contextlib
    import io
    import oopao_gb300 as og
    from tests import goldens as G
    d = G.load('c1')
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=120, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm16 = og.DeformableMirror(tel, nSubap=20, mechCoupling=0.35, if_dtype='bf16')
        wfs = og.Pyramid(nSubap=20, telescope=tel, modulation=3, lightRatio=0.5, nTheta_user_defined=48,
                         max_batch=64)
    # the factorising IFs would take the exact separable projection: force the
    # tensor-core GEMM over the BF16 IF matrix (the GEMV at one column)
    dm16.separable_projection = False
    assert dm16.projection_path(1) == 'bf16' and dm16.projection_path(64) == 'bf16'
    dm16.coefs = d['dm_coefs']
    ngs ** tel * dm16 * wfs
    assert dm16.tensor_core_status() == 0
    assert O.rel_l2(wfs.signal, d['dm_signal']) < 2e-3
    # the golden IM has three modes: batches of up to 4 columns take the
    # BF16 GEMV; a fixed 64-column tile forces the tcgen05 GEMM as well
    for rule in ([], [(1 << 30, 64)]):
        dm16.tc_tile_rule = rule
        D16 = og.InteractionMatrix(ngs, tel, dm16, wfs, d['im_m2c'], 1e-8, single_pass=False, invert=False).D
        assert dm16.tensor_core_status() == 0
        assert O.rel_l2(D16, d['im_pp_D']) < 2e-3, rule
