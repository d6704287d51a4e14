"""The reference's public signalProcessing(cameraFrame) on the drop-in sensors
(OOPAO/Pyramid.py:835-926, OOPAO/BioEdge.py:729-767): the slopes-maps modes
read the camera's own frame whatever the argument; the full-frame modes map
the argument, fullFrame_sum_flux over the camera frame's sum.  FP32 kernel
against float64 host arithmetic: relative L2 <= 1e-5."""
import contextlib
import io

import numpy as np
import pytest

from oracle import pwfs_oracle as O

pytestmark = pytest.mark.gpu


def _system(post='slopesMaps', bioedge=False):
    import oopao_gb300 as og
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=24, diameter=8.0, samplingTime=1e-3)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = og.DeformableMirror(tel, nSubap=4, mechCoupling=0.35)
        if bioedge:
            wfs = og.BioEdge(nSubap=4, telescope=tel, modulation=3, lightRatio=0.5)
        else:
            wfs = og.Pyramid(nSubap=4, telescope=tel, modulation=3, lightRatio=0.5, postProcessing=post)
    dm.coefs = np.random.default_rng(5).standard_normal(dm.nValidAct) * 50e-9
    ngs ** tel * dm * wfs
    return wfs


@pytest.mark.parametrize('bioedge', [False, True])
def test_slopes_maps_read_the_camera_frame(bioedge):
    wfs = _system(bioedge=bioedge)
    s2d, s = wfs.signalProcessing()
    assert O.rel_l2(s2d, wfs.signal_2D) < 1e-6
    assert O.rel_l2(s, wfs.signal) < 1e-6
    # the argument does not reach the slopes-maps modes
    s2d0, s0 = wfs.signalProcessing(np.zeros_like(wfs.cam.frame))
    np.testing.assert_array_equal(s0, s)
    np.testing.assert_array_equal(s2d0, s2d)


@pytest.mark.parametrize('post', ['fullFrame', 'fullFrame_sum_flux'])
def test_full_frame_modes_map_the_argument(post):
    wfs = _system(post)
    f = np.asarray(wfs.cam.frame, dtype=np.float64)
    s2d, s = wfs.signalProcessing()
    assert O.rel_l2(s, wfs.signal) < 1e-6
    g = 2.0 * f + 0.1 * f.max()
    valid = np.asarray(wfs.validSignal, dtype=bool)
    norma = g[valid].sum() if post == 'fullFrame' else f.sum()
    want = g / norma - wfs.referenceSignal_2D
    s2d, s = wfs.signalProcessing(g)
    assert O.rel_l2(s2d, want) < 1e-5
    assert O.rel_l2(s, want[valid]) < 1e-5
