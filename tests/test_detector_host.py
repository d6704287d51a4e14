"""Host-side behaviour of the drop-in Detector (no GPU): the frame a batch
leaves on the camera is its last one, as the reference's sensor integrates a
batch of wavefronts frame by frame (OOPAO/Pyramid.py:825-830); a single
frame reads back as [cam, cam]; an assigned frame is returned as given."""
import numpy as np
import torch

from oopao_gb300.detector import Detector


def test_batch_leaves_its_last_frame():
    cam = Detector(6)
    frames = torch.arange(3 * 6 * 6, dtype=torch.float32).reshape(3, 6, 6)
    cam._set_device_frame(frames)
    f = cam.frame
    assert f.shape == (6, 6) and f.dtype == np.float64
    np.testing.assert_array_equal(f, frames[-1].double().numpy())
    assert cam.device_frame.shape == (3, 6, 6)


def test_single_frame_and_assignment():
    cam = Detector(4)
    one = torch.ones((1, 4, 4), dtype=torch.float32)
    cam._set_device_frame(one)
    assert cam.frame.shape == (4, 4)
    cam.frame = np.full((4, 4), 2.0)
    np.testing.assert_array_equal(cam.frame, np.full((4, 4), 2.0))


def _golden():
    from tests.goldens import load
    return load('detector_tiny')


def test_integration_time_sequence_on_host_tensors():
    """integrationTime = 2 loop steps: the camera shows the sum of two frames
    at every second step and keeps it in between, zeros before the first
    readout (OOPAO/Detector.py:331-354), whether the steps come one by one or
    as one batch."""
    g = _golden()
    frames = torch.as_tensor(g['frames'], dtype=torch.float32)
    cam = Detector(12, integrationTime=2e-3)
    one = torch.stack([cam._integrate_device(frames[i][None], dt=float(g['dt']), wfs=False)[0]
                       for i in range(frames.shape[0])])
    np.testing.assert_allclose(one.double().numpy(), g['int2_plain'], rtol=1e-6)
    cam = Detector(12, integrationTime=2e-3)
    batch = cam._integrate_device(frames, dt=float(g['dt']), wfs=False)
    np.testing.assert_allclose(batch.double().numpy(), g['int2_plain'], rtol=1e-6)
    assert len(cam.buffer_frame) == 1   # the 7th step is still integrating


def test_readout_errors():
    import pytest
    from oopao_gb300.tools import OopaoError
    f = torch.ones((1, 12, 12))
    with pytest.raises(OopaoError, match='integrationTime'):
        Detector(12, darkCurrent=10.0)._integrate_device(f, wfs=False)
    with pytest.raises(OopaoError, match='backgroung map'):
        Detector(12, bits=16, FWC=1000, backgroundMap=np.zeros((12, 12)))._integrate_device(f, wfs=False)
    with pytest.raises(OopaoError, match='backgroung map'):
        Detector(12, backgroundMap=np.zeros((5, 5)), gain=2)._integrate_device(f, wfs=False)
    with pytest.raises(OopaoError, match='binning'):
        Detector(12, binning=2)._integrate_device(f)
    with pytest.raises(OopaoError, match='backgroundFlux'):
        Detector(12, backgroundNoise=True)._integrate_device(f, wfs=False)
    with pytest.raises(ValueError, match='Binning factor'):
        Detector(12, binning=5)._integrate_device(f, wfs=False)


def test_integration_time_setter_restarts():
    cam = Detector(4, integrationTime=3e-3)
    cam._integrate_device(torch.ones((2, 4, 4)), dt=1e-3, wfs=False)
    assert len(cam.buffer_frame) == 2 and cam._integrated_time > 0
    cam.integrationTime = 5e-3
    assert cam.buffer_frame == [] and cam._integrated_time == 0


def test_properties_lines():
    cam = Detector(8, integrationTime=2e-3, bits=12, FWC=1000, gain=2, binning=2)
    p = cam.properties()
    assert p['resolution'].endswith('4'.center(9)) and 'Exposure' in p['exposure'] and '12' in p['quantization']
    assert 'Detector' in repr(cam)
