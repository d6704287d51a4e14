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
