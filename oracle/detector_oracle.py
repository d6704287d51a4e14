"""CPU restatement of the reference Detector's readout chain for the stages
without random draws (``OOPAO/Detector.py:192-354``), in float64 and in the
reference's order of operations.

Test infrastructure only: the tests use it as the checker of the device
camera (``oopao_gb300.detector``); nothing in the product imports it.
Pinned to frames the unmodified reference produced
(``tests/golden/detector_tiny.npz``, ``tests/test_oracle_detector.py``).
"""
import numpy as np

_UNSIGNED = {8: np.uint8, 16: np.uint16, 32: np.uint32, 64: np.uint64}


def set_binning_sum(frame: np.ndarray, b: int) -> np.ndarray:
    """tools.set_binning(mode='sum') of a 2-D frame (OOPAO/tools/tools.py:464-473)."""
    n = frame.shape[0]
    if n % b != 0:
        raise ValueError('Binning factor %d not compatible with the array size' % b)
    m = int(np.round(n / b))
    return frame.reshape(m, n // m, m, n // m).sum(-1).sum(1)


def output_width(bits, output_precision=None):
    """set_output_precision (OOPAO/Detector.py:192-213): the unsigned output
    width (0: floating point)."""
    if output_precision is not None:
        dt = np.dtype(output_precision)
        return dt.itemsize * 8 if np.issubdtype(dt, np.unsignedinteger) else 0
    return bits if bits in _UNSIGNED else 0


def to_unsigned(frame: np.ndarray, width: int) -> np.ndarray:
    """frame.astype(uint<width>) (OOPAO/Detector.py:313) as an x86 numpy
    performs it: truncation toward zero, values outside the type wrap."""
    t = np.trunc(frame)
    if width < 64:
        t = np.mod(t, 2.0 ** width)
    return t


def readout(frame, FWC=None, sensor='CCD', gain=1, binning=1, bits=None, output_precision=None,
            log_scale=False, backgroundMap=None) -> np.ndarray:
    """Detector.readout (OOPAO/Detector.py:273-329) of an integrated frame,
    without dark current, EMCCD amplification or readout noise (the random
    stages)."""
    f = np.asarray(frame, dtype=np.float64)
    if FWC is not None:                                    # set_saturation :219-224
        f = np.clip(f, 0, FWC)
    if binning != 1:                                       # applied twice, :290-297
        f = set_binning_sum(set_binning_sum(f, binning), binning)
    width = output_width(bits, output_precision)
    clip_unsigned = 0 if width else -np.inf
    if sensor in ('CCD', 'CMOS'):                          # :304-305
        f = f * gain
    if bits is not None:                                   # digitalization :226-238
        if FWC is None:
            f = f / f.max() * 2 ** bits
        else:
            f = f / FWC * (2 ** bits - 1)
            f = np.clip(f, max(f.min(), clip_unsigned), 2 ** bits - 1)
    if log_scale:                                          # :311-312
        f = np.log10(f)
    if width:                                              # :313
        f = to_unsigned(f, width)
    if backgroundMap is not None:                          # remove_bakground :266-271
        f = f - backgroundMap
    return f


def camera_sequence(frames, dt: float, integrationTime=None, **readout_kw) -> np.ndarray:
    """Detector.integrate (OOPAO/Detector.py:331-354) over loop steps, the
    sensor adding dt to the integrated time before each (OOPAO/Pyramid.py:1179-1201):
    the camera frame after every step (the last readout; zeros before the first)."""
    frames = np.asarray(frames, dtype=np.float64)
    out, buf, t = [], [], 0.0
    cur = None
    for f in frames:
        t += dt
        buf.append(f)
        if integrationTime is None or t >= integrationTime:
            cur = readout(np.sum(buf, axis=0), **readout_kw)
            buf, t = [], 0.0
        out.append(cur if cur is not None else np.zeros_like(f))
    return np.array(out)
