"""The detector oracle against frames of the unmodified reference Detector
(tests/golden/detector_tiny.npz, made by make_golden.py): integration over
loop steps, full well, CCD/CMOS gain, ADC with and without full well,
unsigned casts, log scale, background map, hardware binning."""
import numpy as np

from oracle import detector_oracle as D
from tests.goldens import load as load_golden


def test_detector_oracle_matches_reference():
    g = load_golden('detector_tiny')
    for tag, kw in g['params']['cases'].items():
        kw = dict(kw)
        if tag == 'log_bg':
            kw['backgroundMap'] = g['bg']
        it = kw.pop('integrationTime', None)
        seq = D.camera_sequence(g['frames'], float(g['dt']), it, **kw)
        np.testing.assert_allclose(seq, g[tag], rtol=1e-12, atol=1e-9, err_msg=tag)


def test_unsigned_widths():
    g = load_golden('detector_tiny')
    assert str(g['adc16_fwc_dtype']) == 'uint16' and str(g['adc8_nofwc_dtype']) == 'uint8'
    assert str(g['int3_fwc_adc12_dtype']) == 'float64'
    assert D.output_width(16) == 16 and D.output_width(12) == 0 and D.output_width(None, np.uint32) == 32
