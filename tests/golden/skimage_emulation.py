"""Stand-in for the two scikit-image calls the reference atmosphere makes
(``OOPAO/tools/tools.py:202-209``), for fixture generation where
scikit-image is not installed.

``SimilarityTransform(translation=(tx, ty))`` and ``warp(image,
tform.inverse, order=3)``: scikit-image's fast warp path for a homography
interpolates with the bicubic convolution kernel (Keys, a = -0.5), reads
``cval = 0`` outside the image (mode 'constant') and, with the default
``clip=True``, clips the output to the input's value range.  This module
implements exactly that, for translations only.
"""
import numpy as np


class SimilarityTransform:
    def __init__(self, matrix=None, scale=None, rotation=None, translation=None):
        if matrix is not None or scale not in (None, 1) or rotation not in (None, 0):
            raise NotImplementedError('only pure translations are emulated')
        self.translation = np.zeros(2) if translation is None else np.asarray(translation, dtype=np.float64)

    @property
    def inverse(self):
        return SimilarityTransform(translation=-self.translation)


def _cubic(x, f0, f1, f2, f3):
    return f1 + 0.5 * x * (f2 - f0 + x * (2.0 * f0 - 5.0 * f1 + 4.0 * f2 - f3 + x * (3.0 * (f1 - f2) + f3 - f0)))


def warp(image, inverse_map, order=3, mode='constant', cval=0.0, clip=True, preserve_range=False):
    if order != 3 or mode != 'constant' or not isinstance(inverse_map, SimilarityTransform):
        raise NotImplementedError('only order-3 translations with constant mode are emulated')
    image = np.asarray(image, dtype=np.float64)
    R, C = image.shape
    dx, dy = inverse_map.translation           # output (r, c) reads input (r + dy, c + dx)
    rr, cc = np.meshgrid(np.arange(R) + dy, np.arange(C) + dx, indexing='ij')
    r0 = np.floor(rr).astype(int)
    c0 = np.floor(cc).astype(int)
    xr, xc = rr - r0, cc - c0

    def pix(r, c):
        ok = (r >= 0) & (r < R) & (c >= 0) & (c < C)
        return np.where(ok, image[np.clip(r, 0, R - 1), np.clip(c, 0, C - 1)], cval)

    rows = [_cubic(xc, *[pix(r0 + pr - 1, c0 + pc - 1) for pc in range(4)]) for pr in range(4)]
    out = _cubic(xr, *rows)
    if clip:
        lo, hi = image.min(), image.max()
        keep = mode == 'constant' and not (lo <= cval <= hi)
        mask = out == cval if keep else None
        out = np.clip(out, lo, hi)
        if keep:
            out[mask] = cval
    return out
