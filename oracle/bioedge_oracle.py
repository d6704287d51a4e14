"""CPU oracle for the reference's Bi-O Edge sensor.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker, never by the
``oopao_gb300`` package.  A float64 restatement of ``OOPAO/BioEdge.py``: the
four Fourier masks (``mask_computation`` :331-392), the per-point transform
with its sqrt(0.5) field and four masked inverse transforms tiled 2x2
(``bio_edge_transform`` :510-544, ``convolution`` :435-443), sum-binning to
the camera (``__mul__`` :1033-1057), the quadrants of ``grabQuadrant``
(:840-853), ``signalProcessing`` 'slopesMaps' (:729-742), and the
construction sequence (``initialization`` :445-490, ``wfs_calibration``
:492-507).  Geometry, modulation path and tip/tilt buffers are those of the
pyramid (``pwfs_oracle``), which the reference BioEdge computes the same way.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.fft

from . import pwfs_oracle as P


def bioedge_masks(res, n_subap, n_pix_separation=2., n_pix_edge=None, grey_width=0., grey_length=False,
                  quadrants_numbering=(0, 1, 2, 3), sx=(0, 0, 0, 0), sy=(0, 0, 0, 0), initial_res=None):
    """The four complex Fourier masks [4, N, N] (``mask_computation``)."""
    if n_pix_edge is None:
        n_pix_edge = n_pix_separation // 2
    if initial_res is None:
        initial_res = res
    N = int((n_subap * 2 + n_pix_separation + n_pix_edge * 2) * res / n_subap)
    zp = N / res
    norma = (n_subap * 2) * (res / n_subap) * (1 / (n_subap * 2))
    tip, tilt = np.meshgrid(np.linspace(-np.pi, np.pi, N, endpoint=False), np.linspace(-np.pi, np.pi, N, endpoint=False))
    bw = np.zeros(N)
    bw[0:N // 2] = 1.
    r = int(np.round(zp * grey_width * res / initial_res))
    if grey_width != 0:
        bw[N // 2 - r:N // 2 + r] = np.hstack([np.linspace(1, 0.5, r, endpoint=True),
                                              np.linspace(0.5, 0, r, endpoint=True)])
    X, _ = np.meshgrid(bw, bw)
    A = np.sqrt(X)
    if grey_length is not False:
        rl = int(np.round(zp * grey_length))
        A[0:N // 2 - rl, 0:N // 2] = 1.
        A[N // 2 + rl:, 0:N // 2] = 1.
        A[0:N // 2 - rl, N // 2:] = 0.
        A[N // 2 + rl:, N // 2:] = 0.
    B = np.sqrt(1 - A ** 2)
    C, D = A.T.copy(), B.T.copy()
    # one shift for all four masks (OOPAO/BioEdge.py:361-364)
    sx = [sx] * 4 if np.isscalar(sx) else sx
    sy = [sy] * 4 if np.isscalar(sy) else sy
    tts = [-sx[3] * tip * norma + sy[3] * tilt * norma, -sx[2] * tip * norma + sy[2] * tilt * norma,
           -sx[1] * tip * norma + sy[1] * tilt * norma, -sx[0] * tip * norma + sy[0] * tilt * norma]
    base = [A, B, C, D]
    return np.stack([base[quadrants_numbering[i]] * np.exp(1j * tts[i]) for i in range(4)])


@dataclass
class OracleBioEdge:
    geom: P.PyramidGeometry
    masks: np.ndarray
    intensity: np.ndarray
    tt: np.ndarray
    valid_i4q: np.ndarray
    reference_2d: np.ndarray
    n_theta: int

    def raw(self, phase):
        """raw_data [2N, 2N] for one phase map: sum over points of the four
        |ifft2(F * mask_q)|^2 tiled [[0, 1], [2, 3]]."""
        g = self.geom
        N, res, c = g.N, g.res, g.center
        lo = c - res // 2
        amp = np.sqrt(self.intensity / self.tt.shape[0])
        out = np.zeros((2 * N, 2 * N))
        for k in range(self.tt.shape[0]):
            sup = np.zeros((N, N), dtype=np.complex128)
            sup[lo:lo + res, lo:lo + res] = np.sqrt(0.5) * amp * np.exp(1j * (phase + self.tt[k].astype(np.float64)))
            F = np.fft.fft2(sup * g.phasor)
            for q in range(4):
                i, j = divmod(q, 2)
                out[i * N:(i + 1) * N, j * N:(j + 1) * N] += np.abs(np.fft.ifft2(F * self.masks[q])) ** 2
        return out

    def focal(self, phase):
        """What the focal-plane camera sums: each point's focal field
        fft2(sqrt(0.5) A exp(i(phi + TT_k)) phasor), kept once per mask
        (``convolution`` :435-443), |.|^2 summed over that list
        (``__mul__`` :1036-1038)."""
        g = self.geom
        N, res, c = g.N, g.res, g.center
        lo = c - res // 2
        amp = np.sqrt(self.intensity / self.tt.shape[0])
        out = np.zeros((N, N))
        for k in range(self.tt.shape[0]):
            sup = np.zeros((N, N), dtype=np.complex128)
            sup[lo:lo + res, lo:lo + res] = np.sqrt(0.5) * amp * np.exp(1j * (phase + self.tt[k].astype(np.float64)))
            out += len(self.masks) * np.abs(np.fft.fft2(sup * g.phasor)) ** 2
        return out

    def frame(self, phase):
        return P.set_binning(self.raw(phase), self.geom.N / self.geom.cam)

    def quadrant(self, frame, n):
        cp = int(np.round(self.geom.cam / 2))
        rows = slice(0, cp) if n in (1, 2) else slice(cp, 2 * cp)
        cols = slice(0, cp) if n in (1, 3) else slice(cp, 2 * cp)
        return frame[rows, cols]

    def slopes(self, frame, reference_2d=None):
        ref = self.reference_2d if reference_2d is None else reference_2d
        I1, I2, I3, I4 = [self.quadrant(frame, n) * self.valid_i4q for n in (1, 2, 3, 4)]
        norma = np.mean((I1 + I2 + I3 + I4)[self.valid_i4q])
        maps = np.concatenate(((I1 - I2 + I4 - I3), (I1 - I4 + I2 - I3)) / norma) - ref
        valid = np.concatenate((self.valid_i4q, self.valid_i4q))
        return maps, maps[np.where(valid == 1)]

    def measure(self, phase):
        f = self.frame(phase)
        s2d, s = self.slopes(f)
        return f, s2d, s


def build_bioedge(res, n_subap, modulation, light_ratio, intensity, n_pix_separation=2., n_pix_edge=None,
                  calib_modulation=50., n_theta_user=None, extra=0, delta_theta=0., grey_width=0.,
                  grey_length=False, quadrants_numbering=(0, 1, 2, 3)) -> OracleBioEdge:
    """Construction of ``BioEdge.__init__``: valid pixels at the calibration
    modulation, then the flat-wavefront reference slopes."""
    geom = P.pyramid_geometry(res, n_subap, n_pix_separation, n_pix_edge, True)
    masks = bioedge_masks(res, n_subap, n_pix_separation, n_pix_edge, grey_width, grey_length, quadrants_numbering)
    if calib_modulation >= res / 2:
        calib_modulation = res / 2 - 1
    cpath, _ = P.modulation_path(calib_modulation, n_theta_user, extra, delta_theta)
    flat = np.zeros((res, res))
    b0 = OracleBioEdge(geom, masks, intensity, P.tt_buffers(cpath, geom), None, 0.0, 0)
    f0 = b0.frame(flat)
    I4Q = sum(b0.quadrant(f0, n) for n in (1, 2, 3, 4))
    valid = I4Q >= light_ratio * I4Q.max()
    path, n_theta = P.modulation_path(modulation, n_theta_user, extra, delta_theta)
    b = OracleBioEdge(geom, masks, intensity, P.tt_buffers(path, geom), valid, 0.0, n_theta)
    ref2d, _ = b.slopes(b.frame(flat), reference_2d=0.0)
    b.reference_2d = ref2d
    return b
