"""CPU oracle for the reference's GainSensingCamera (optical-gain estimation
from the focal-plane frame of a modulated pyramid, Chambouleyron et al. 2021).

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker, never by the
``oopao_gb300`` package.  A float64 restatement of
``OOPAO/GainSensingCamera.py``:

* ``padder`` :140-147: symmetric zero padding of the [n, n, modes] basis to
  the mask size;
* transforms are numpy's, as in the reference: a complex64 mask is
  transformed in single precision;
* ``fft3`` / ``ifft3`` :150-155: centred 2-D transforms over the first two
  axes, scaled by 1/n and n;
* ``split_basis_product`` :158-173: fft3(basis) * ifft3(basis) per mode;
* ``impulse_response`` :184-185: 2 Im(conj(M^) (mask frame)^) with the
  centred, 1/n-scaled transform;
* ``sensitivity`` :188-193 and ``optical_gains`` :196-199;
* ``calibration`` / ``compute_optical_gains`` :78-120 (frames normalised
  to unit sum).
"""
from __future__ import annotations

import numpy as np


def _sh(a, axes=(-2, -1)):
    return np.fft.fftshift(a, axes=axes)


def centred_fft2(a, axes=(-2, -1)):
    """fftshift(fft2(fftshift(a))) / n over `axes` (``fft3`` :150-151)."""
    n = a.shape[axes[0]]
    return _sh(np.fft.fft2(_sh(a, axes), axes=axes), axes) / n


def centred_ifft2(a, axes=(-2, -1)):
    """fftshift(ifft2(fftshift(a))) * n over `axes` (``ifft3`` :154-155)."""
    n = a.shape[axes[0]]
    return _sh(np.fft.ifft2(_sh(a, axes), axes=axes), axes) * n


def pad_basis(basis, n_out):
    """``padder``: [n, n, modes] -> [n_out, n_out, modes], (n_out - n)//2 zeros each side."""
    n = basis.shape[0]
    if n_out <= n:
        raise ValueError('Output size %d should be higher than input size %d' % (n_out, n))
    p = (n_out - n) // 2
    return np.pad(basis, ((p, p), (p, p), (0, 0)))


def basis_product(basis, n_out):
    """``split_basis_product``: fft3(b) * ifft3(b) for every mode, [n_out, n_out, modes] complex."""
    b = pad_basis(np.asarray(basis, dtype=np.float64), n_out)
    return centred_fft2(b, axes=(0, 1)) * centred_ifft2(b, axes=(0, 1))


def impulse_response(mask, frame):
    """``impulse_response`` :184-185."""
    return 2 * np.imag(np.conj(centred_fft2(mask)) * centred_fft2(mask * frame))


def sensitivity(ir_1, ir_2, bp):
    """``sensitivity`` :188-193: (fft3(IR_1) ifft3(IR_2)).flatten() @ bp."""
    v = (centred_fft2(ir_1) * centred_ifft2(ir_2)).reshape(-1)
    return v @ bp.reshape(-1, bp.shape[-1])


def optical_gains(ir_sky, ir_calib, bp, sensi_calib):
    """``optical_gains`` :196-199."""
    return np.real(sensitivity(ir_sky, ir_calib, bp) / sensi_calib)


class OracleGSC:
    """``GainSensingCamera`` in float64."""

    def __init__(self, mask, basis):
        self.mask = np.asarray(mask)
        self.basis = np.asarray(basis)
        self.n_modes = self.basis.shape[-1]
        self.calibration_ready = False

    def calibration(self, frame):
        frame = frame / frame.sum()
        self.basis_product = basis_product(self.basis, self.mask.shape[0])
        self.IR_calib = impulse_response(self.mask, frame)
        self.sensi_calib = sensitivity(self.IR_calib, self.IR_calib, self.basis_product)
        self.calibration_ready = True
        self.og = np.ones(self.n_modes)

    def compute_optical_gains(self, frame):
        if not self.calibration_ready:
            raise ValueError('Optical gains must be initialized first!')
        frame = frame / frame.sum()
        self.IR_sky = impulse_response(self.mask, frame)
        self.og = optical_gains(self.IR_sky, self.IR_calib, self.basis_product, self.sensi_calib)
