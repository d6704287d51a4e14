"""CPU oracle for the modulated pyramid WFS and DM influence-function path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: it is imported by
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py``, never by the ``oopao_gb300``
package.  It restates, in float64 numpy, the algorithm of cheritier/OOPAO for
this path; every function cites the reference file:line it follows (paths are
relative to the OOPAO project root).

Parity of this restatement is pinned against golden vectors produced by
running the unmodified reference (``tests/golden/make_golden.py`` writes
``tests/golden/*.npz``; ``tests/test_oracle_golden.py`` checks them).

Conventions shared with the reference:
  * everything is float64 / complex128 (``OOPAO/__init__.py:55-60`` forces 64),
    except the pyramid mask, stored as complex64 (``OOPAO/Pyramid.py:388``),
    and the modulation tip/tilt buffers, stored as float32
    (``OOPAO/Pyramid.py:1133-1139``);
  * forward transform = ``scipy.fft.fft2``, inverse = ``numpy.fft.ifft2``
    (``OOPAO/Pyramid.py:17-22``, ``:629-630``);
  * 2-D maps are row-major [row, col]; ``meshgrid(x, x)`` puts x along columns.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.fft

# ---------------------------------------------------------------------------
# Source / Telescope (boundary objects)
# ---------------------------------------------------------------------------

# Source.photometry, OOPAO/Source.py:340-405: [wavelength, bandwidth, zero point]
_CST = 368.0
PHOTOMETRY = {
    'U': (0.360e-6, 0.070e-6, 1.96e12 / _CST),
    'B': (0.440e-6, 0.100e-6, 5.38e12 / _CST),
    'V0': (0.500e-6, 0.090e-6, 3.64e12 / _CST),
    'V': (0.550e-6, 0.090e-6, 3.31e12 / _CST),
    'R': (0.640e-6, 0.150e-6, 4.01e12 / _CST),
    'I': (0.790e-6, 0.150e-6, 2.69e12 / _CST),
    'J': (1.215e-6, 0.260e-6, 1.90e12 / _CST),
    'H': (1.654e-6, 0.290e-6, 1.05e12 / _CST),
    'K': (2.179e-6, 0.410e-6, 0.70e12 / _CST),
}


def n_photon(band: str, magnitude: float) -> float:
    """Photons / m^2 / s, ``OOPAO/Source.py:125`` (zeroPoint*10**(-0.4*mag))."""
    return PHOTOMETRY[band][2] * 10 ** (-0.4 * magnitude)


def telescope_pupil(res: int, central_obstruction: float = 0.0) -> np.ndarray:
    """Circular pupil with central obstruction, ``OOPAO/Telescope.py:226-246``."""
    D = res + 1
    x = np.linspace(-res / 2, res / 2, res, dtype=np.float64)
    xx, yy = np.meshgrid(x, x)
    circle = xx ** 2 + yy ** 2
    obs = circle >= (central_obstruction * D / 2) ** 2
    return (circle < (D / 2) ** 2) * obs


def source_intensity(pupil: np.ndarray, nphoton: float, sampling_time: float,
                     diameter: float) -> np.ndarray:
    """fluxMap * scintillation after ``tel.relay``: ``OOPAO/Telescope.py:199-224``
    (fluxMap ``:223``, scintillation = ones*pupil ``:214-216``) and
    ``OOPAO/Source.py:206-229`` (intensity = fluxMap * scintillation)."""
    res = pupil.shape[0]
    refl = (pupil * 1.0).astype(np.float64)
    flux = refl * nphoton * sampling_time * (diameter / res) ** 2
    scint = np.ones(pupil.shape) * pupil
    return (np.array(flux) * np.array(scint)).astype(np.float64)


# ---------------------------------------------------------------------------
# Deformable mirror
# ---------------------------------------------------------------------------

MISREG_FIELDS = ('rotationAngle', 'shiftX', 'shiftY', 'anamorphosisAngle', 'tangentialScaling', 'radialScaling')


def _misreg(misreg):
    m = dict.fromkeys(MISREG_FIELDS, 0.0)
    m.update(misreg or {})
    return m


def dm_actuator_pixels(res: int, diameter: float, n_subap: int,
                       central_obstruction: float = 0.0, misreg=None):
    """Fried-geometry actuator grid and radial selection, then pixel centres.

    ``OOPAO/DeformableMirror.py:306-340`` (grid, r_in/r_out selection) and
    ``:359-386`` (mis-registration, pixel coordinates u0x/u0y): the valid
    actuators are stretched along the anamorphosis direction (``:564-570``,
    by 1+tangentialScaling along it and 1+radialScaling across it, the
    order in which the reference passes them), rotated (``:559-562``), then
    shifted by -shiftX, -shiftY metres.
    """
    mr = _misreg(misreg)
    pitch = diameter / n_subap
    n_act = n_subap + 1
    x = np.linspace(-diameter / 2, diameter / 2, n_act)
    X, Y = np.meshgrid(x, x)
    xIF0 = np.reshape(X, [n_act ** 2])
    yIF0 = np.reshape(Y, [n_act ** 2])
    r = np.sqrt(xIF0 ** 2 + yIF0 ** 2)
    r_in = central_obstruction * diameter / 2 - 0.5 * pitch
    r_out = diameter / 2 + 0.7533 * pitch
    valid = (r >= r_in) * (r <= r_out)
    x0 = xIF0[valid]
    y0 = yIF0[valid]
    ang = mr['anamorphosisAngle'] * np.pi / 180
    along, across = 1 + mr['tangentialScaling'], 1 + mr['radialScaling']
    c2, s2, cs = np.cos(ang) ** 2, np.sin(ang) ** 2, np.sin(2 * ang) / 2
    x3 = x0 * (along * c2 + across * s2) + y0 * (across - along) * cs
    y3 = y0 * (along * s2 + across * c2) + x0 * (across - along) * cs
    rot = mr['rotationAngle'] * np.pi / 180
    xIF = x3 * np.cos(rot) - y3 * np.sin(rot) - mr['shiftX']
    yIF = y3 * np.cos(rot) + x3 * np.sin(rot) - mr['shiftY']
    u0x = res / 2 + xIF * res / diameter
    u0y = res / 2 + yIF * res / diameter
    return u0x, u0y, valid


def dm_modes(res: int, diameter: float, n_subap: int, mech_coupling: float = 0.35,
             central_obstruction: float = 0.0, misreg=None) -> np.ndarray:
    """Gaussian influence functions [res*res, nAct] (row-major pixel index).

    ``OOPAO/DeformableMirror.py:572-600`` (modesComputation: widths scaled by
    1+radialScaling and 1+tangentialScaling, Gaussian axes along the
    anamorphosis angle) stacked as in ``:389-394``.
    """
    mr = _misreg(misreg)
    u0x, u0y, _ = dm_actuator_pixels(res, diameter, n_subap, central_obstruction, misreg)
    n_along = n_subap
    w = (res / n_along) / np.sqrt(2 * np.log(1. / mech_coupling))
    cx = (1 + mr['radialScaling']) * w
    cy = (1 + mr['tangentialScaling']) * w
    theta = mr['anamorphosisAngle'] * np.pi / 180
    xg = np.linspace(0, 1, res) * res
    X, Y = np.meshgrid(xg, xg)
    a = np.cos(theta) ** 2 / (2 * cx ** 2) + np.sin(theta) ** 2 / (2 * cy ** 2)
    b = -np.sin(2 * theta) / (4 * cx ** 2) + np.sin(2 * theta) / (4 * cy ** 2)
    c = np.sin(theta) ** 2 / (2 * cx ** 2) + np.cos(theta) ** 2 / (2 * cy ** 2)
    out = np.empty((res * res, len(u0x)))
    for i, (x0, y0) in enumerate(zip(u0x, u0y)):
        G = np.exp(-(a * (X - x0) ** 2 + 2 * b * (X - x0) * (Y - y0) + c * (Y - y0) ** 2))
        out[:, i] = G.reshape(res * res)
    return out


def dm_opd(modes: np.ndarray, coefs: np.ndarray, res: int) -> np.ndarray:
    """``dm.coefs`` setter, ``OOPAO/DeformableMirror.py:651-686``:
    OPD = reshape(modes @ coefs) -> [res,res] (1-D coefs) or [res,res,B]."""
    coefs = np.asarray(coefs, dtype=np.float64)
    if coefs.ndim == 1:
        return np.reshape(modes @ coefs, [res, res])
    return np.reshape(modes @ coefs, [res, res, coefs.shape[1]])


# ---------------------------------------------------------------------------
# Pyramid geometry
# ---------------------------------------------------------------------------

@dataclass
class PyramidGeometry:
    res: int
    n_subap: int
    n_pix_separation: float
    n_pix_edge: float
    psf_centering: bool
    N: int
    cam: int
    center: int
    mask: np.ndarray            # complex64 [N,N]
    phasor: np.ndarray          # complex128 [N,N]
    tip: np.ndarray             # float64 [res,res]
    tilt: np.ndarray            # float64 [res,res]
    binning: int = 1
    extra: dict = field(default_factory=dict)
    spatial_filter: object = None  # [N,N] or None; mask already includes it


def with_spatial_filter(geom: PyramidGeometry, filt, initial_mask=None) -> PyramidGeometry:
    """``spatialFilter`` setter, ``OOPAO/Pyramid.py:1051-1085``: mask =
    initial_mask * filter (initial_mask again for None or a wrong shape)."""
    import dataclasses
    m0 = geom.mask if initial_mask is None else initial_mask
    if filt is not None and np.shape(filt) == m0.shape:
        mask = m0 * filt
    else:
        mask = m0
    return dataclasses.replace(geom, mask=mask, spatial_filter=filt)


def phase_mask(res: int, n_subap: int, n_pix_separation: float, n_pix_edge: float,
               psf_centering: bool, rooftop: float = 0.0, theta_rotation: float = 0.0,
               sx=(0, 0, 0, 0), sy=(0, 0, 0, 0)) -> np.ndarray:
    """Four-face pyramid phase (max of four tilted planes), ``OOPAO/Pyramid.py:453-480``."""
    rooftop_pixels = rooftop / np.sqrt(2)
    n_tot = int((n_subap * 2 + n_pix_separation + n_pix_edge * 2) * res / n_subap)
    norma = res / n_subap
    lim = np.pi
    x = np.linspace(-(1 - psf_centering * 1 / n_tot) * lim, (1 - psf_centering * 1 / n_tot) * lim,
                    n_tot, endpoint=psf_centering)
    x_, y_ = np.meshgrid(x, x)
    xr = x_ * np.cos(theta_rotation) - y_ * np.sin(theta_rotation)
    yr = y_ * np.cos(theta_rotation) + x_ * np.sin(theta_rotation)
    r = (n_subap + n_pix_separation) / 2
    P1 = xr * r + x_ * sx[0] + yr * r - y_ * sy[0] + rooftop_pixels
    P2 = -xr * r + x_ * sx[1] + yr * r - y_ * sy[1]
    P3 = -xr * r + x_ * sx[2] - yr * r - y_ * sy[2] + rooftop_pixels
    P4 = xr * r + x_ * sx[3] - yr * r - y_ * sy[3]
    stacked = np.stack([P1, P2, P3, P4]) * norma
    return -np.max(stacked, axis=0)


def phase_mask_old(res: int, n_subap: int, n_pix_separation: float, n_pix_edge: float,
                   psf_centering: bool, sx=(0, 0, 0, 0), sy=(0, 0, 0, 0)) -> np.ndarray:
    """Quadrant tip/tilt pyramid phase (``old_mask``), ``OOPAO/Pyramid.py:482-539``.

    Each quadrant holds a zero-mean plane ±tip·(s ± sx_q) ± tilt·(s ± sy_q),
    s = n_subap + n_pix_separation, scaled by (res/n_subap)/4.  Centred on
    four pixels the quadrants are n/2 square with grids linspace(-pi, pi,
    n/2, endpoint=False); centred on one pixel they are n/2+1 or n/2-1 wide
    (grids over ±pi with the endpoint, or ±(pi - 2pi/n) without), the later
    quadrants overwriting the shared row and column in the order 1, 2, 3, 4.
    """
    n = int((n_subap * 2 + n_pix_separation + n_pix_edge * 2) * res / n_subap)
    h = n // 2
    s = n_subap + n_pix_separation
    scale = res / n_subap / 4
    m = np.zeros((n, n))

    def grid(x_len, x_full, y_len, y_full):
        # zero-mean tip (along x) and tilt (along y) planes of one quadrant
        def axis(length, full):
            if psf_centering:
                return np.linspace(-np.pi, np.pi, length, endpoint=False)
            if full:
                return np.linspace(-np.pi, np.pi, length, endpoint=True)
            lim = np.pi - 2 * np.pi / n
            return np.linspace(-lim, lim, length, endpoint=False)
        tip, tilt = np.meshgrid(axis(x_len, x_full), axis(y_len, y_full))
        return tip - tip.mean(), tilt - tilt.mean()

    if psf_centering:
        g = grid(h, True, h, True)
        quads = [((slice(0, h), slice(0, h)), g, (+1, +1, +1, -1)),
                 ((slice(0, h), slice(n - h, n)), g, (-1, -1, +1, -1)),
                 ((slice(n - h, n), slice(n - h, n)), g, (-1, -1, -1, +1)),
                 ((slice(n - h, n), slice(0, h)), g, (+1, +1, -1, +1))]
    else:
        big, small = h + 1, h - 1
        g1 = grid(big, True, big, True)
        g2 = grid(big, True, small, False)
        g3 = grid(small, False, small, False)
        g4 = grid(small, False, big, True)
        quads = [((slice(0, big), slice(0, big)), g1, (+1, +1, +1, -1)),
                 ((slice(0, big), slice(n - small, n)), g4, (-1, -1, +1, -1)),
                 ((slice(n - small, n), slice(n - small, n)), g3, (-1, -1, -1, +1)),
                 ((slice(n - small, n), slice(0, big)), g2, (+1, +1, -1, +1))]
    for q, ((rows, cols), (tip, tilt), (a, b, c, d)) in enumerate(quads):
        # a*tip*(s + b*sx) + c*tilt*(s + d*sy)
        m[rows, cols] = (a * tip * (s + b * sx[q]) + c * tilt * (s + d * sy[q])) * scale
    return -m


def pyramid_geometry(res: int, n_subap: int, n_pix_separation: float = 2,
                     n_pix_edge: float | None = None, psf_centering: bool = True,
                     rooftop: float = 0.0, theta_rotation: float = 0.0,
                     initial_res: int | None = None, old_mask: bool = False,
                     sx=(0, 0, 0, 0), sy=(0, 0, 0, 0)) -> PyramidGeometry:
    """FFT grid, camera size, tip/tilt grids, centring phasor and mask.

    ``OOPAO/Pyramid.py:276-285`` (N, zero padding, camera), ``:334-344``
    (Tip/Tilt, phasor), ``:368-391`` (mask, complex64; ``old_mask`` picks the
    quadrant tip/tilt mask, sx/sy the face shifts as ``apply_shift_wfs``
    hands them to the mask, ``:400-451``).
    """
    if n_pix_edge is None:
        n_pix_edge = n_pix_separation // 2
    if initial_res is None:
        initial_res = res
    N = int((n_subap * 2 + n_pix_separation + n_pix_edge * 2) * res / n_subap)
    zp = N / res
    cam = round(n_subap * zp)
    tip, tilt = np.meshgrid(np.linspace(-np.pi, np.pi, res), np.linspace(-np.pi, np.pi, res))
    tilt = tilt * (res / initial_res)
    tip = tip * (res / initial_res)
    xx, yy = np.meshgrid(np.linspace(0, N - 1, N), np.linspace(0, N - 1, N))
    phasor = np.exp(-(1j * np.pi * (N + 1) / N) * (xx + yy))
    if old_mask:
        m = phase_mask_old(res, n_subap, n_pix_separation, n_pix_edge, psf_centering, sx, sy)
    else:
        m = phase_mask(res, n_subap, n_pix_separation, n_pix_edge, psf_centering, rooftop, theta_rotation, sx, sy)
    mask = np.complex64(np.exp(1j * m))
    return PyramidGeometry(res=res, n_subap=n_subap, n_pix_separation=n_pix_separation,
                           n_pix_edge=n_pix_edge, psf_centering=psf_centering, N=N, cam=cam,
                           center=N // 2, mask=mask, phasor=phasor, tip=tip, tilt=tilt)


def modulation_path(modulation: float, n_theta_user: int | None = None, extra: int = 0,
                    delta_theta: float = 0.0, delta_tip: float = 0.0, delta_tilt: float = 0.0,
                    user_path=None, length: float = 2 * np.pi):
    """Modulation points [K,2] in lambda/D, ``OOPAO/Pyramid.py:1112-1132``.

    Returns ``(path, n_theta)``; ``path`` is None for the non-modulated case
    (``:1151-1152``: nTheta = 1).
    """
    if modulation == 0 and user_path is None:
        return None, 1
    if user_path is not None:
        return np.asarray(user_path, dtype=np.float64), len(user_path)
    perimeter = length * modulation
    if n_theta_user is None:
        n_theta = 4 * int((extra + np.ceil(perimeter / 4)))
    else:
        n_theta = n_theta_user
    theta = np.linspace(0 + delta_theta, 2 * np.pi + delta_theta, n_theta, endpoint=False)
    path = [[modulation * np.cos(t) + delta_tip, modulation * np.sin(t) + delta_tilt] for t in theta]
    return np.asarray(path, dtype=np.float64), n_theta


def tt_buffers(path, geom: PyramidGeometry) -> np.ndarray:
    """Per-point tip/tilt phase, float32 [K,res,res], ``OOPAO/Pyramid.py:1133-1139``."""
    if path is None:
        return np.zeros((1, geom.res, geom.res), dtype=np.float32)
    out = np.zeros((len(path), geom.res, geom.res), dtype=np.float32)
    for i, (px, py) in enumerate(path):
        out[i] = (px * geom.tip + py * geom.tilt)
    return out


# ---------------------------------------------------------------------------
# Propagation
# ---------------------------------------------------------------------------

def pyramid_transform_stack(phase_pts: np.ndarray, amplitude: np.ndarray,
                            geom: PyramidGeometry, workers: int = 1,
                            spatial_filter=None) -> np.ndarray:
    """Detector-plane intensity for a stack of per-point pupil phases.

    ``phase_pts`` [P,res,res] holds ``phase + TT_k`` for P (mode, point)
    pairs.  Follows ``OOPAO/Pyramid.py:612-646``: E = A*exp(i*phase) placed
    in the centre of an NxN zero array, ``F = fft2(E*phasor)`` (psfCentering)
    or ``fftshift(fft2(E))[*spatialFilter]``, ``G = ifft2(F*mask)``, |G|^2.
    Returns float64 [P,N,N].
    """
    N, res, c = geom.N, geom.res, geom.center
    lo = c - res // 2
    P = phase_pts.shape[0]
    if spatial_filter is None:
        spatial_filter = geom.spatial_filter
    support = np.zeros((P, N, N), dtype=np.complex128)
    support[:, lo:lo + res, lo:lo + res] = amplitude[None] * np.exp(1j * phase_pts)
    if geom.psf_centering:
        F = scipy.fft.fft2(support * geom.phasor[None], axes=(1, 2), workers=workers)
    else:
        F = np.fft.fftshift(scipy.fft.fft2(support, axes=(1, 2), workers=workers), axes=(1, 2))
        if spatial_filter is not None:
            F = F * spatial_filter[None]
    G = scipy.fft.ifft2(F * geom.mask[None], axes=(1, 2), workers=workers)
    return np.abs(G) ** 2


def focal_plane_image(phase: np.ndarray, intensity: np.ndarray, tt: np.ndarray, geom: PyramidGeometry) -> np.ndarray:
    """Intensity the focal-plane camera reads for a phase map: sum over the
    modulation points of |F_k / N|^2, F_k the focal field of
    ``pyramid_transform`` before the mask (``OOPAO/Pyramid.py:629-642``,
    summed by ``Pyramid.__mul__`` ``:1182-1185``)."""
    N, res, c = geom.N, geom.res, geom.center
    lo = c - res // 2
    K = tt.shape[0]
    amp = np.sqrt(intensity / K)
    out = np.zeros((N, N))
    for k in range(K):
        support = np.zeros((N, N), dtype=np.complex128)
        support[lo:lo + res, lo:lo + res] = amp * np.exp(1j * (phase + tt[k].astype(np.float64)))
        if geom.psf_centering:
            F = scipy.fft.fft2(support * geom.phasor)
        else:
            F = np.fft.fftshift(scipy.fft.fft2(support))
            if geom.spatial_filter is not None:
                F = F * geom.spatial_filter
        out += np.abs(F / N) ** 2
    return out


def wfs_raw(phase: np.ndarray, intensity: np.ndarray, tt: np.ndarray, geom: PyramidGeometry,
            weight_vector=None, workers: int = 1, chunk: int = 16) -> np.ndarray:
    """``raw_data`` for one phase map or a cube [res,res,B].

    ``OOPAO/Pyramid.py:666-833``: maskAmplitude = sqrt(intensity/nTheta)
    (``:674``); 2-D input: raw = sum_k I_k (``:741-751``) or the weighted
    variant (``:753-755``); 3-D input: per-mode sums over that mode's K
    points (``:758-824``).  Returns [N,N] or [B,N,N].
    """
    K = tt.shape[0]
    amp = np.sqrt(intensity / K)
    single = phase.ndim == 2
    cube = phase[..., None] if single else phase
    B = cube.shape[2]
    out = np.zeros((B, geom.N, geom.N))
    if workers > 1 and weight_vector is None:
        # one modulation point per task on a thread pool, as the reference's
        # joblib 'threads' backend does (OOPAO/Pyramid.py:741-746)
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(workers) as ex:
            for b in range(B):
                ph = cube[:, :, b]
                maps = ex.map(lambda k: pyramid_transform_stack(
                    (ph + tt[k].astype(np.float64))[None], amp, geom, workers=1)[0], range(K))
                acc = np.zeros((geom.N, geom.N))
                for m in maps:
                    acc += m
                out[b] = acc
        return out[0] if single else out
    for b in range(B):
        acc = np.zeros((geom.N, geom.N))
        maps = []
        for k0 in range(0, K, chunk):
            pts = cube[:, :, b][None] + tt[k0:k0 + chunk].astype(np.float64)
            I = pyramid_transform_stack(pts, amp, geom, workers=workers)
            if weight_vector is None:
                acc += I.sum(axis=0)
            else:
                maps.append(I)
        if weight_vector is not None:
            maps = np.concatenate(maps).reshape(K, -1)
            acc = (np.diag(weight_vector) @ maps).sum(axis=0).reshape(geom.N, geom.N) / K
        out[b] = acc
    return out[0] if single else out


def set_binning(array: np.ndarray, binning_factor: float) -> np.ndarray:
    """Sum binning, ``OOPAO/tools/tools.py:464-483`` (2-D case)."""
    if array.shape[0] % binning_factor != 0:
        raise ValueError('Binning factor %d not compatible with the array size' % binning_factor)
    n0 = int(np.round(array.shape[0] / binning_factor))
    n1 = int(np.round(array.shape[1] / binning_factor))
    shape = (n0, array.shape[0] // n0, n1, array.shape[1] // n1)
    return array.reshape(shape).sum(-1).sum(1)


def camera_frame(raw: np.ndarray, geom: PyramidGeometry, qe: float = 1.0, gain: float = 1.0) -> np.ndarray:
    """Noise-free camera frame: ``Pyramid.__mul__`` binning
    (``OOPAO/Pyramid.py:1178-1203``) then ``Detector.integrate``/``readout``
    with noise off (``OOPAO/Detector.py:331-354``, ``:273-329``)."""
    frame = set_binning(raw, geom.N / geom.cam)
    frame = frame * qe
    frame = np.sum([frame], axis=0)
    frame = frame * gain
    return frame.astype(float)


def grab_quadrant(frame: np.ndarray, n: int, geom: PyramidGeometry) -> np.ndarray:
    """Pupil-image quadrant ``n`` of the camera frame, ``OOPAO/Pyramid.py:946-961``."""
    res, ns, b = geom.res, geom.n_subap, geom.binning
    nE = int(np.round((geom.n_pix_separation / ns) * res / (res / ns) / 2 / b))
    cp = int(np.round((geom.cam / b) / 2))
    npx = int(np.ceil(ns / b))
    if n == 3:
        return frame[nE + cp:nE + cp + npx, nE + cp:nE + cp + npx]
    if n == 4:
        return frame[nE + cp:nE + cp + npx, -nE + cp - npx:-nE + cp]
    if n == 1:
        return frame[-nE + cp - npx:-nE + cp, -nE + cp - npx:-nE + cp]
    if n == 2:
        return frame[-nE + cp - npx:-nE + cp, nE + cp:nE + cp + npx]
    raise ValueError(n)


def valid_pixels(frame: np.ndarray, geom: PyramidGeometry, light_ratio: float):
    """Flux-based valid-pixel map, ``OOPAO/Pyramid.py:541-589`` (slopesMaps)."""
    I4Q = sum(grab_quadrant(frame, n, geom) for n in (1, 2, 3, 4))
    valid = I4Q >= light_ratio * I4Q.max()
    return valid, I4Q


def slopes_maps(frame: np.ndarray, geom: PyramidGeometry, valid_i4q: np.ndarray,
                reference_2d=0.0, slopes_units=1.0):
    """``signalProcessing`` 'slopesMaps' branch, ``OOPAO/Pyramid.py:838-854``.

    Returns (signal_2D [2n,n], signal [nSignal], norma)."""
    I = [grab_quadrant(frame, n, geom) * valid_i4q for n in (1, 2, 3, 4)]
    I1, I2, I3, I4 = I
    I4Q = I1 + I2 + I3 + I4
    norma = np.mean(I4Q[valid_i4q])
    Sx = (I1 - I2 + I4 - I3)
    Sy = (I1 - I4 + I2 - I3)
    maps = (np.concatenate((Sx, Sy) / norma) - reference_2d) * slopes_units
    valid_signal = np.concatenate((valid_i4q, valid_i4q))
    return maps, maps[np.where(valid_signal == 1)], norma


def full_frame(frame: np.ndarray, valid_signal: np.ndarray, reference_2d=0.0):
    """``signalProcessing`` 'fullFrame' branch, ``OOPAO/Pyramid.py:918-926``."""
    norma = np.sum(frame[valid_signal])
    maps = (frame / norma) - reference_2d
    return maps, maps[np.where(valid_signal == 1)], norma


# ---------------------------------------------------------------------------
# A complete sensor (construction sequence of Pyramid.__init__)
# ---------------------------------------------------------------------------

@dataclass
class OraclePyramid:
    geom: PyramidGeometry
    intensity: np.ndarray
    tt: np.ndarray
    valid_i4q: np.ndarray
    reference_2d: np.ndarray
    n_theta: int
    path: object
    calib_tt: np.ndarray

    @property
    def valid_signal(self):
        return np.concatenate((self.valid_i4q, self.valid_i4q))

    def measure(self, phase: np.ndarray, workers: int = 1):
        """Phase [res,res] or [res,res,B] -> (raw, frame, signal_2D, signal)."""
        raw = wfs_raw(phase, self.intensity, self.tt, self.geom, workers=workers)
        if raw.ndim == 2:
            frame = camera_frame(raw, self.geom)
            s2d, s, _ = slopes_maps(frame, self.geom, self.valid_i4q, self.reference_2d)
            return raw, frame, s2d, s
        frames, s2ds, ss = [], [], []
        for b in range(raw.shape[0]):
            f = camera_frame(raw[b], self.geom)
            s2d, s, _ = slopes_maps(f, self.geom, self.valid_i4q, self.reference_2d)
            frames.append(f), s2ds.append(s2d), ss.append(s)
        return raw, np.stack(frames), np.stack(s2ds, axis=-1), np.stack(ss, axis=-1)


def build_pyramid(res: int, n_subap: int, modulation: float, light_ratio: float,
                  intensity: np.ndarray, n_pix_separation: float = 2,
                  n_pix_edge=None, psf_centering: bool = True, calib_modulation: float = 50.,
                  n_theta_user: int | None = None, extra: int = 0, delta_theta: float = 0.,
                  rooftop: float = 0., theta_rotation: float = 0., user_path=None,
                  workers: int = 1, spatial_filter=None, old_mask: bool = False,
                  user_valid=None) -> OraclePyramid:
    """Construction sequence of ``Pyramid.__init__`` (``OOPAO/Pyramid.py:26-366``):
    geometry, calibration modulation clamp (``:292-296``), valid pixels at
    ``calibModulation`` (``initialization`` ``:541-589``), flat-wavefront
    reference slopes (``wfs_calibration`` ``:591-610``).  With
    ``spatial_filter``, the filter is then attached as the ``spatialFilter``
    setter does (``:1051-1085``): the mask is filtered and the reference
    slopes are measured again; the valid pixels stay those of the
    unfiltered initialization.  ``user_valid`` (``userValidSignal``,
    slopes maps) replaces the flux selection (``:574-580``)."""
    geom = pyramid_geometry(res, n_subap, n_pix_separation, n_pix_edge, psf_centering,
                            rooftop, theta_rotation, old_mask=old_mask)
    if calib_modulation >= res / 2:
        calib_modulation = res / 2 - 1
    flat = np.zeros((res, res))
    cpath, _ = modulation_path(calib_modulation, n_theta_user, extra, delta_theta, user_path=user_path)
    ctt = tt_buffers(cpath, geom)
    if user_valid is not None:
        valid = np.asarray(user_valid, dtype=bool)
    else:
        if light_ratio == 0:
            frame0 = np.ones((geom.cam, geom.cam))
        else:
            raw0 = wfs_raw(flat, intensity, ctt, geom, workers=workers)
            frame0 = camera_frame(raw0, geom)
        valid, _ = valid_pixels(frame0, geom, light_ratio)
    path, n_theta = modulation_path(modulation, n_theta_user, extra, delta_theta, user_path=user_path)
    tt = tt_buffers(path, geom)
    if spatial_filter is not None:
        geom = with_spatial_filter(geom, spatial_filter)
    raw1 = wfs_raw(flat, intensity, tt, geom, workers=workers)
    frame1 = camera_frame(raw1, geom)
    ref2d, _, _ = slopes_maps(frame1, geom, valid, 0)
    return OraclePyramid(geom=geom, intensity=intensity, tt=tt, valid_i4q=valid,
                         reference_2d=ref2d, n_theta=n_theta, path=path, calib_tt=ctt)


# ---------------------------------------------------------------------------
# Calibration
# ---------------------------------------------------------------------------

def interaction_matrix(wfs: OraclePyramid, modes: np.ndarray, m2c: np.ndarray, stroke: float,
                       wavelength: float, pupil: np.ndarray, single_pass: bool = True,
                       workers: int = 1) -> np.ndarray:
    """``InteractionMatrix`` column rule, ``OOPAO/calibration/InteractionMatrix.py:99-167``:
    push (and pull) through DM -> pupil mask -> phase -> WFS; column =
    factor*0.5*(s+ - s-)/stroke with factor 2 and s- = 0 when single_pass."""
    res = wfs.geom.res
    cols = []
    for m in range(m2c.shape[1]):
        opd = dm_opd(modes, m2c[:, m] * stroke, res) * pupil
        sp = wfs.measure(opd * 2 * np.pi / wavelength, workers=workers)[3]
        if single_pass:
            cols.append(2 * 0.5 * sp / stroke)
        else:
            opd = dm_opd(modes, -m2c[:, m] * stroke, res) * pupil
            sm = wfs.measure(opd * 2 * np.pi / wavelength, workers=workers)[3]
            cols.append(0.5 * (sp - sm) / stroke)
    return np.stack(cols, axis=1)


def calibration_vault(D: np.ndarray, n_trunc: int = 0):
    """SVD pseudo-inverse, ``OOPAO/calibration/CalibrationVault.py:44-70``.
    Returns (M, Mtrunc, s, cond)."""
    U, s, V = np.linalg.svd(D, full_matrices=False)
    M = V.T @ np.diag(1 / s) @ U.T
    ne = len(s) - n_trunc
    Mtrunc = V[:ne, :].T @ np.diag(1 / s[:ne]) @ U.T[:ne, :]
    cond = s[0] / s[-n_trunc - 1]
    return M, Mtrunc, s, cond


def rel_l2(a, b) -> float:
    """||a-b|| / ||b|| in float64."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ---------------------------------------------------------------------------
# Closed loop and science image (float64)
# ---------------------------------------------------------------------------

def science_psf(opd: np.ndarray, intensity: np.ndarray, pupil: np.ndarray, wavelength: float) -> np.ndarray:
    """On-axis ``Telescope.computePSF`` with zero padding 2 and an image of
    2*res pixels (``OOPAO/Telescope.py:251-420``): the field
    sqrt(I)*pupil*exp(i*2*pi*opd/lambda) zero-padded to N = 2 res (res/2 on
    each side), times exp(-i*pi*(N+1)/N*(x+y)), EMF = fft2(.)/N, PSF = |EMF|^2."""
    res = opd.shape[0]
    n2 = 2 * res
    lo = (n2 - res) // 2
    xx, yy = np.meshgrid(np.arange(n2), np.arange(n2))
    phasor = np.exp(-1j * np.pi * (n2 + 1) / n2 * (xx + yy))
    sup = np.zeros((n2, n2), dtype=np.complex128)
    sup[lo:lo + res, lo:lo + res] = np.sqrt(intensity) * pupil * np.exp(1j * 2 * np.pi / wavelength * opd)
    emf = np.fft.fft2(sup * phasor) / n2
    return np.abs(emf) ** 2


def strehl_meter(psf: np.ndarray, psf_ref: np.ndarray) -> float:
    """``strehlMeter`` (``OOPAO/tools/tools.py:102-157``) for images of equal
    size: sum of the max-normalised |OTF| over that of the reference, in %."""
    otf = np.abs(np.fft.fftshift(np.fft.fft2(psf)))
    otfa = np.abs(np.fft.fftshift(np.fft.fft2(psf_ref)))
    return float(np.sum(otf / np.max(otf)) / np.sum(otfa / np.max(otfa)) * 100)


def closed_loop(wfs: OraclePyramid, modes: np.ndarray, reconstructor: np.ndarray, turbulence_opd,
                pupil: np.ndarray, wavelength: float, gain: float, n_steps: int, frame_delay: int = 1,
                science: bool = True, workers: int = 1, record_signals: bool = False) -> dict:
    """The loop of ``tutorials/AO_closed_loop_Pyramid_WFS.py:601-639`` in
    float64: at step t the residual OPD = turbulence_opd(t) + modes @ coefs;
    its standard deviation over the pupil is logged; the sensor measures it;
    coefs -= gain * R @ s_t (frame delay 1) or R @ s_{t-1} (delay 2).  With
    ``science``, the science PSF of every residual is summed and the
    long-exposure Strehl ratio is returned with the flat-wavefront PSF.  With
    ``record_signals``, the slopes of every step are returned too."""
    res = pupil.shape[0]
    coefs = np.zeros(modes.shape[1])
    s_prev = np.zeros(reconstructor.shape[1])
    ip = pupil > 0
    wfe = np.zeros(n_steps)
    psf_le = 0.0
    signals = []
    for t in range(n_steps):
        opd = turbulence_opd(t) + (modes @ coefs).reshape(res, res)
        wfe[t] = np.std(opd[ip])
        if science:
            psf_le = psf_le + science_psf(opd, wfs.intensity, pupil, wavelength)
        _, _, _, s = wfs.measure(opd * 2 * np.pi / wavelength, workers=workers)
        if record_signals:
            signals.append(s)
        if frame_delay == 1:
            coefs = coefs - gain * reconstructor @ s
        else:
            coefs = coefs - gain * reconstructor @ s_prev
            s_prev = s
    out = {'wfe': wfe, 'coefs': coefs}
    if record_signals:
        out['signals'] = np.stack(signals)
    if science:
        ref = science_psf(np.zeros((res, res)), wfs.intensity, pupil, wavelength)
        out.update(psf_le=psf_le, psf_ref=ref, strehl_le=strehl_meter(psf_le, ref))
    return out
