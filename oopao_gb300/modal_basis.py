"""KL modal basis of a deformable mirror: drop-in for the reference's
``compute_KL_basis(tel, atm, dm, lim, remove_piston)``
(``OOPAO/calibration/compute_KL_modal_basis.py:14-35`` -> ``compute_M2C``).

The construction is the reference's:

* specific modes: piston, tip and tilt (Noll 1-3 on the pupil, mean-removed
  and unit-std, ``OOPAO/Zernike.py:17-66``) fitted by the influence functions
  through the truncated inverse of DELTA = IF^T IF and orthonormalised by a QR
  decomposition (``build_SpecificBasis_C``, ``ao_cockpit_psim.py:582-624``);
* seed basis: the DELTA-eigenmodes orthogonal to them (``build_SeedBasis_C``
  :659-690);
* KL modes: the seed basis rotated to diagonalise the covariance HHt of the
  influence functions' projections on von Karman turbulence
  (``build_KLBasis`` :724-760), HHt from the piston-removed von Karman PSD on
  a 2 res FFT grid (``VK_DSP_up`` :155-195, ``DO_HHt`` :847-1100).

HHt (O(n_act^2 res^2) work) is computed in float64 on the GPU with torch:
HHt = Re(F^H diag(PSD df^2) F), F the FFTs of the zero-padded influence
functions.  The O(n_act^3) steps run in float64 with numpy's LAPACK, the
routines the reference calls, so the modes come out with the reference's
signs (modes of equal variance span the same space; within such a cluster
the basis can differ by round-off-level rotations).
"""
import math

import numpy as np
import torch

from .tools import OopaoError


def _zernike_ptt(tel, j=3):
    """Noll modes 1..j on the pupil pixels [npup, j] (``zernike_tel`` with
    remove_piston=0)."""
    pupil = np.asarray(tel.pupil)
    res, D = tel.resolution, tel.D
    X, Y = np.where(pupil > 0)
    X = (X - (res + res % 2 - 1) / 2) / res * D
    Y = (Y - (res + res % 2 - 1) / 2) / res * D
    R = np.sqrt(X ** 2 + Y ** 2)
    R = R / R.max()
    theta = np.arctan2(Y, X)
    out = np.zeros((X.size, j))
    for i in range(j):
        jj = i + 1
        n = int((-1. + np.sqrt(8 * (jj - 1) + 1)) / 2.)
        p = jj - (n * (n + 1)) / 2.
        k = n % 2
        m = int((p + k) / 2.) * 2 - k
        if m != 0:
            m *= 1 if jj % 2 == 0 else -1
        rad = np.zeros(R.shape)
        mm = abs(m)
        for s in range(0, int((n - mm) / 2) + 1):
            rad += R ** (n - 2 * s) * ((-1) ** s) * math.factorial(n - s) / (
                math.factorial(s) * math.factorial(int(0.5 * (n + mm) - s)) * math.factorial(int(0.5 * (n - mm) - s)))
        if m == 0:
            Z = np.sqrt(n + 1) * rad
        elif m > 0:
            Z = np.sqrt(2 * (n + 1)) * rad * np.cos(m * theta)
        else:
            Z = np.sqrt(2 * (n + 1)) * rad * np.sin(mm * theta)
        if n != 0:
            Z = Z - Z.mean()
            Z = Z * (1 / np.std(Z))
        out[:, i] = Z
    return out


def _vk_psd(diameter, r0, L0, size, dim, pupil):
    """Piston-removed von Karman phase PSD on a size x size grid and its
    frequency step (``VK_DSP_up`` with Pcor=1)."""
    dom = pupil.shape[0]
    pad = np.zeros((size, size))
    pad[size // 2 - dom // 2:size // 2 + dom // 2, size // 2 - dom // 2:size // 2 + dom // 2] = pupil
    fmax = dim / diameter * 0.5
    if L0 == 0:
        L0 = 1.e6
    f = np.linspace(-size / 2, size / 2 - 1, size) / (size / 2) * fmax
    ffx, ffy = np.meshgrid(f, f)
    ffr = np.sqrt(ffx ** 2 + ffy ** 2)
    cst = (math.gamma(11. / 6.) ** 2 / (2. * np.pi ** (11. / 3.))) * (24. * math.gamma(6. / 5.) / 5.) ** (5. / 6.)
    pupils = np.roll(np.roll(pad, size // 2, 0), size // 2, 1)
    ft = np.fft.fft2(pupils)
    ft = np.roll(np.roll(ft, size // 2, 0), size // 2, 1)
    pterm = np.abs(ft) ** 2
    psd = (cst * r0 ** (-5 / 3) * (ffr ** 2 + (1. / L0) ** 2) ** (-11 / 6)) * (1. - pterm / np.max(pterm))
    df = abs(f[size // 2] - f[size // 2 - 1])
    return psd, df


def hht_matrix(if_2d, psd, df, size, device=None, block=64):
    """HHt [n_act, n_act] float64: covariance of the projections of the
    influence functions if_2d [n_act, res, res] (already times the pupil) on
    turbulence of PSD `psd` (centred), on a size x size FFT grid."""
    dev = torch.device(device) if device is not None else (
        torch.device('cuda') if torch.cuda.is_available() else torch.device('cpu'))
    n_act, res = if_2d.shape[0], if_2d.shape[1]
    w = torch.as_tensor(np.fft.fftshift(psd).reshape(-1) * df ** 2, dtype=torch.float64, device=dev)
    sw = torch.sqrt(w)
    cols = []
    lo = size // 2 - res // 2
    ifd = torch.as_tensor(if_2d, dtype=torch.float64, device=dev)
    for a0 in range(0, n_act, block):
        a1 = min(n_act, a0 + block)
        pad = torch.zeros((a1 - a0, size, size), dtype=torch.float64, device=dev)
        pad[:, lo:lo + res, lo:lo + res] = ifd[a0:a1]
        F = torch.fft.fft2(pad).reshape(a1 - a0, -1) * sw
        cols.append(F)
    F = torch.cat(cols)
    # Re(F^H diag(w) F) = Fr Fr^T + Fi Fi^T with the weights folded in
    out = F.real @ F.real.T + F.imag @ F.imag.T
    return out.cpu().numpy()


def _n_above(s, lim):
    """The reference's count: index of the last value above lim * max."""
    return int(np.max(np.where(s / np.max(s) > lim)))


def compute_KL_basis(tel, atm, dm, lim=1e-3, remove_piston=True, n_batch=1):
    """M2C [n_act, n_modes] of KL modes (piston first unless removed)."""
    if getattr(dm, 'isM4', False):
        raise OopaoError('M4 force-minimised KL bases are not supported by oopao_gb300')
    pupil = np.asarray(tel.pupil, dtype=np.float64)
    res = tel.resolution
    n_act = dm.nValidAct
    if_2d = np.moveaxis(np.asarray(dm.modes, dtype=np.float64).reshape(res, res, n_act) * pupil[:, :, None], -1, 0)
    size = int(2 * res)
    psd, df = _vk_psd(tel.D, atm.r0, atm.L0, size, res, pupil)
    HHt = hht_matrix(if_2d, psd, df, size)
    idx = np.where(pupil.reshape(-1) == 1)[0]
    IFma = if_2d.reshape(n_act, -1)[:, idx].T                     # [tpup, n_act]
    tpup = IFma.shape[0]
    Tspm = _zernike_ptt(tel, 3)                                   # [tpup, 3]
    DELTA = IFma.T @ IFma
    # specific modes (build_SpecificBasis_C, ortho)
    ud, sd, vdh = np.linalg.svd(DELTA)
    nmax = _n_above(sd, lim) if lim <= 1. else int(lim)
    mev = np.zeros((n_act, n_act))
    mev[0:nmax, 0:nmax] = np.diag(1. / sd[0:nmax])
    cmd = (vdh.T @ mev @ ud.T) @ IFma.T @ Tspm
    _, R = np.linalg.qr(IFma @ cmd)
    SpM = cmd @ np.linalg.inv(R) * np.sqrt(tpup)
    # seed basis (build_SeedBasis_C)
    G = np.eye(n_act) - SpM @ np.linalg.inv(SpM.T @ DELTA @ SpM) @ SpM.T @ DELTA
    Mp, D2, _ = np.linalg.svd(G.T @ DELTA @ G)
    nmax = _n_above(D2, lim) if lim <= 1 else int(lim)
    if lim == 0.:
        nmax = n_act - SpM.shape[1]
    SB = G @ (Mp[:, 0:nmax] @ np.diag(np.sqrt(1. / D2[0:nmax])) * np.sqrt(tpup))
    # KL rotation (build_KLBasis)
    dsb_inv = np.linalg.inv(SB.T @ DELTA @ SB)
    Cp = dsb_inv @ SB.T @ HHt @ SB @ dsb_inv.T
    _, Sc, VcT = np.linalg.svd(Cp)
    KL = SB @ VcT.T
    basis = np.concatenate([SpM, KL], axis=1)
    if remove_piston:
        basis = basis[:, 1:]
    compute_KL_basis.last_variances = Sc
    return np.asarray(basis)
