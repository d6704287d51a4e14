"""Generate golden vectors by running the unmodified OOPAO reference.

Run in a container that holds the reference source tree:

    python tests/golden/make_golden.py /path/to/OOPAO/project [case ...]

(or with the project root in the environment variable OOPAO_REFERENCE).

It imports the reference through ``refimport.import_reference`` (display and
I/O dependencies stubbed), builds Telescope / Source / DeformableMirror /
Pyramid objects exactly as a user script does, propagates seeded inputs with
``ngs**tel*dm*wfs`` (or ``wfs.wfs_measure``), and stores inputs and outputs
in ``tests/golden/<case>.npz``.  The reference always computes in float64.

Inputs are stored in the fixtures (rather than regenerated from seeds) so the
tests never depend on a random-number stream.
"""
import contextlib
import io
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


def screen(res, seed, rms_rad):
    """Seeded smooth random phase map (power-law spectrum), rms in radians."""
    rng = np.random.default_rng(seed)
    f = np.fft.fftfreq(res)
    fx, fy = np.meshgrid(f, f)
    fr = np.sqrt(fx ** 2 + fy ** 2)
    fr[0, 0] = 1.0
    spec = fr ** (-11 / 6)
    spec[0, 0] = 0
    ph = np.real(np.fft.ifft2(spec * (rng.standard_normal((res, res)) + 1j * rng.standard_normal((res, res)))))
    ph -= ph.mean()
    return ph / ph.std() * rms_rad


def build(OOPAO, res, n_subap, modulation, light_ratio, co=0.0, diameter=8.0, **wfs_kw):
    from OOPAO.Telescope import Telescope
    from OOPAO.Source import Source
    from OOPAO.DeformableMirror import DeformableMirror
    from OOPAO.Pyramid import Pyramid
    with _quiet():
        tel = Telescope(resolution=res, diameter=diameter, samplingTime=1e-3, centralObstruction=co)
        ngs = Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = DeformableMirror(tel, nSubap=n_subap, mechCoupling=0.35)
        wfs = Pyramid(nSubap=n_subap, telescope=tel, modulation=modulation, lightRatio=light_ratio,
                      **wfs_kw)
    return tel, ngs, dm, wfs


def measure_dm(tel, ngs, dm, wfs, coefs):
    with _quiet():
        dm.coefs = coefs
        ngs ** tel * dm * wfs
        # focal-plane (modulation) camera of the same measurement
        wfs * wfs.focal_plane_camera
    return dict(raw=np.array(wfs.raw_data), frame=np.array(wfs.cam.frame),
                signal=np.array(wfs.signal), signal_2D=np.array(wfs.signal_2D),
                phase=np.array(ngs.phase),
                focal=np.sum(np.abs(np.asarray(wfs.modulation_camera_em)) ** 2, axis=0),
                focal_cam=np.array(wfs.focal_plane_camera.frame))


def measure_phase(tel, ngs, dm, wfs, phase):
    with _quiet():
        dm.coefs = 0
        ngs ** tel
        wfs.wfs_measure(phase_in=phase)
    return dict(raw=np.array(wfs.raw_data), frame=np.array(wfs.cam.frame),
                signal=np.array(wfs.signal), signal_2D=np.array(wfs.signal_2D))


def geometry_record(tel, ngs, dm, wfs):
    return dict(
        pupil=np.array(tel.pupil), intensity=np.array(ngs.intensity), wavelength=ngs.wavelength,
        N=wfs.resolution, cam=wfs.cam.resolution, n_theta=wfs.nTheta, n_signal=wfs.nSignal,
        valid_i4q=np.array(wfs.validI4Q), reference_2d=np.array(wfs.referenceSignal_2D),
        n_act=dm.nValidAct, modulation_path=np.array(wfs.modulation_path if wfs.modulation != 0 or wfs.user_modulation_path is not None else np.zeros((1, 2))),
    )


def circular_filter(n, radius, centred_on_pixel):
    """Top-hat focal-plane filter of `radius` pixels around the PSF centre
    (pixel n/2 for the 1-pixel-centred mask, the 4-pixel corner otherwise)."""
    c = n / 2 if centred_on_pixel else (n - 1) / 2
    yy, xx = np.mgrid[:n, :n]
    return (np.hypot(xx - c, yy - c) <= radius).astype(np.float64)


def case_small(OOPAO, name, res, n_subap, modulation, light_ratio, co=0.0, full=True, n_im=6,
               seeds=(1, 2), sf_radius=None, **kw):
    tel, ngs, dm, wfs = build(OOPAO, res, n_subap, modulation, light_ratio, co=co, **kw)
    import json
    params = dict(res=res, n_subap=n_subap, modulation=modulation, light_ratio=light_ratio, co=co, **kw)
    filt = None
    if sf_radius is not None:
        # attached after construction through the reference's own setter,
        # which filters the mask and re-measures the reference slopes
        filt = circular_filter(wfs.mask.shape[0], sf_radius, not kw.get('psfCentering', True))
        with _quiet():
            wfs.spatialFilter = filt
        params['sf_radius'] = sf_radius
    rec = geometry_record(tel, ngs, dm, wfs)
    if filt is not None:
        rec['spatial_filter'] = filt
    rec['params'] = json.dumps(params)
    if full and res <= 32:
        rec['mask'] = np.array(wfs.mask)
        rec['tt'] = np.array(wfs.phaseBuffModulationLowres) if wfs.modulation != 0 else np.zeros((1, res, res), np.float32)
        rec['phasor'] = np.array(wfs.phasor)
        rec['modes'] = np.array(dm.modes)
    rng = np.random.default_rng(seeds[0])
    coefs = rng.standard_normal(dm.nValidAct) * 60e-9
    out = measure_dm(tel, ngs, dm, wfs, coefs)
    rec['dm_coefs'] = coefs
    for k, v in out.items():
        if k == 'raw' and not full:
            continue
        rec['dm_' + k] = v
    ph = screen(res, seeds[1], 2.0) * tel.pupil
    out = measure_phase(tel, ngs, dm, wfs, ph)
    rec['screen_phase'] = ph
    for k, v in out.items():
        if k == 'raw' and not full:
            continue
        rec['screen_' + k] = v
    if n_im:
        from OOPAO.calibration.InteractionMatrix import InteractionMatrix
        m2c = np.eye(dm.nValidAct)[:, :n_im]
        with _quiet():
            calib = InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=4,
                                      single_pass=True)
            calib_pp = InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=1,
                                         single_pass=False)
        rec['im_m2c'] = m2c
        rec['im_D'] = np.array(calib.D)
        rec['im_M'] = np.array(calib.M)
        rec['im_pp_D'] = np.array(calib_pp.D)
    if not full or res > 32:
        # influence-function summaries (the full matrix is too large to store)
        rec['modes_colsum'] = dm.modes.sum(axis=0)
        rec['modes_col0'] = dm.modes[:, 0]
        rec['modes_sq'] = float((dm.modes ** 2).sum())
        rec['mask_real_sum'] = float(np.real(wfs.mask).astype(np.float64).sum())
        rec['mask_imag_sum'] = float(np.imag(wfs.mask).astype(np.float64).sum())
        rec['mask_row0'] = np.array(wfs.mask[0])
        rec['mask_col_mid'] = np.array(wfs.mask[:, wfs.resolution // 2 - 3])
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'N', rec['N'], 'cam', rec['cam'], 'K', rec['n_theta'], 'nSignal', rec['n_signal'],
          'nAct', rec['n_act'])


ATM_CASE = dict(res=32, diameter=8.0, r0=0.15, L0=25.0, fractionalR0=[0.5, 0.3, 0.2],
                windSpeed=[10.0, 370.0, 300.0], windDirection=[0.0, 135.0, 30.0],
                altitude=[0.0, 5000.0, 10000.0], steps=40)


# boiling (AR(1) decorrelation): a still layer that boils, a fast diagonal
# layer that boils, a slow layer that does not
ATM_BOIL_CASE = dict(name='atm_boil', windSpeed=[0.0, 370.0, 10.0], windDirection=[0.0, 135.0, 30.0],
                     t_boiling=[0.01, 0.005, None], steps=20)


def case_atmosphere(OOPAO, name='atm_small', **p):
    """Infinite-screen atmosphere: OPD seen by an on-axis NGS after each of
    `steps` updates (the wind speeds are large so that every branch of the
    integer-step logic of updateLayer runs: axis-aligned sub-pixel drift, a
    diagonal layer moving more than one pixel per step, unequal components)."""
    import json
    from OOPAO.Atmosphere import Atmosphere
    from OOPAO.Source import Source
    from OOPAO.Telescope import Telescope
    p = dict(ATM_CASE, **p)
    with _quiet():
        tel = Telescope(resolution=p['res'], diameter=p['diameter'], samplingTime=1e-3)
        ngs = Source(optBand='V0', magnitude=8)
        ngs * tel
        extra = {'t_boiling': p['t_boiling']} if p.get('t_boiling') is not None else {}
        atm = Atmosphere(telescope=tel, r0=p['r0'], L0=p['L0'], fractionalR0=p['fractionalR0'],
                         windSpeed=p['windSpeed'], windDirection=p['windDirection'], altitude=p['altitude'],
                         **extra)
        atm.initializeAtmosphere(tel)
        opds = []
        ngs ** atm * tel
        opds.append(np.array(ngs.OPD_no_pupil))
        for _ in range(p['steps']):
            atm.update()
            ngs ** atm * tel
            opds.append(np.array(ngs.OPD_no_pupil))
    layer = atm.layer_1
    rec = dict(params=json.dumps(p), opd=np.stack(opds), A=np.array(layer.A), B=np.array(layer.B),
               screen0=np.array(atm.layer_1.initial_OPD))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'steps', p['steps'], 'A', layer.A.shape, 'B', layer.B.shape)


def case_large(OOPAO, name='c5_screen'):
    """80x80 pyramid on a 39 m, 480 px pupil (N = 1920 with n_pix_separation
    80, n_pix_edge 40; 320x320 camera; modulation 4 l/D with 128 points):
    geometry, valid pixels, reference slopes and one seeded screen measured
    through wfs_measure.  No DM (its 230400 x 5209 float64 IF matrix is not
    needed for the sensor)."""
    import json
    from OOPAO.Pyramid import Pyramid
    from OOPAO.Source import Source
    from OOPAO.Telescope import Telescope
    p = dict(res=480, diameter=39.0, n_subap=80, modulation=4, light_ratio=0.5, n_pix_separation=80,
             n_pix_edge=40, nTheta_user_defined=128)
    with _quiet():
        tel = Telescope(resolution=p['res'], diameter=p['diameter'], samplingTime=1e-3)
        ngs = Source(optBand='V0', magnitude=8)
        ngs * tel
        wfs = Pyramid(nSubap=p['n_subap'], telescope=tel, modulation=p['modulation'], lightRatio=p['light_ratio'],
                      n_pix_separation=p['n_pix_separation'], n_pix_edge=p['n_pix_edge'],
                      nTheta_user_defined=p['nTheta_user_defined'])
        ph = screen(p['res'], 5, 2.0) * tel.pupil
        ngs ** tel
        wfs.wfs_measure(phase_in=ph)
    rec = dict(params=json.dumps(p), pupil=np.array(tel.pupil), intensity=np.array(ngs.intensity),
               wavelength=ngs.wavelength, N=wfs.resolution, cam=wfs.cam.resolution, n_theta=wfs.nTheta,
               n_signal=wfs.nSignal, valid_i4q=np.array(wfs.validI4Q), reference_2d=np.array(wfs.referenceSignal_2D),
               screen_phase=ph, screen_frame=np.array(wfs.cam.frame), screen_signal=np.array(wfs.signal),
               screen_signal_2D=np.array(wfs.signal_2D))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'N', rec['N'], 'cam', rec['cam'], 'K', rec['n_theta'], 'nSignal', rec['n_signal'])


def case_bioedge(OOPAO, name, res, n_subap, modulation, light_ratio, seeds=(3, 4), n_im=4, **kw):
    """Bi-O Edge sensor: masks, geometry, valid pixels, reference slopes, a DM
    measurement, a screen measurement and push-pull IM columns."""
    import json
    from OOPAO.BioEdge import BioEdge
    from OOPAO.DeformableMirror import DeformableMirror
    from OOPAO.Source import Source
    from OOPAO.Telescope import Telescope
    with _quiet():
        tel = Telescope(resolution=res, diameter=8.0, samplingTime=1e-3)
        ngs = Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = DeformableMirror(tel, nSubap=n_subap, mechCoupling=0.35)
        wfs = BioEdge(nSubap=n_subap, telescope=tel, modulation=modulation, lightRatio=light_ratio, **kw)
    rec = dict(params=json.dumps(dict(res=res, n_subap=n_subap, modulation=modulation, light_ratio=light_ratio,
                                      **kw)),
               masks=np.array(wfs.mask), N=wfs.resolution, cam=wfs.cam.resolution, n_theta=wfs.nTheta,
               n_signal=wfs.nSignal, valid_i4q=np.array(wfs.validI4Q), reference_2d=np.array(wfs.referenceSignal_2D),
               intensity=np.array(ngs.intensity), pupil=np.array(tel.pupil), wavelength=ngs.wavelength)
    coefs = np.random.default_rng(seeds[0]).standard_normal(dm.nValidAct) * 60e-9
    with _quiet():
        dm.coefs = coefs
        ngs ** tel * dm * wfs
    rec.update(dm_coefs=coefs, dm_phase=np.array(ngs.phase), dm_raw=np.array(wfs.raw_data),
               dm_frame=np.array(wfs.cam.frame), dm_signal=np.array(wfs.signal), dm_signal_2D=np.array(wfs.signal_2D))
    # focal-plane (modulation) camera of the same measurement: the reference
    # keeps each point's field once per mask (BioEdge.py:435-443, :1036-1044)
    with _quiet():
        wfs * wfs.focal_plane_camera
    rec.update(dm_focal=np.sum(np.abs(np.asarray(wfs.modulation_camera_em)) ** 2, axis=0),
               dm_focal_cam=np.array(wfs.focal_plane_camera.frame), n_focal_fields=len(wfs.modulation_camera_em))
    ph = screen(res, seeds[1], 2.0) * tel.pupil
    with _quiet():
        dm.coefs = 0
        ngs ** tel
        wfs.wfs_measure(phase_in=ph)
    rec.update(screen_phase=ph, screen_frame=np.array(wfs.cam.frame), screen_signal=np.array(wfs.signal))
    if n_im:
        from OOPAO.calibration.InteractionMatrix import InteractionMatrix
        m2c = np.eye(dm.nValidAct)[:, :n_im]
        with _quiet():
            calib = InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=1, single_pass=False)
        rec.update(im_m2c=m2c, im_pp_D=np.array(calib.D))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'N', rec['N'], 'cam', rec['cam'], 'K', rec['n_theta'], 'nSignal', rec['n_signal'])


KL_CASES = [('kl_tiny', dict(res=24, n_subap=4)), ('kl_c1', dict(res=120, n_subap=20))]


def case_kl(OOPAO, name, res, n_subap, r0=0.15, L0=25.0):
    """KL modal basis of the reference (compute_KL_basis, lim 1e-3, piston
    removed) for a Gaussian-IF DM, with its input IFs summarised."""
    import json
    from OOPAO.Atmosphere import Atmosphere
    from OOPAO.DeformableMirror import DeformableMirror
    from OOPAO.Source import Source
    from OOPAO.Telescope import Telescope
    from OOPAO.calibration.compute_KL_modal_basis import compute_KL_basis
    with _quiet():
        tel = Telescope(resolution=res, diameter=8.0, samplingTime=1e-3)
        ngs = Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = DeformableMirror(tel, nSubap=n_subap, mechCoupling=0.35)
        atm = Atmosphere(telescope=tel, r0=r0, L0=L0, fractionalR0=[1.0], windSpeed=[10.], windDirection=[0.],
                         altitude=[0.])
        m2c = compute_KL_basis(tel, atm, dm, lim=1e-3, remove_piston=True)
    rec = dict(params=json.dumps(dict(res=res, n_subap=n_subap, r0=r0, L0=L0)), m2c=np.asarray(m2c),
               n_act=dm.nValidAct)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'M2C', rec['m2c'].shape)


def case_c3(OOPAO, name='c3', n_kl=24, r0=0.12, L0=30.0):
    """The 40x40 closed-loop optics: 8 m, 240 px, 40x40 pyramid, modulation
    5 l/D with 96 points, N = 504, 84x84 camera, 41x41 Gaussian DM (coupling
    0.35).  Geometry, valid pixels, reference slopes, one DM shape and one
    seeded screen measured through the reference's own Pyramid, and push-pull
    interaction-matrix columns (stroke 1e-8, nMeasurements 1) of the first
    `n_kl` modes of the reference's compute_KL_basis (r0 0.12 m, L0 30 m,
    lim 1e-3, piston removed).  The 504 x 504 focal image is not stored."""
    import json
    from refimport import install_kl_shims
    install_kl_shims()
    from OOPAO.Atmosphere import Atmosphere
    from OOPAO.calibration.InteractionMatrix import InteractionMatrix
    from OOPAO.calibration.compute_KL_modal_basis import compute_KL_basis
    res, n_subap, modulation, light_ratio = 240, 40, 5, 0.5
    tel, ngs, dm, wfs = build(OOPAO, res, n_subap, modulation, light_ratio, nTheta_user_defined=96)
    rec = geometry_record(tel, ngs, dm, wfs)
    rec['params'] = json.dumps(dict(res=res, n_subap=n_subap, modulation=modulation, light_ratio=light_ratio,
                                    nTheta_user_defined=96, n_kl=n_kl, r0=r0, L0=L0))
    coefs = np.random.default_rng(31).standard_normal(dm.nValidAct) * 60e-9
    out = measure_dm(tel, ngs, dm, wfs, coefs)
    rec['dm_coefs'] = coefs
    for k, v in out.items():
        if k not in ('raw', 'focal'):
            rec['dm_' + k] = v
    ph = screen(res, 32, 2.0) * tel.pupil
    out = measure_phase(tel, ngs, dm, wfs, ph)
    rec['screen_phase'] = ph
    for k, v in out.items():
        if k != 'raw':
            rec['screen_' + k] = v
    with _quiet():
        atm = Atmosphere(telescope=tel, r0=r0, L0=L0, fractionalR0=[1.0], windSpeed=[10.], windDirection=[0.],
                         altitude=[0.])
        m2c = np.asarray(compute_KL_basis(tel, atm, dm, lim=1e-3, remove_piston=True))[:, :n_kl]
        dm.coefs = 0
        ngs ** tel
        calib_pp = InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=1,
                                     single_pass=False)
        # the float64 derivative: the same push-pull with a stroke 1000x
        # smaller, whose O(stroke^2) truncation is ~1e-6 of the 1e-8 m one
        calib_fine = InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-11, nMeasurements=1,
                                       single_pass=False)
    rec['im_m2c'] = m2c
    rec['im_pp_D'] = np.array(calib_pp.D)
    rec['im_fine_D'] = np.array(calib_fine.D)
    rec['modes_colsum'] = dm.modes.sum(axis=0)
    rec['modes_sq'] = float((dm.modes ** 2).sum())
    rec['mask_row0'] = np.array(wfs.mask[0])
    rec['mask_col_mid'] = np.array(wfs.mask[:, wfs.resolution // 2 - 3])
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'N', rec['N'], 'cam', rec['cam'], 'K', rec['n_theta'], 'nSignal', rec['n_signal'],
          'nAct', rec['n_act'], 'IM', rec['im_pp_D'].shape)


POSTPROCESSING_MODES = ['slopesMaps', 'slopesMaps_incidence_flux', 'slopesMaps_camera_flux', 'fullFrame_camera_flux',
                        'fullFrame_incidence_flux', 'fullFrame_sum_flux', 'fullFrame']


def case_modes(OOPAO, name='modes_tiny', res=24, n_subap=4, modulation=3, light_ratio=0.5, seed=5):
    """Every postProcessing normalisation of signalProcessing (OOPAO/Pyramid.py
    :835-926) on one DM shape, plus the detector binning (binning=2, the
    Pyramid.__mul__ rebin, :1195-1201) with slopesMaps."""
    import json
    rng = np.random.default_rng(seed)
    rec = {}
    coefs = None
    for mode in POSTPROCESSING_MODES + ['binning2']:
        kw = dict(binning=2) if mode == 'binning2' else dict(postProcessing=mode)
        tel, ngs, dm, wfs = build(OOPAO, res, n_subap, modulation, light_ratio, **kw)
        if coefs is None:
            coefs = rng.standard_normal(dm.nValidAct) * 60e-9
        with _quiet():
            dm.coefs = coefs
            ngs ** tel * dm * wfs
        rec[mode + '_signal'] = np.array(wfs.signal)
        rec[mode + '_signal_2D'] = np.array(wfs.signal_2D)
        rec[mode + '_frame'] = np.array(wfs.cam.frame)
        rec[mode + '_n_signal'] = wfs.nSignal
    rec['coefs'] = coefs
    rec['params'] = json.dumps(dict(res=res, n_subap=n_subap, modulation=modulation, light_ratio=light_ratio,
                                    modes=POSTPROCESSING_MODES))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, [(m, int(rec[m + '_n_signal'])) for m in POSTPROCESSING_MODES + ['binning2']])


# Constructor options and post-construction calls of the Pyramid and Bi-O Edge
# operators: (name, sensor, constructor keywords, calls).  A call is
# ('call', method, keywords) or ('set', attribute, value); the values
# 'corner' (userValidSignal) and 'ramp' (weight_vector) are arrays the
# generator and the test build the same way (options_array below).
OPTION_CASES = [
    ('old_mask', 'pyramid', dict(old_mask=True), []),
    ('old_mask_nocenter', 'pyramid', dict(old_mask=True, psfCentering=False, modulation=2), []),
    ('shift', 'pyramid', {}, [('call', 'apply_shift_wfs', dict(sx=[1, -1, 0.5, 0], sy=[0, 0.5, -1, 1]))]),
    ('shift_old_metres', 'pyramid', dict(old_mask=True),
     [('call', 'apply_shift_wfs', dict(sx=0.5, sy=-0.25, units='m'))]),
    ('shift_nocenter', 'pyramid', dict(psfCentering=False),
     [('call', 'apply_shift_wfs', dict(sx=[0.5, 0, -0.5, 1], sy=[1, -1, 0, 0.5]))]),
    # a grid of points as in the reference's closed-loop tutorial, with the
    # modulation radius non-zero (with modulation 0 the reference's
    # single-wavefront path drops the source phase, Pyramid.py:617-618)
    ('user_path', 'pyramid', dict(user_modulation_path=[[x, y] for x in (-2, 0, 2) for y in (-2, 0, 2)] + [[1, 0.5]]),
     []),
    ('delta_extra', 'pyramid', dict(delta_theta=0.3, extraModulationFactor=1), []),
    ('user_valid', 'pyramid', dict(userValidSignal='corner'), []),
    ('user_valid_fullframe', 'pyramid', dict(userValidSignal='corner', postProcessing='fullFrame'), []),
    ('setters', 'pyramid', {}, [('set', 'modulation', 2), ('set', 'lightRatio', 0.2), ('set', 'delta_Tip', 0.5),
                                ('set', 'delta_Tilt', -0.25)]),
    ('weights', 'pyramid', {}, [('set', 'weight_vector', 'ramp')]),
    ('bioedge_shift', 'bioedge', {}, [('call', 'apply_shift_wfs', dict(sx=[1, 0, -1, 0.5], sy=[0, 1, 0.5, -1]))]),
    ('bioedge_path_tip', 'bioedge', dict(delta_theta=0.2, extraModulationFactor=1),
     [('set', 'delta_Tip', 0.5), ('set', 'delta_Tilt', 0.25)]),
]


def options_array(tag, wfs=None, shape=None):
    """The arrays named in OPTION_CASES: 'corner' is a user valid-pixel map
    (every pixel but a 2-pixel corner block, of the valid-pixel map's shape),
    'ramp' a weight per modulation point, 0.5 .. 1.5."""
    if tag == 'corner':
        v = np.ones(shape, dtype=bool)
        v[0, 0] = False
        v[1, 2] = False
        return v
    if tag == 'ramp':
        return np.linspace(0.5, 1.5, wfs.nTheta)
    raise ValueError(tag)


def build_option_sensor(OOPAO, sensor, res, n_subap, modulation, light_ratio, kw):
    """Telescope, source, DM and the sensor of one OPTION_CASES entry."""
    from OOPAO.Telescope import Telescope
    from OOPAO.Source import Source
    from OOPAO.DeformableMirror import DeformableMirror
    kw = dict(kw)
    modulation = kw.pop('modulation', modulation)
    with _quiet():
        tel = Telescope(resolution=res, diameter=8.0, samplingTime=1e-3)
        ngs = Source(optBand='V0', magnitude=8)
        ngs * tel
        dm = DeformableMirror(tel, nSubap=n_subap, mechCoupling=0.35)
        if sensor == 'pyramid':
            from OOPAO.Pyramid import Pyramid as cls
        else:
            from OOPAO.BioEdge import BioEdge as cls
        if kw.get('userValidSignal') == 'corner':
            # the valid-pixel map's shape: one quadrant (slopes maps) or the
            # whole detector (full frame)
            probe = cls(nSubap=n_subap, telescope=tel, modulation=modulation, lightRatio=light_ratio,
                        postProcessing=kw.get('postProcessing', 'slopesMaps'))
            shape = np.shape(probe.validI4Q if kw.get('postProcessing', 'slopesMaps')[:10] == 'slopesMaps'
                             else probe.validSignal)
            kw['userValidSignal'] = options_array('corner', shape=shape)
        wfs = cls(nSubap=n_subap, telescope=tel, modulation=modulation, lightRatio=light_ratio, **kw)
    return tel, ngs, dm, wfs


def apply_option_calls(wfs, calls):
    with _quiet():
        for kind, name, val in calls:
            if kind == 'call':
                getattr(wfs, name)(**val)
            else:
                setattr(wfs, name, options_array(val, wfs) if isinstance(val, str) else val)


def case_options(OOPAO, name='options_tiny', res=24, n_subap=4, modulation=3, light_ratio=0.5, seed=9):
    """Constructor options (old_mask, psfCentering with the old mask,
    user_modulation_path, delta_theta, extraModulationFactor, userValidSignal)
    and post-construction calls (apply_shift_wfs in pixels and metres, the
    modulation / lightRatio / delta_Tip / delta_Tilt setters, weight_vector) of
    OOPAO/Pyramid.py and OOPAO/BioEdge.py, each with one DM shape and a batch
    of two DM shapes (the reference's 3-D phase path)."""
    import json
    rng = np.random.default_rng(seed)
    rec, coefs, coefs2 = {}, None, None
    for case, sensor, kw, calls in OPTION_CASES:
        tel, ngs, dm, wfs = build_option_sensor(OOPAO, sensor, res, n_subap, modulation, light_ratio, kw)
        apply_option_calls(wfs, calls)
        if coefs is None:
            coefs = rng.standard_normal(dm.nValidAct) * 60e-9
            coefs2 = rng.standard_normal((dm.nValidAct, 2)) * 60e-9
        with _quiet():
            dm.coefs = coefs
            ngs ** tel * dm * wfs
            rec[case + '_frame'] = np.array(wfs.cam.frame)
            rec[case + '_signal'] = np.array(wfs.signal)
            rec[case + '_signal_2D'] = np.array(wfs.signal_2D)
            dm.coefs = coefs2
            ngs ** tel * dm * wfs
            rec[case + '_batch_signal'] = np.array(wfs.signal)
        if 'userValidSignal' in kw:
            rec[case + '_user_valid'] = np.array(wfs.userValidSignal)
        rec[case + '_n_signal'] = int(wfs.nSignal)
        rec[case + '_n_theta'] = int(wfs.nTheta)
        rec[case + '_reference_2D'] = np.array(wfs.referenceSignal_2D)
        if wfs.modulation != 0 or wfs.user_modulation_path is not None:
            rec[case + '_modulation_path'] = np.array(wfs.modulation_path, dtype=np.float64)
    rec['coefs'], rec['coefs2'] = coefs, coefs2
    rec['params'] = json.dumps(dict(res=res, n_subap=n_subap, modulation=modulation, light_ratio=light_ratio,
                                    cases=OPTION_CASES))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, [(c, int(rec[c + '_n_signal']), int(rec[c + '_n_theta'])) for c, *_ in OPTION_CASES])


MISREG_CASES = {
    'rot_shift': dict(rotationAngle=3.0, shiftX=0.12, shiftY=-0.07, anamorphosisAngle=0.0, tangentialScaling=0.0,
                      radialScaling=0.0),
    'anamorphosis': dict(rotationAngle=-1.5, shiftX=-0.05, shiftY=0.03, anamorphosisAngle=30.0,
                         tangentialScaling=0.04, radialScaling=-0.03),
}


def case_misreg(OOPAO, name='misreg_tiny', res=24, n_subap=4, modulation=3, light_ratio=0.5, seed=11):
    """DeformableMirror with a MisRegistration (OOPAO/DeformableMirror.py
    :359-386, :559-600): actuator coordinates, influence functions and the
    pyramid measurement of one DM shape through the mis-registered mirror."""
    import json
    from OOPAO.DeformableMirror import DeformableMirror
    from OOPAO.MisRegistration import MisRegistration
    tel, ngs, dm0, wfs = build(OOPAO, res, n_subap, modulation, light_ratio)
    coefs = np.random.default_rng(seed).standard_normal(dm0.nValidAct) * 60e-9
    rec = dict(coefs=coefs)
    for tag, mr in MISREG_CASES.items():
        with _quiet():
            dm = DeformableMirror(tel, nSubap=n_subap, mechCoupling=0.35, misReg=MisRegistration(mr))
            dm.coefs = coefs
            ngs ** tel * dm * wfs
        rec[tag + '_coordinates'] = np.array(dm.coordinates)
        rec[tag + '_modes'] = np.array(dm.modes)
        rec[tag + '_frame'] = np.array(wfs.cam.frame)
        rec[tag + '_signal'] = np.array(wfs.signal)
        rec[tag + '_name'] = MisRegistration(mr).misRegName
    rec['params'] = json.dumps(dict(res=res, n_subap=n_subap, modulation=modulation, light_ratio=light_ratio,
                                    misreg=MISREG_CASES))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, {t: rec[t + '_modes'].shape for t in MISREG_CASES})


def case_im_offset(OOPAO, name='im_offset_tiny', res=24, n_subap=4, modulation=3, light_ratio=0.5, n_im=4,
                   seed=13):
    """InteractionMatrix with a phaseOffset, push-pull and single pass, in
    chunks of 2 modes (OOPAO/calibration/InteractionMatrix.py:13-169): the
    reference applies the offset to ngs.phase only after the pull is
    measured, so it leaves D unchanged.  (A last chunk of one mode makes its
    push-pull branch fail on the offset's shape, so the mode count is even.)"""
    import json
    from OOPAO.calibration.InteractionMatrix import InteractionMatrix
    tel, ngs, dm, wfs = build(OOPAO, res, n_subap, modulation, light_ratio)
    m2c = np.random.default_rng(seed).standard_normal((dm.nValidAct, n_im))
    offset = screen(res, seed + 1, 0.5) * tel.pupil
    rec = dict(m2c=m2c, offset=offset)
    with _quiet():
        for tag, kw in (('pp', dict(single_pass=False)), ('sp', dict(single_pass=True))):
            c0 = InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=2, nTrunc=1, **kw)
            c1 = InteractionMatrix(ngs, tel, dm, wfs, M2C=m2c, stroke=1e-8, nMeasurements=2, nTrunc=1,
                                   phaseOffset=offset, **kw)
            rec[tag + '_D'] = np.array(c0.D)
            rec[tag + '_D_offset'] = np.array(c1.D)
            rec[tag + '_Mtrunc'] = np.array(c1.Mtrunc)
    rec['params'] = json.dumps(dict(res=res, n_subap=n_subap, modulation=modulation, light_ratio=light_ratio,
                                    n_im=n_im))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'offset changes D by', float(np.abs(rec['pp_D_offset'] - rec['pp_D']).max()))


GSC_CASES = [('gsc_tiny', dict(res=24, n_subap=4, modulation=3, n_modes=12)),
             ('gsc_small', dict(res=40, n_subap=10, modulation=2, n_modes=40))]


def case_gsc(OOPAO, name, res, n_subap, modulation, n_modes, light_ratio=0.5, seed=7):
    """GainSensingCamera: calibration on the flat-wavefront focal-plane frame,
    optical gains on a screen, following the reference's GSC tutorial (basis =
    tel.OPD of a DM mode set, full-resolution focal-plane camera)."""
    import json
    from OOPAO.GainSensingCamera import GainSensingCamera
    tel, ngs, dm, wfs = build(OOPAO, res, n_subap, modulation, light_ratio)
    rng = np.random.default_rng(seed)
    m2c = rng.standard_normal((dm.nValidAct, n_modes)) * 20e-9
    with _quiet():
        dm.coefs = m2c
        ngs ** tel * dm
        basis = np.array(tel.OPD)
        dm.coefs = 0
        gsc = GainSensingCamera(mask=wfs.mask, basis=basis)
        wfs.focal_plane_camera.resolution = wfs.nRes
        ngs ** tel * wfs
        wfs * wfs.focal_plane_camera
        calib_frame = np.array(wfs.focal_plane_camera.frame)
        wfs.focal_plane_camera * gsc
    sky_opd = screen(res, seed + 1, 1.5) * tel.pupil * ngs.wavelength / (2 * np.pi)
    with _quiet():
        ngs ** tel
        # tel.OPD alone would be reset by the relay (OPD = OPD_no_pupil * pupil)
        tel.OPD_no_pupil = sky_opd
        tel * wfs
        wfs * wfs.focal_plane_camera
        sky_frame = np.array(wfs.focal_plane_camera.frame)
        wfs.focal_plane_camera * gsc
    rec = dict(params=json.dumps(dict(res=res, n_subap=n_subap, modulation=modulation, n_modes=n_modes,
                                      light_ratio=light_ratio)),
               m2c=m2c, basis=basis, mask=np.array(wfs.mask), sky_opd=sky_opd, calib_frame=calib_frame,
               sky_frame=sky_frame, ir_calib=np.array(gsc.IR_calib), ir_sky=np.array(gsc.IR_sky),
               sensi_calib=np.array(gsc.sensi_calib), og=np.array(gsc.og), N=wfs.resolution)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, 'N', rec['N'], 'modes', n_modes, 'og', rec['og'][:4])


DETECTOR_CASES = {
    # integration over 3 loop steps, saturation, CCD gain, 12-bit ADC (floating-point output)
    'int3_fwc_adc12': dict(integrationTime=3e-3, FWC=20000, bits=12, gain=2),
    # 16-bit ADC with a full well: unsigned 16-bit output clipped at 0
    'adc16_fwc': dict(bits=16, FWC=50000),
    # 8-bit ADC without full well: scaled by the frame maximum, unsigned 8-bit output
    'adc8_nofwc': dict(bits=8),
    # log scale and background-map removal, floating-point output
    'log_bg': dict(log_scale=True, gain=3),
    # CMOS with hardware binning (applied twice by the reference) and a gain
    'cmos_bin2': dict(sensor='CMOS', binning=2, gain=2),
    # integration over 2 steps, no other effect
    'int2_plain': dict(integrationTime=2e-3),
}


def case_detector(OOPAO, name='detector_tiny', n=12, steps=7, seed=13):
    """The reference Detector's integrate/readout on seeded frames, one loop
    step (1 ms) at a time as the sensor drives it (OOPAO/Pyramid.py:1179-1201),
    for settings without random draws; the camera frame after every step."""
    from OOPAO.Detector import Detector
    rng = np.random.default_rng(seed)
    frames = rng.exponential(4000.0, (steps, n, n))
    frames[:, 3, 4] = 30000.0   # a pixel above the full wells once summed
    bg = rng.uniform(0.0, 50.0, (n, n))
    rec = dict(frames=frames, bg=bg, dt=1e-3,
               params=json.dumps(dict(n=n, steps=steps, seed=seed, cases=DETECTOR_CASES)))
    for tag, kw in DETECTOR_CASES.items():
        with _quiet():
            det = Detector(nRes=n, **kw)
            if tag == 'log_bg':
                det.backgroundMap = bg
            out = []
            for i in range(steps):
                det._integrated_time += 1e-3
                det.integrate(frames[i].copy())
                out.append(np.array(det.frame, dtype=np.float64))
        rec[tag] = np.array(out)
        rec[tag + '_dtype'] = str(np.asarray(det.frame).dtype)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, {t: (rec[t].shape, rec[t + '_dtype']) for t in DETECTOR_CASES})


BIOEDGE_CASES = [
    ('bioedge_tiny', (24, 4, 3, 0.5), {}),
    ('bioedge_grey', (32, 4, 2, 0.3), dict(grey_width=1.0, quadrants_numbering=[2, 3, 0, 1], n_pix_separation=4,
                                           nTheta_user_defined=12)),
]


CASES = [
    ('tiny', (24, 4, 3, 0.5), {}),
    ('tiny_nocenter', (24, 4, 2, 0.5), dict(psfCentering=False, n_im=0)),
    ('tiny_rooftop', (24, 4, 2, 0.3), dict(rooftop=0.5, theta_rotation=0.1, nTheta_user_defined=8, n_im=0)),
    ('tiny_nomod', (32, 4, 0, 0.2), dict(co=0.25, n_im=0, n_pix_separation=4)),
    ('small_sep', (40, 10, 2, 0.5), dict(n_pix_separation=4, n_pix_edge=2, nTheta_user_defined=12, n_im=4)),
    ('c1', (120, 20, 3, 0.5), dict(full=False, n_im=3, nTheta_user_defined=48)),
    ('tiny_sf', (24, 4, 3, 0.5), dict(n_im=4, sf_radius=14)),
    ('tiny_nocenter_sf', (24, 4, 2, 0.5), dict(psfCentering=False, n_im=4, sf_radius=12)),
]


def main():
    """argv: reference project root (or $OOPAO_REFERENCE), then case names (default: every case)."""
    from refimport import import_reference
    args = sys.argv[1:]
    if args and os.path.isdir(os.path.join(args[0], 'OOPAO')):
        ref_root, only = args[0], set(args[1:])
    else:
        ref_root, only = os.environ.get('OOPAO_REFERENCE'), set(args)
    if not ref_root:
        raise SystemExit('usage: make_golden.py REFERENCE_ROOT [case ...] (or set OOPAO_REFERENCE)')
    OOPAO = import_reference(ref_root)
    for name, args, kw in CASES:
        if not only or name in only:
            case_small(OOPAO, name, *args, **kw)
    if not only or 'atm_small' in only:
        case_atmosphere(OOPAO)
    if not only or 'atm_boil' in only:
        case_atmosphere(OOPAO, **ATM_BOIL_CASE)
    if not only or 'c5_screen' in only:
        case_large(OOPAO)
    if not only or 'c3' in only:
        case_c3(OOPAO)
    for name, args, kw in BIOEDGE_CASES:
        if not only or name in only:
            case_bioedge(OOPAO, name, *args, **kw)
    for name, kw in GSC_CASES:
        if not only or name in only:
            case_gsc(OOPAO, name, **kw)
    if not only or 'modes_tiny' in only:
        case_modes(OOPAO)
    if not only or 'options_tiny' in only:
        case_options(OOPAO)
    if not only or 'misreg_tiny' in only:
        case_misreg(OOPAO)
    if not only or 'im_offset_tiny' in only:
        case_im_offset(OOPAO)
    if not only or 'detector_tiny' in only:
        case_detector(OOPAO)
    if not only or any(n in only for n, _ in KL_CASES):
        from refimport import install_kl_shims
        install_kl_shims()
        for name, kw in KL_CASES:
            if not only or name in only:
                case_kl(OOPAO, name, **kw)


if __name__ == '__main__':
    main()
