"""Autotuner for the pyramid propagation kernels.

Each FFT size has several compile-time plans (radix split N = R1*R2,
threads per line, lines per CTA of the three passes; see
``oopao_pwfs_variant_info``) plus the generic runtime-planned kernels.
``tune_pyramid`` times every candidate on the sensor's own plan and batch
size with CUDA events and keeps the fastest.  Results are cached in a JSON
file (``$OOPAO_GB300_AUTOTUNE_CACHE``, default
``~/.cache/oopao_gb300/autotune.json``) keyed by GPU, grid, modulation
points and batch, so later runs reuse the choice without timing.
"""
import json
import os

import numpy as np
import torch

from . import _native as N


def cache_path():
    return os.environ.get('OOPAO_GB300_AUTOTUNE_CACHE',
                          os.path.join(os.path.expanduser('~'), '.cache', 'oopao_gb300', 'autotune.json'))


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(d):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + '.tmp'
        with open(tmp, 'w') as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def _key(wfs, batch):
    name = torch.cuda.get_device_name(wfs._dev).replace(' ', '_')
    return '%s|N%d|res%d|K%d|cam%d|B%d' % (name, wfs.resolution, wfs.telescope.resolution, wfs.nTheta,
                                           wfs._cam_eff, batch)


def variants(wfs):
    """[(index, description)] of the candidate kernel variants of the sensor's plan."""
    h = wfs.plan.h
    lib = N.load()
    out = [(0, 'generic runtime-planned passes')]
    info = (N.ctypes.c_int * 6)()
    for v in range(1, lib.oopao_pwfs_num_variants(h) + 1):
        N.call('oopao_pwfs_variant_info', h, v, info)
        out.append((v, 'N=%d*%d, %d threads/line, lines per CTA %d/%d/%d' % tuple(info)))
    return out


def time_variant(wfs, variant, batch, reps=5, seed=0):
    """Average ms of one oopao_pwfs_measure call over `batch` random OPD maps."""
    h = wfs.plan.h
    N.call('oopao_pwfs_set_variant', h, variant)
    g = torch.Generator(device=wfs._dev).manual_seed(seed)
    res = wfs.telescope.resolution
    opd = torch.randn((batch, res, res), device=wfs._dev, generator=g) * 1e-7
    scale = 2 * np.pi / wfs.src.wavelength
    for _ in range(2):
        wfs._measure_frames(opd, scale)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        wfs._measure_frames(opd, scale)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_pyramid(wfs, batch=1, reps=5, force=False, verbose=False):
    """Select the fastest kernel variant for this sensor and batch size.
    Returns {'variant': v, 'ms': {v: ms}} and leaves the plan on the winner."""
    cache = _load()
    key = _key(wfs, batch)
    h = wfs.plan.h
    if not force and key in cache:
        v = int(cache[key]['variant'])
        if v <= N.load().oopao_pwfs_num_variants(h):
            N.call('oopao_pwfs_set_variant', h, v)
            return cache[key]
    times = {}
    for v, desc in variants(wfs):
        times[v] = time_variant(wfs, v, batch, reps)
        if verbose:
            print('variant %d (%s): %.3f ms' % (v, desc, times[v]))
    best = min(times, key=times.get)
    N.call('oopao_pwfs_set_variant', h, best)
    entry = {'variant': best, 'ms': {str(k): v for k, v in times.items()}}
    cache[key] = entry
    _save(cache)
    return entry
