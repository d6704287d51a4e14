"""Autotuner for the pyramid propagation and the DM projection.

Pyramid (``tune_pyramid``): when the sensor's mask factorises per axis the
two-pass propagation runs, and the candidates are its compile-time plans
(radix order, columns per CTA: ``oopao_pwfs_num_separable``) times the
number of partial slots over the modulation points (the points each
column-pass CTA sums, i.e. the work per CTA); otherwise the candidates are
the three-pass compile-time plans (radix split N = R1*R2, threads per
line, lines per CTA: ``oopao_pwfs_variant_info``) plus the generic
runtime-planned kernels.  DM (``tune_dm``): the cut-over batch between the
separable projection and the BF16 tensor-core GEMM, and the GEMM's batch
tile (64 or 128 columns) per batch.  Every candidate is timed on the
object's own sizes with CUDA events and the fastest kept.  Results are
cached in a JSON file (``$OOPAO_GB300_AUTOTUNE_CACHE``, default
``~/.cache/oopao_gb300/autotune.json``) keyed by GPU and sizes, so later
runs reuse the choice without timing.
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


def _time_call(fn, reps):
    for _ in range(2):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _divisors(k, cap=64):
    return [d for d in range(1, min(k, cap) + 1) if k % d == 0]


def tune_two_pass(wfs, batch, reps=5, seed=0, verbose=False):
    """Time every (two-pass plan, slot count) of the sensor at `batch`;
    returns {(plan, slots): ms} with slots 0 = the library's model."""
    h = wfs.plan.h
    g = torch.Generator(device=wfs._dev).manual_seed(seed)
    res = wfs.telescope.resolution
    opd = torch.randn((batch, res, res), device=wfs._dev, generator=g) * 1e-7
    scale = 2 * np.pi / wfs.src.wavelength
    times = {}
    for sp in range(1, N.call('oopao_pwfs_num_separable', h) + 1):
        if N.load().oopao_pwfs_set_separable(h, sp) != 0:
            continue
        for ks in [0] + _divisors(wfs.nTheta):
            N.call('oopao_pwfs_set_launch', h, 0, 0, 0, ks)
            times[(sp, ks)] = _time_call(lambda: wfs._measure_frames(opd, scale), reps)
            if verbose:
                print('two-pass plan %d, slots %d: %.3f ms' % (sp, ks, times[(sp, ks)]))
    N.call('oopao_pwfs_set_launch', h, 0, 0, 0, 0)
    return times


def tune_pyramid(wfs, batch=1, reps=5, force=False, verbose=False):
    """Select the fastest propagation for this sensor and batch size.
    Returns {'variant': v, 'ms': {v: ms}} (and, on the two-pass path,
    'two_pass': {'plan', 'slots', 'ms'}) and leaves the plan on the winner."""
    cache = _load()
    key = _key(wfs, batch)
    h = wfs.plan.h
    if not force and key in cache:
        e = cache[key]
        v = int(e['variant'])
        if v <= N.load().oopao_pwfs_num_variants(h):
            N.call('oopao_pwfs_set_variant', h, v)
            tp = e.get('two_pass')
            if tp and N.call('oopao_pwfs_separable', h) == 1 and \
                    N.load().oopao_pwfs_set_separable(h, int(tp['plan'])) == 0:
                N.call('oopao_pwfs_set_launch', h, 0, 0, 0, int(tp['slots']))
            return e
    if N.call('oopao_pwfs_separable', h) == 1:
        # the two passes run: the three-pass variants do not matter, keep the default one
        v = N.call('oopao_pwfs_get_variant', h)
        t2 = tune_two_pass(wfs, batch, reps, verbose=verbose)
        (sp, ks) = min(t2, key=t2.get)
        N.call('oopao_pwfs_set_separable', h, sp)
        N.call('oopao_pwfs_set_launch', h, 0, 0, 0, ks)
        entry = {'variant': v, 'ms': {str(v): t2[(sp, ks)]},
                 'two_pass': {'plan': sp, 'slots': ks, 'ms': {'%d/%d' % k: t for k, t in t2.items()}}}
        cache[key] = entry
        _save(cache)
        return entry
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


def _dm_key(dm, batch):
    name = torch.cuda.get_device_name(dm._dev).replace(' ', '_')
    return 'dm|%s|res%d|act%d|%s|B%s' % (name, dm.resolution, dm.nValidAct, dm.if_dtype, batch)


def tune_dm(dm, batches=(1, 4, 16, 32, 64, 128, 300), reps=5, force=False, verbose=False):
    """Choose the DM's projection path per batch size: the separable
    projection (Gaussian IFs that factorise) against the BF16 tensor-core
    GEMM with the library's tile rule or a 64- or 128-column batch tile
    (if_dtype='bf16'); for FP32 IFs without factors, the CUDA-core FP32 GEMM
    against the FP32-accuracy tensor-core GEMM (three TF32 products).  Sets
    dm.separable_max_batch (the largest timed batch the separable projection
    wins, when it wins every smaller one), dm.tc_tile_rule and
    dm.tf32_min_batch (the smallest timed batch from which the TF32 GEMM wins
    every larger one, None if it never does); returns {batch: {path: ms}}."""
    cache = _load()
    key = _dm_key(dm, ','.join(str(b) for b in batches))
    if not force and key in cache:
        e = cache[key]
        dm.separable_max_batch = int(e['separable_max_batch'])
        dm.tc_tile_rule = [tuple(r) for r in e['tc_tile_rule']]
        dm.tf32_min_batch = e.get('tf32_min_batch', dm.tf32_min_batch)
        return e['ms']
    has_sep = dm._sep is not None
    has_tc = dm._modes_bf16 is not None
    has_tf32 = not has_tc and not (has_sep and dm.separable_projection)
    saved = (dm.separable_projection, dm.separable_max_batch, list(dm.tc_tile_rule), dm.tf32_min_batch)
    out = {}
    g = torch.Generator(device=dm._dev).manual_seed(0)
    for B in batches:
        c = torch.randn((dm.nValidAct, B), device=dm._dev, generator=g) * 1e-8
        row = {}
        if has_sep:
            dm.separable_projection, dm.separable_max_batch = True, 1 << 30
            row['separable'] = _time_call(lambda: dm.opd_device(c), reps)
        if has_tc:
            dm.separable_projection = False
            for tile in (0, 64, 128):   # 0: the library's rule (a GEMV up to 4 columns)
                dm.tc_tile_rule = [(1 << 30, tile)]
                row['bf16_%d' % tile] = _time_call(lambda: dm.opd_device(c), reps)
        if has_tf32:
            for key, first in (('fp32', None), ('tf32', 1)):
                dm.tf32_min_batch = first
                row[key] = _time_call(lambda: dm.opd_device(c), reps)
        out[B] = row
        if verbose:
            print('B=%d' % B, row)
    dm.separable_projection = saved[0]
    sep_max = saved[1]
    if has_sep and has_tc:
        sep_max = 0
        for B in batches:
            r = out[B]
            if r['separable'] <= min(r['bf16_0'], r['bf16_64'], r['bf16_128']):
                sep_max = B
            else:
                break
        if sep_max == batches[-1]:
            sep_max = 1 << 30   # the separable projection won every timed batch
    rule = []
    if has_tc:
        for B in batches:
            r = out[B]
            rule.append((B, min((0, 64, 128), key=lambda t: r['bf16_%d' % t])))
        rule.append((1 << 30, rule[-1][1]))
    tf32_min = saved[3]
    if has_tf32:
        tf32_min = None
        for B in reversed(batches):
            if out[B]['tf32'] < out[B]['fp32']:
                tf32_min = B
            else:
                break
    dm.separable_max_batch = sep_max
    dm.tc_tile_rule = rule
    dm.tf32_min_batch = tf32_min
    cache[key] = {'separable_max_batch': sep_max, 'tc_tile_rule': rule, 'tf32_min_batch': tf32_min,
                  'ms': {str(b): r for b, r in out.items()}}
    _save(cache)
    return out
