"""Build the in-tree CUDA library ``oopao_gb300/_lib/liboopao_gb300.so``.

One nvcc invocation per translation unit, run in parallel, then one link.
Target: GB300 only (``-gencode arch=compute_103a,code=sm_103a``).  Works on a
machine without a GPU (cross-compilation).  Usage:

    python -m oopao_gb300.build [--force] [--ptxas-verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
LIBDIR = os.path.join(HERE, '_lib')
OBJDIR = os.path.join(HERE, '_lib', 'obj')
LIBNAME = 'liboopao_gb300.so'
SOURCES = ['capi.cu', 'pwfs.cu', 'pwfs_sep.cu', 'dm.cu', 'dm_sep.cu', 'dm_tc.cu', 'cl.cu', 'atm.cu', 'gsc.cu', 'det.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc_path():
    cand = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(cand):
        raise RuntimeError('nvcc not found')
    return cand


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _deps_mtime():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(os.path.dirname(HERE), 'include', 'oopao_gb300.h'))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def build(force=False, verbose=False, ptxas_verbose=False):
    sys.path.insert(0, CSRC)
    try:
        import gen_radix_consts
        gen_radix_consts.main()
    finally:
        sys.path.pop(0)
    out = lib_path()
    if not force and os.path.exists(out) and os.path.getmtime(out) >= _deps_mtime():
        return out
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = nvcc_path()
    common = ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
                     '--expt-relaxed-constexpr', '-I', os.path.join(os.path.dirname(HERE), 'include')]
    if ptxas_verbose:
        common += ['-Xptxas', '-v']

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + '.o')
        cmd = [nvcc] + common + ['-c', os.path.join(CSRC, src), '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    for obj, log in results:
        if (verbose or ptxas_verbose) and log:
            print(log)
    tmp = out + '.tmp'
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + [o for o, _ in results] + ['-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (r.stdout, r.stderr))
    os.replace(tmp, out)
    return out


if __name__ == '__main__':
    p = build(force='--force' in sys.argv, verbose=True, ptxas_verbose='--ptxas-verbose' in sys.argv)
    print(p)
