"""Import the unmodified OOPAO reference in a container that lacks its display
and I/O dependencies.

Used only by ``make_golden.py`` (fixture generation) where the reference
source tree is present.  The tests never import it: they read the fixtures.

Recipe:
  * the package writes ``precision_oopao.npy`` into the shortest ``sys.path``
    entry containing "OOPAO" (``OOPAO/__init__.py:55-60``), so the source tree
    is copied to a writable directory whose name contains "OOPAO";
  * matplotlib, astropy, jsonpickle and skimage are replaced by no-op stub
    modules.  None of them is used by the Pyramid / DeformableMirror /
    Detector / InteractionMatrix path (display and FITS/JSON I/O only; skimage
    is used by the atmosphere screen shift only).
"""
import importlib
import os
import shutil
import sys
import types


class _Anything:
    """Callable, attribute-able, iterable no-op used for every stubbed symbol."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()

    def __iter__(self):
        return iter(())

    def __mro_entries__(self, bases):
        return (object,)


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith('__'):
            raise AttributeError(name)
        return _Anything()


_STUBS = [
    'matplotlib', 'matplotlib.pyplot', 'matplotlib.gridspec', 'matplotlib.offsetbox',
    'matplotlib.backends', 'matplotlib.backends.backend_tkagg', 'matplotlib.colors',
    'astropy', 'astropy.io', 'astropy.io.fits', 'jsonpickle',
    'skimage', 'skimage.transform',
]


def install_kl_shims():
    """Numerical stand-ins for the three accelerators the reference's KL basis
    imports (``OOPAO/calibration/ao_cockpit_psim.py:13-22``): numba.jit as the
    identity, pyfftw's in-place FFTW object as numpy's fftn, and
    numexpr.evaluate as numpy evaluation of the expression in the caller's
    scope.  They change how the arithmetic is scheduled, not what it is."""
    import numpy as np

    numba = types.ModuleType('numba')

    def jit(*a, **k):
        if a and callable(a[0]) and len(a) == 1 and not k:
            return a[0]
        return lambda f: f
    numba.jit = numba.njit = jit
    numba.prange = range
    sys.modules['numba'] = numba

    pyfftw = types.ModuleType('pyfftw')
    pyfftw.empty_aligned = lambda shape, dtype='complex128', n=None: np.empty(shape, dtype=dtype)

    class FFTW:
        def __init__(self, a, b, axes=(-1,), flags=(), direction='FFTW_FORWARD', threads=1):
            self.a, self.b, self.axes, self.direction = a, b, axes, direction

        def __call__(self):
            f = np.fft.fftn if self.direction == 'FFTW_FORWARD' else np.fft.ifftn
            self.b[...] = f(self.a, axes=self.axes)
            return self.b
    pyfftw.FFTW = FFTW
    sys.modules['pyfftw'] = pyfftw

    numexpr = types.ModuleType('numexpr')

    def evaluate(expr, local_dict=None, global_dict=None, **k):
        frame = sys._getframe(1)
        scope = dict(frame.f_globals)
        scope.update(frame.f_locals if local_dict is None else local_dict)
        scope.update(complex=lambda a, b: np.asarray(a) + 1j * np.asarray(b), conj=np.conj)
        return np.asarray(eval(expr, {'__builtins__': {}}, scope))
    numexpr.evaluate = evaluate
    sys.modules['numexpr'] = numexpr


def import_reference(ref_root, work=None):
    """Return the imported ``OOPAO`` package from a stubbed copy of ``ref_root``
    (the reference project root, which holds ``OOPAO/``).  The copy goes to a
    fresh temporary directory (or to `work`, which must not exist yet), so a
    copy of older reference sources is never reused."""
    if 'OOPAO' in sys.modules:
        return sys.modules['OOPAO']
    if not ref_root or not os.path.isdir(os.path.join(ref_root, 'OOPAO')):
        raise SystemExit('reference project root without an OOPAO/ package: %r' % (ref_root,))
    if work is None:
        import tempfile
        work = tempfile.mkdtemp(prefix='OOPAO_refcopy_')
    dst = os.path.join(work, 'OOPAO')
    if os.path.exists(dst):
        raise SystemExit('%s exists: give a fresh directory' % dst)
    os.makedirs(work, exist_ok=True)
    shutil.copytree(os.path.join(ref_root, 'OOPAO'), dst)
    for root, dirs, files in os.walk(dst):
        os.chmod(root, 0o755)
        for f in files:
            os.chmod(os.path.join(root, f), 0o644)
    for name in _STUBS:
        if name not in sys.modules:
            sys.modules[name] = _StubModule(name)
    sys.modules['astropy.io'].fits = sys.modules['astropy.io.fits']
    # the atmosphere's sub-pixel shift needs a working warp (see skimage_emulation)
    import skimage_emulation
    sys.modules['skimage.transform'] = skimage_emulation
    sys.modules['skimage'].transform = skimage_emulation
    sys.modules['matplotlib'].pyplot = sys.modules['matplotlib.pyplot']
    sys.modules['matplotlib'].gridspec = sys.modules['matplotlib.gridspec']
    if work not in sys.path:
        sys.path.insert(0, work)
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        mod = importlib.import_module('OOPAO')
    return mod
