"""Import the unmodified OOPAO reference in a container that lacks its display
and I/O dependencies.

Used only by ``make_golden.py`` (fixture generation) where the reference
source tree is present.  Nothing here runs on a GPU machine.

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


def import_reference(ref_root='/root/reference', work='/tmp/OOPAO_refcopy'):
    """Return the imported ``OOPAO`` package from a stubbed copy of ``ref_root``."""
    if 'OOPAO' in sys.modules:
        return sys.modules['OOPAO']
    dst = os.path.join(work, 'OOPAO')
    if not os.path.isdir(dst):
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
