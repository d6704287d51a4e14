"""oopao_gb300: GB300-native modulated pyramid WFS and DM influence-function
projection behind the cheritier/OOPAO operator surface.

    from oopao_gb300 import Telescope, Source, DeformableMirror, Pyramid
    ngs * tel
    dm = DeformableMirror(tel, nSubap=20)
    wfs = Pyramid(nSubap=20, telescope=tel, modulation=3, lightRatio=0.5)
    dm.coefs = c
    ngs ** tel * dm * wfs
    wfs.signal, wfs.signal_2D, wfs.cam.frame

The compute path is the CUDA library ``_lib/liboopao_gb300.so`` (built by
``python -m oopao_gb300.build``); importing the classes does not need a GPU,
constructing a DeformableMirror or Pyramid does.
"""
from .tools import OopaoError, warning
from .source import Source
from .telescope import Telescope
from .detector import Detector
from .deformable_mirror import DeformableMirror
from .mis_registration import MisRegistration
from .pyramid import Pyramid
from .calibration import InteractionMatrix, CalibrationVault
from .atmosphere import Atmosphere
from .bioedge import BioEdge
from .gain_sensing import GainSensingCamera

__all__ = ['OopaoError', 'warning', 'Source', 'Telescope', 'Detector', 'DeformableMirror', 'Pyramid',
           'InteractionMatrix', 'CalibrationVault', 'Atmosphere', 'BioEdge', 'GainSensingCamera',
           'MisRegistration']
