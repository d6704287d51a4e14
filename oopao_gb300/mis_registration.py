"""DM mis-registration: drop-in for the reference ``MisRegistration``
(``OOPAO/MisRegistration.py``).

Six parameters move the actuator grid of a DeformableMirror and reshape its
Gaussian influence functions: a rotation (degrees), shifts along x and y
(metres), and an anamorphosis (a stretch of the grid and of each IF along the
direction ``anamorphosisAngle``, by ``radialScaling`` along it and
``tangentialScaling`` across it, both fractions: 0.01 is 1 %).
"""
from .tools import OopaoError

_FIELDS = ('rotationAngle', 'shiftX', 'shiftY', 'anamorphosisAngle', 'tangentialScaling', 'radialScaling')


class MisRegistration:
    """Mis-registration parameters (``OOPAO/MisRegistration.py:11-73``): built
    empty, from a dict holding the six keys, or as a copy of another
    MisRegistration.  ``+`` and ``-`` combine two of them field by field
    (``:75-102``)."""

    def __init__(self, param=None):
        self.tag = 'misRegistration'
        for f in _FIELDS:
            setattr(self, f, 0)
        if param is None:
            return
        if isinstance(param, dict):
            for f in _FIELDS:
                setattr(self, f, param[f])
        elif getattr(param, 'tag', None) == 'misRegistration':
            for f in _FIELDS:
                setattr(self, f, getattr(param, f))
        else:
            print('wrong type of object passed to a MisRegistration object')

    @property
    def misRegName(self):
        """Name of the mis-registration used by the reference for file names
        (``:60-73``): two decimals, four for the scalings when one is set."""
        d = 2 if self.radialScaling == 0 and self.tangentialScaling == 0 else 4
        return ('rot_%.2f_sX_%.2f_m_sY_%.2f_m_anam_%.2f_mR_%.*f_mT_%.*f'
                % (self.rotationAngle, self.shiftX, self.shiftY, self.anamorphosisAngle,
                   d, self.radialScaling + 1., d, self.tangentialScaling + 1.))

    def _combine(self, other, sign):
        if getattr(other, 'tag', None) != 'misRegistration':
            raise OopaoError('A MisRegistration combines only with another MisRegistration')
        out = MisRegistration()
        for f in _FIELDS:
            setattr(out, f, getattr(self, f) + sign * getattr(other, f))
        return out

    def __add__(self, other):
        return self._combine(other, 1)

    def __sub__(self, other):
        return self._combine(other, -1)

    def __eq__(self, other):
        return isinstance(other, MisRegistration) and all(getattr(self, f) == getattr(other, f) for f in _FIELDS)

    def __ne__(self, other):
        return not self.__eq__(other)

    def properties(self) -> dict:
        self.prop = {
            'rotation': f"{'Rotation [°]':<25s}|{self.rotationAngle:^9.3f}",
            'shift_x': f"{'Shift X [m]':<25s}|{self.shiftX:^9.3e}",
            'shift_y': f"{'Shift Y [m]':<25s}|{self.shiftY:^9.3e}",
            'anamophosis_angle': f"{'Anamorphosis angle [°]':<25s}|{self.anamorphosisAngle:^9.3f}",
            'tengential_scaling': f"{'Tangential scaling [%]':<25s}|{self.tangentialScaling * 100:^9.3f}",
            'radial_scaling': f"{'Radial scaling [%]':<25s}|{self.radialScaling * 100:^9.3f}",
        }
        return self.prop

    def print_properties(self):
        print(self)

    def __repr__(self):
        rows = list(self.properties().values())
        n = len(max(rows))
        return f'\n{"Misregistration":-^{n}}\n' + ''.join(r + '\n' for r in rows) + f'{"":-^{n}}\n'
