"""Error type, warnings and small host helpers shared by the drop-in classes.

Mirrors ``OopaoError`` / ``warning`` of the reference
(``OOPAO/tools/tools.py:558-570``): errors raise ``OopaoError(str)`` and
warnings are printed.
"""
import numpy as np


class OopaoError(Exception):
    """Error raised by oopao_gb300 objects (same role as the reference's)."""

    def __init__(self, string):
        self.string = string
        self.message = string
        super().__init__(string)


def warning(string):
    print('\033[01m\033[33m' + 'OOPAO Warning: \n' + string + '\033[0m')


def print_(text, condition=True):
    if condition:
        print(text)


def set_binning(array, binning_factor, mode='sum'):
    """Host sum/mean binning of a 2-D map (``OOPAO/tools/tools.py:464-483``)."""
    if array.shape[0] % binning_factor != 0:
        raise ValueError('Binning factor %d not compatible with the array size' % binning_factor)
    n0 = int(np.round(array.shape[0] / binning_factor))
    n1 = int(np.round(array.shape[1] / binning_factor))
    shape = (n0, array.shape[0] // n0, n1, array.shape[1] // n1)
    if mode == 'sum':
        return array.reshape(shape).sum(-1).sum(1)
    return array.reshape(shape).mean(-1).mean(1)
