"""Write radix_consts.cuh: cos/sin(2*pi*t/R) for the in-register DFT kernels.

The values are the mathematical constants, evaluated in float64 by Python's
math module and rounded to float32 literals.  Run by the package build step.
Lookups use compile-time (R, t) so the switch folds to a literal.
"""
import math
import os
import sys

RADICES = tuple(range(2, 65))


def render():
    lines = ['// Generated by gen_radix_consts.py: cos/sin(2*pi*t/R) rounded to float.',
             '#pragma once', '']
    for fn, f in (('rad_cos', math.cos), ('rad_sin', math.sin)):
        lines.append('__device__ __forceinline__ constexpr float %s(int R, int t) {' % fn)
        lines.append('  switch (R * 128 + t) {')
        for R in RADICES:
            for t in range(R):
                v = f(2 * math.pi * t / R)
                if abs(v) < 1e-15:
                    v = 0.0
                lines.append('    case %d: return %.9ef;' % (R * 128 + t, v))
        lines.append('    default: return 0.0f;')
        lines.append('  }')
        lines.append('}')
        lines.append('')
    return '\n'.join(lines)


def main(out=None):
    out = out or os.path.join(os.path.dirname(os.path.abspath(__file__)), 'radix_consts.cuh')
    txt = render()
    old = open(out).read() if os.path.exists(out) else None
    if old != txt:
        with open(out, 'w') as fh:
            fh.write(txt)
    return out


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else None)
