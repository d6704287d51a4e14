"""The atmosphere's host planner (``Atmosphere._plan_one``: the one-pixel
moves of each layer and step, the sub-pixel remainder left in its buffer, the
extrusion normals drawn from each layer's RandomState) against the oracle's
replay of ``updateLayer`` (OOPAO/Atmosphere.py:447-514), step by step, without
a GPU.  The oracle is pinned to the reference's OPD sequence by
``test_oracle_atm.py``."""
import contextlib
import io

import numpy as np
import pytest
from numpy.random import RandomState

from oracle import atm_oracle as A

RES, D, DT = 32, 8.0, 1e-3

CASES = [
    # the golden's winds: still-ish axis drift, > 1 pixel per step diagonal, unequal components
    ([10.0, 370.0, 300.0], [0.0, 135.0, 30.0]),
    # a still layer, exact whole-pixel steps, directions on the axes and the diagonals
    ([0.0, 250.0, 125.0, 177.0], [45.0, 90.0, 180.0, 225.0]),
    # components just below and above one pixel per step, negative directions
    ([240.0, 260.0, 90.0], [-10.0, 300.0, 271.0]),
]


def _planner(ws, wd, seed=0):
    """An Atmosphere with the host state of initializeAtmosphere +
    generateNewPhaseScreen(seed), minus the device arrays the planner does not
    read (the generation's one extrusion draw per layer included)."""
    import oopao_gb300 as og
    from oopao_gb300 import atmosphere as P
    with contextlib.redirect_stdout(io.StringIO()):
        tel = og.Telescope(resolution=RES, diameter=D, samplingTime=DT)
        ngs = og.Source(optBand='V0', magnitude=8)
        ngs * tel
    n_layers = len(ws)
    atm = og.Atmosphere(telescope=tel, r0=0.15, L0=25.0, fractionalR0=[1.0 / n_layers] * n_layers, windSpeed=ws,
                        windDirection=wd, altitude=[0.0] * n_layers)
    atm.layers = []
    for i in range(n_layers):
        L = P._Layer()
        L.resolution = int(np.ceil((RES / D) * D)) + 4
        L.D = L.resolution * D / RES
        L.pixel_size = L.D / L.resolution
        L.rs = RandomState(seed + i * 1000)
        atm.layers.append(L)
    n = atm.layers[0].resolution + P.N_EXTRA
    n_outer = 4 * n - 4
    atm._B = np.zeros((n_outer, n_outer))
    for L in atm.layers:
        L.rs.normal(size=n_outer)
    atm._reset_plan()
    return atm


@pytest.mark.parametrize('ws, wd', CASES)
def test_host_plan_matches_oracle(ws, wd):
    atm = _planner(ws, wd)
    ora = A.OracleAtmosphere(RES, D, DT, 0.15, 25.0, [1.0 / len(ws)] * len(ws), ws, wd, [0.0] * len(ws))
    index = {id(L): i for i, L in enumerate(ora.layers)}
    moves = []
    add_row = ora._add_row

    def record(L, step):
        moves[-1][index[id(L)]].append((int(step[0]), int(step[1])))
        return add_row(L, step)

    ora._add_row = record
    for t in range(60):
        moves.append([[] for _ in ws])
        ora.update()
        atm._plan_one()
        for i, (Lo, Lp) in enumerate(zip(ora.layers, atm.layers)):
            got = [(dx, dy) for dx, dy, _ in atm._plan_moves[t][i]]
            assert got == moves[t][i], (t, i)
            bx, by = atm._plan_buff[t][i]
            if ws[i] == 0:
                assert (bx, by) == (0.0, 0.0)
            else:
                assert (bx, by) == (Lo.buff[0], Lo.buff[1]), (t, i)
            # the same draws in the same order: equal generator states
            so, sp = Lo.rs.get_state(), Lp.rs.get_state()
            assert so[2] == sp[2] and np.array_equal(so[1], sp[1]), (t, i)
    # every move drew one row of normals
    assert len(atm._normals) == sum(len(m) for step in moves for m in step)
