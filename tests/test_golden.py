"""Golden fixtures (tests/golden/*.npz, written by make_golden.py from the
oracle): the oracle built on this machine reproduces them, and the CUDA path
matches them, both within the parity tolerances."""
import glob
import os

import numpy as np
import pytest

import nbg
import oracle_lib as O
import parity as P
from conftest import has_gpu

FIXTURES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _load(path):
    return dict(np.load(path))


class _S:
    pass


def _check(g, tt, dtdq0, dtdel, count, x, v, jac, dqdt, t):
    P.check_counts(count, g["count"])
    P.check_tt(tt, g["tt"], g["count"], float(g["tmax"]))
    P.check_transit_derivs(dtdq0, g["dtdq0"], g["count"])
    P.check_transit_derivs(dtdel, g["dtdelements"], g["count"], "dtdelements", g["dtdq0"], g["jac_init"])
    gs, rs = _S(), _S()
    gs.x, gs.v, gs.jac_step, gs.dqdt = x, v, jac, dqdt
    rs.x, rs.v, rs.jac_step, rs.dqdt = g["x"], g["v"], g["jac_step"], g["dqdt"]
    P.check_state(gs, rs)
    assert float(t) == float(np.ravel(g["t"])[0])


def test_fixtures_present():
    assert len(FIXTURES) >= 4


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_reproduces_fixture(path):
    g = _load(path)
    s = O.OState(g["x0"], g["v0"], g["m"], jac_init=g["jac_init"], t=float(g["t0"]), pair=g["pair"])
    tt = O.OTiming(s.n, int(g["ntt"]), int(g["ti"]) - 1)
    O.integrate_transits(s, tt, float(g["h"]), float(g["tmax"]), grad=True)
    _check(g, tt.tt, tt.dtdq0, tt.dtdelements, tt.count, s.x, s.v, s.jac_step, s.dqdt, s.t[0])


@pytest.mark.gpu
@pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_gpu_matches_fixture(path):
    g = _load(path)
    n = g["x0"].shape[1]
    M = 7 * n
    ntt = int(g["ntt"])
    b = nbg.Batch([n], int(g["ti"]) - 1, float(g["h"]), float(g["tmax"]), ntt, True)
    b.view("t", 0)[:] = float(g["t0"])
    b.view("x", 0)[:] = g["x0"].ravel(order="F")
    b.view("v", 0)[:] = g["v0"].ravel(order="F")
    b.view("m", 0)[:] = g["m"]
    b.view("jac_step", 0)[:] = np.eye(M).ravel(order="F")
    b.view("jac_init", 0)[:] = g["jac_init"].ravel(order="F")
    b.view("pair", 0)[:] = g["pair"].ravel(order="F")
    b.run()
    _check(g, b.view("tt", 0).reshape((n, ntt), order="F"), b.view("dtdq0", 0).reshape((n, ntt, 7, n), order="F"),
           b.view("dtdelements", 0).reshape((n, ntt, 7, n), order="F"), b.view("count", 0),
           b.view("x", 0).reshape((3, n), order="F"), b.view("v", 0).reshape((3, n), order="F"),
           b.view("jac_step", 0).reshape((M, M), order="F"), b.view("dqdt", 0), b.view("t", 0)[0])
