"""Initial conditions on the GPU (nbg_batch_init_nbody) against the oracle's
restatement of init_nbody (src/ics/init_nbody.jl:13-229, kepler_init.jl:66-210).

Tolerances: x, v 1e-13 relative to the array maximum; jac_init 1e-11 of each
column's maximum (column-normwise).  The two differ by rounding only: CUDA's
sin, cos, atan2, cbrt against the host libm.  Entry-wise relative bounds do
not hold: derivatives with respect to e cos w and e sin w of nearly circular
orbits carry the reference's 1/e terms (observed 1.7e-13 of the column
maximum on an entry 35 times smaller than it)."""
import numpy as np
import pytest

import nbg
import oracle_lib as O
from conftest import has_gpu
from nbg import workloads as W

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]


def _rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1e-300, float(np.max(np.abs(b))))


def _jac_close(j, jo, rtol=1e-11):
    colmax = np.max(np.abs(jo), axis=0, keepdims=True)
    return bool(np.all(np.abs(j - jo) <= rtol * colmax))


def test_batch_ics_match_oracle_every_body_count():
    els, _, _ = W.batch_uneven(120, seed=9)
    els += W.batch_8body(4, seed=3)[0] + [W.plain_3body(s)[0] for s in range(4)]
    ics = [nbg.ElementsIC(0.37 * q, el.shape[0], el) for q, el in enumerate(els)]
    out = nbg.init_nbody_batch(ics)
    assert {ic.nbody for ic in ics} == set(range(2, 11))
    for ic, (x, v, j) in zip(ics, out):
        xo, vo, jo = O.init_nbody(ic.elements, ic.t0)
        assert _rel(x, xo) < 1e-13 and _rel(v, vo) < 1e-13, ic.nbody
        assert _jac_close(j, jo), ic.nbody


def test_ics_explicit_hierarchy():
    """A double binary: bodies (1,2) and (3,4) each bound, the pairs orbiting each other."""
    H = np.array([[-1, 1, 0, 0], [0, 0, -1, 1], [-1, -1, 1, 1], [-1, -1, -1, -1.0]])
    el = np.array([[1.0, 0, 0, 0, 0, 0, 0],
                   [0.8, 12.0, 3.0, 0.02, 0.01, np.pi / 2, 0.0],
                   [0.5, 400.0, 50.0, 0.05, -0.03, np.pi / 2 + 0.01, 0.0],
                   [0.3, 20.0, 4.0, -0.01, 0.02, np.pi / 2 - 0.01, 0.0]])
    ic = nbg.ElementsIC(1.5, H, el)
    (x, v, j), = nbg.init_nbody_batch([ic])
    xo, vo, jo = O.init_nbody(el, 1.5, H=H)
    assert _rel(x, xo) < 1e-13 and _rel(v, vo) < 1e-13
    assert _jac_close(j, jo)


def test_device_ics_feed_the_integration_bitwise():
    """A State whose x, v, jac_init come from the GPU initial conditions integrates exactly as one
    built from the same arrays on the host."""
    el, h, _ = W.plain_3body(5)
    ic = nbg.ElementsIC(0.0, 3, el)
    (x, v, j), = nbg.init_nbody_batch([ic])
    s1 = nbg.State(ic)
    s1.x[...] = x
    s1.v[...] = v
    s1.jac_init[...] = j
    s2 = s1.copy()
    tt1, tt2 = nbg.TransitTiming(80.0, ic), nbg.TransitTiming(80.0, ic)
    nbg.Integrator(nbg.ahl21, h, 0.0, 80.0)(s1, tt1)
    nbg.Integrator(nbg.ahl21, h, 0.0, 80.0)(s2, tt2)
    assert np.array_equal(tt1.dtdelements, tt2.dtdelements) and tt1.count.sum() > 0
