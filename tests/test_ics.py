"""The package's host-side initial conditions against the oracle's restatement."""
import numpy as np
import pytest

import nbg
import oracle_lib as O
from nbg import workloads as W


def _rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1e-300, float(np.max(np.abs(b))))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_plain_3body_ics(seed):
    el, _, _ = W.plain_3body(seed)
    x, v, j = nbg.init_nbody(el, 0.0, nbg.hierarchy_nested(3))
    xo, vo, jo = O.init_nbody(el, 0.0)
    assert _rel(x, xo) < 1e-14 and _rel(v, vo) < 1e-14 and _rel(j, jo) < 1e-13


def test_uneven_ics():
    els, _, _ = W.batch_uneven(30, seed=4)
    for el in els:
        x, v, j = nbg.init_nbody(el, 0.0, nbg.hierarchy_nested(el.shape[0]))
        xo, vo, jo = O.init_nbody(el, 0.0)
        assert _rel(x, xo) < 1e-13 and _rel(v, vo) < 1e-13 and _rel(j, jo) < 1e-12


def test_reference_fixture_ics(ref_elements):
    ic = nbg.ElementsIC(7257.93115525, [8, 1, 1, 1, 1, 1, 1, 1], ref_elements)
    x, v, j = ic.init_nbody()
    xo, vo, jo = O.init_nbody(ref_elements, 7257.93115525)
    assert _rel(x, xo) < 1e-14 and _rel(j, jo) < 1e-12


def test_hierarchy_nested_matches_reference_shape():
    H = nbg.hierarchy_nested(4)
    assert np.array_equal(H, np.array([[-1, 1, 0, 0], [-1, -1, 1, 0], [-1, -1, -1, 1], [-1, -1, -1, -1.0]]))


def test_elements_keyword_constructor():
    e = nbg.Elements(m=3e-6, P=10.0, t0=2.0, ecosw=0.01, I=np.pi / 2)
    assert e.row() == [3e-6, 10.0, 2.0, 0.01, 0.0, np.pi / 2, 0.0]
    star = nbg.Elements(m=1.0)
    ic = nbg.ElementsIC(0.0, 2, star, e)
    assert ic.elements.shape == (2, 7)
    with pytest.raises(ValueError):
        nbg.Elements(m=1.0, P=-1.0)
    with pytest.raises(ValueError):
        nbg.Elements(m=1.0, P=1.0, e=1.5)


def test_transit_timing_ntt():
    el, _, _ = W.plain_3body(0)
    ic = W.ic_of(el)
    tt = nbg.TransitTiming(1000.0, ic)
    assert tt.ntt == int(np.ceil(1000.0 / 10.0)) + 3
    assert tt.dtdq0.shape == (3, tt.ntt, 7, 3)
    assert tt.occs == [2, 3]
