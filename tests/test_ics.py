"""The package's host-side initial conditions against the oracle's restatement."""
import os

import numpy as np
import pytest

import nbg
import oracle_lib as O
from conftest import REF_ELEMENTS
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


def test_hierarchy_vectors():
    """hierarchy([N, b1, ...]) (setup_hierarchy.jl:9-179): the documented double binary, fully nested vectors,
    and two traces of the level rules; invalid vectors raise."""
    assert np.array_equal(nbg.hierarchy([4, 2, 1]),
                          np.array([[-1, 1, 0, 0], [0, 0, -1, 1], [-1, -1, 1, 1], [-1, -1, -1, -1.0]]))
    for n in range(2, 11):
        assert np.array_equal(nbg.hierarchy([n] + [1] * (n - 1)), nbg.hierarchy_nested(n))
    # every body on the bottom level: binaries (12)(34)(56)(78), then (12|34), (56|78), then the halves
    H8 = nbg.hierarchy([8, 4, 2, 1])
    assert np.array_equal(H8[:4], np.kron(np.eye(4), [[-1.0, 1.0]]))
    assert np.array_equal(H8[4], [-1, -1, 1, 1, 0, 0, 0, 0]) and np.array_equal(H8[5], [0, 0, 0, 0, -1, -1, 1, 1])
    assert np.array_equal(H8[6], [-1] * 4 + [1] * 4) and np.all(H8[7] == -1)
    # two binaries, their pair, then a fifth body outside
    H5 = nbg.hierarchy([5, 2, 1, 1])
    assert np.array_equal(H5, np.array([[-1, 1, 0, 0, 0], [0, 0, -1, 1, 0], [-1, -1, 1, 1, 0], [-1, -1, -1, -1, 1],
                                        [-1, -1, -1, -1, -1.0]]))
    for bad in ([4, 1, 1], [4, 3, 1], [6, 4, 1], [3]):
        with pytest.raises(ValueError):
            nbg.hierarchy(bad)


def test_double_binary_ics_match_oracle():
    """init_nbody for the hierarchy [4, 2, 1] (two binaries orbiting each other) against the oracle.  Row r of
    the elements holds body r's mass; the orbits go to the Keplerians as kepcalc assigns them (init_nbody.jl:
    60-95): a-b takes row 2, c-d (a new branch) row 4, the outer orbit row 3."""
    el = np.array([[1.0, 0, 0, 0, 0, 0, 0],                                  # body a
                   [0.8, 10.0, 2.0, 0.01, 0.02, np.pi / 2, 0.0],              # body b; orbit a-b
                   [0.5, 400.0, 100.0, 0.05, 0.0, np.pi / 2, 0.0],            # body c; orbit (ab)-(cd)
                   [0.3, 12.0, 5.0, -0.02, 0.01, np.pi / 2, 0.1]])            # body d; orbit c-d
    H = nbg.hierarchy([4, 2, 1])
    ic = nbg.ElementsIC(0.0, [4, 2, 1], el)
    assert np.array_equal(ic.H, H)
    x, v, j = ic.init_nbody()
    xo, vo, jo = O.init_nbody(el, 0.0, H)
    # the binaries are tight and the outer orbit wide: |c - d| is the 12-day separation, not the 400-day one
    assert np.linalg.norm(x[:, 2] - x[:, 3]) < 0.2 * np.linalg.norm(x[:, :2].mean(axis=1) - x[:, 2:].mean(axis=1))
    assert _rel(x, xo) < 1e-13 and _rel(v, vo) < 1e-13 and _rel(j, jo) < 1e-12
    assert float(np.abs((x * ic.m).sum(axis=1)).max()) < 1e-12 * float(np.abs(x).max())  # centre of mass at 0


REF_COORDINATES = os.path.join(os.path.dirname(REF_ELEMENTS), "coordinates.txt")


def test_initial_conditions_every_specification(ref_elements):
    """test/test_initial_conditions.jl: for n = 2..8, ElementsIC from the file, the array and a list of Elements,
    with H as a matrix, a vector and a body count, are all the same; CartesianIC from the file and the array too."""
    t0 = 7257.93115525 - 7300.0
    fields = ("elements", "H", "amat", "nbody", "m", "t0", "der")
    for n in range(2, 9):
        Hv = [n] + [1] * (n - 1)
        Hm = nbg.hierarchy(Hv)
        base = nbg.ElementsIC(t0, Hm, REF_ELEMENTS)
        elems = [nbg.Elements(*row) for row in ref_elements[:n]]
        for H in (Hm, Hv, n):
            for spec in (REF_ELEMENTS, ref_elements, elems):
                ic = nbg.ElementsIC(t0, H, spec)
                for f in fields:
                    assert np.array_equal(np.asarray(getattr(ic, f)), np.asarray(getattr(base, f))), (n, f)
        if os.path.exists(REF_COORDINATES):
            cf = nbg.CartesianIC(t0, n, REF_COORDINATES)
            ca = nbg.CartesianIC(t0, n, np.loadtxt(REF_COORDINATES, delimiter=","))
            for f in ("x", "v", "m"):
                assert np.array_equal(getattr(cf, f), getattr(ca, f))
            assert cf.x.shape == (3, n) and cf.m.shape == (n,)


def test_elements_constructors():
    """InitialConditions.jl:21-107: seven positional fields (e, w derived; no checks), eleven (as given), keywords
    (checked; Greek spellings accepted); a zero period gives IEEE results, as in Julia."""
    e7 = nbg.Elements(3e-6, 10.0, 2.0, 0.03, 0.04, np.pi / 2, 0.1)
    assert e7.row() == [3e-6, 10.0, 2.0, 0.03, 0.04, np.pi / 2, 0.1]
    assert e7.e == np.hypot(0.03, 0.04) and e7.w == np.arctan2(0.04, 0.03) and e7.a == 0.0 and e7.tp == 0.0
    e11 = nbg.Elements(*range(1, 12))
    assert [getattr(e11, f) for f in nbg.Elements.ALL_FIELDS] == [float(q) for q in range(1, 12)]
    star = nbg.Elements(1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)  # the star row of an elements file: no checks
    assert star.row() == [1.0] + [0.0] * 6
    g = nbg.Elements(m=3e-6, P=10.0, t0=2.0, **{"ecosω": 0.01, "Ω": 0.2})
    k = nbg.Elements(m=3e-6, P=10.0, t0=2.0, ecosw=0.01, Omega=0.2)
    assert g.row() == k.row() and g.tp == k.tp
    z = nbg.Elements(m=1.0, P=0.0, t0=1.0)  # Julia: n = 2 pi / 0 = Inf, tp = (pi/2 + w) / n = 0
    assert z.tp == 0.0
    with pytest.raises(TypeError):
        nbg.Elements(1.0, 2.0)
    with pytest.raises(TypeError):
        nbg.Elements(P=1.0)
    with pytest.raises(TypeError):
        nbg.Elements(m=1.0, Q=1.0)
