"""Pin of the oracle's forward map by its order of accuracy and its energy error.

The reference's tests check derivatives against finite differences of its own
map, so a wrong coefficient in the map itself would pass them.  This test
restates the reference's energy study (examples/energy_conservation.jl:
96-183: compute_energy, the energy error against the step size) as a
convergence test of the oracle's no-gradient ahl21! (ahl21_no_grad.jl:6-18,
the same x, v arithmetic as the gradient step, which the grad = no-grad
identity pins bit for bit), run in quad precision so that rounding stays far
below the truncation error:

  * the end state after a fixed span, against a run with a step 8 times
    smaller than the smallest tested, converges as h^4 over more than a decade
    of h (AHL21 is a fourth-order method);
  * the largest relative energy error over the span falls as h^4;
  * Richardson's estimate (q(h) - q(h/2)) / 15 predicts the error of q(h/2);
  * the same holds with a planet pair integrated by kicks and the phic!
    corrector (pair = true);
  * the test rejects the map with a planted wrong coefficient: phisalpha!'s
    alpha = 1 instead of 2 (ahl21.jl:60, ahl21_no_grad.jl:14), or outer kicks
    of h/5 instead of h/6 (ahl21_no_grad.jl:8,17), both fall to second order
    or worse.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle_lib as O
from nbg import workloads as W

T_SPAN = {"trappist3": 15.0, "plain3": 120.0}
H0 = {"trappist3": 0.0375, "plain3": 0.4}
HALVINGS = 4   # h0 .. h0/16: 1.2 decades
REF_DIV = 128  # the reference run's step: h0/128


def _setups(ref_elements=None):
    out = {}
    if ref_elements is not None:
        x, v, _ = O.init_nbody(ref_elements[:3], 7257.93115525)
        out["trappist3"] = (x, v, ref_elements[:3, 0].copy())
    el, _, _ = W.plain_3body(4)
    x, v, _ = O.init_nbody(el, 0.0)
    out["plain3"] = (x, v, el[:, 0].copy())
    return out


def _study(x, v, m, span, h0, **kw):
    hs = [h0 / 2 ** k for k in range(HALVINGS + 1)] + [h0 / REF_DIV]
    with ThreadPoolExecutor(max_workers=len(hs)) as ex:
        runs = list(ex.map(lambda h: O.order_run_quad(x, v, m, h, int(round(span / h)), **kw), hs))
    ref = runs[-1]

    def diff(a, b):  # (hi, lo) pairs: hi - hi is exact for close values
        return (a[0] - b[0]) + (a[1] - b[1])

    def err(r):
        return (np.max(np.abs(diff(r[0], ref[0]))) / np.max(np.abs(ref[0][0])) +
                np.max(np.abs(diff(r[1], ref[1]))) / np.max(np.abs(ref[1][0])))

    errs = np.array([err(r) for r in runs[:-1]])
    de = np.array([r[2] for r in runs[:-1]])
    # Richardson: the error of q(h/2) estimated from q(h) and q(h/2), against the reference run
    rich = []
    for k in range(1, HALVINGS + 1):
        est = diff(runs[k - 1][0], runs[k][0]) / 15.0
        act = diff(runs[k][0], ref[0])
        rich.append(float(np.max(np.abs(est - act)) / np.max(np.abs(act))))
    return errs, de, np.array(rich)


def _slopes(a):
    return np.log2(a[:-1] / a[1:])


@pytest.fixture(scope="module")
def setups(request):
    try:
        ref = request.getfixturevalue("ref_elements")
    except pytest.skip.Exception:
        ref = None
    return _setups(ref)


@pytest.mark.parametrize("kick_pair", [False, True])
def test_fourth_order_and_energy(setups, kick_pair):
    for name, (x, v, m) in setups.items():
        pair = None
        if kick_pair:
            pair = np.zeros((3, 3), dtype=np.uint8)
            pair[1, 2] = pair[2, 1] = 1
        errs, de, rich = _study(x, v, m, T_SPAN[name], H0[name], pair=pair)
        s_state, s_energy = _slopes(errs), _slopes(de)
        assert np.all((s_state > 3.8) & (s_state < 4.2)), (name, s_state)
        assert np.all((s_energy > 3.7) & (s_energy < 4.3)), (name, s_energy)
        assert np.all(rich < 0.05), (name, rich)


@pytest.mark.parametrize("planted", [{"alpha": 1.0}, {"kick_den": 5.0}])
def test_a_wrong_coefficient_fails_the_order_test(setups, planted):
    x, v, m = setups["plain3"]
    pair = None
    if "kick_den" in planted:  # the outer kicks act only on pairs integrated by kicks
        pair = np.zeros((3, 3), dtype=np.uint8)
        pair[1, 2] = pair[2, 1] = 1
    errs, de, _ = _study(x, v, m, T_SPAN["plain3"], H0["plain3"], pair=pair, **planted)
    s_state = _slopes(errs)
    assert np.all(s_state < 3.0), s_state  # second order (or worse): the h^4 test above would fail
