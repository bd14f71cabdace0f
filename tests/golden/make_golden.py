"""Generates the golden fixtures of tests/golden/ with the CPU oracle.

Each fixture holds the seeded inputs of one case (initial state, masses,
jac_init, pair flags, h, tmax, t0, ti) and the oracle's outputs of
intr(s, tt; grad = true): tt, dtdq0, dtdelements, count and the final x, v,
jac_step, dqdt.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import conftest  # noqa: E402  (loads the package as `nbg`)
import oracle_lib as O  # noqa: E402

nbg = conftest.load_package()
W = nbg.workloads


def cases():
    el, h, _ = W.plain_3body(0)
    yield "plain_3body_t100", el, h, 100.0, 0.0, 1, None
    els, hs, _ = W.batch_uneven(40, seed=7, nmin=5, nmax=5)
    yield "uneven_5body_t30", els[0], hs[0], 30.0, 0.0, 1, None
    els, hs, _ = W.batch_uneven(40, seed=8, nmin=4, nmax=4)
    pair = np.ones((4, 4), dtype=np.uint8)
    pair[0, :] = 0
    pair[:, 0] = 0
    yield "kick_4body_t20", els[0], hs[0], 20.0, 0.0, 1, pair
    els, h, _ = W.batch_8body(1, seed=3)
    yield "trappist_8body_t12", els[0], h, 12.0, 0.0, 1, None


def make(name, el, h, tmax, t0, ti, pair):
    ic = nbg.ElementsIC(t0, el.shape[0], el)
    x, v, jinit = ic.init_nbody()
    n = ic.nbody
    ntt = nbg.TransitTiming(tmax, ic, ti).ntt
    s = O.OState(x, v, ic.m, jac_init=jinit, t=t0, pair=pair)
    tt = O.OTiming(n, ntt, ti - 1)
    O.integrate_transits(s, tt, h, tmax, grad=True)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), x0=x, v0=v, m=ic.m, jac_init=jinit,
                        pair=s.pair, h=h, tmax=tmax, t0=t0, ti=ti, ntt=ntt, tt=tt.tt, dtdq0=tt.dtdq0,
                        dtdelements=tt.dtdelements, count=tt.count, x=s.x, v=s.v, jac_step=s.jac_step,
                        dqdt=s.dqdt, t=s.t)


if __name__ == "__main__":
    for c in cases():
        make(*c)
        print("wrote", c[0])
