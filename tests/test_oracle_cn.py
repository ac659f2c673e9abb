"""The oracle's Crank-Nicolson restatement (not in the reference, which is backward Euler
only): on a passive tree (a linear system) it converges at second order in the time step,
backward Euler at first order, both towards the same solution."""
import numpy as np
import pytest

from conftest import load_golden


@pytest.mark.parametrize("name", ["example8_passive"])
def test_crank_nicolson_is_second_order(orc, name):
    g = load_golden(name)
    spec = g["spec"]
    d = orc.derive(spec)
    T = 0.4e-3                      # inside the stimulus window
    spec.init_time, spec.end_input = 0.0, 1.0

    def run(dt, scheme):
        steps = int(round(T / dt))
        V, _, _, _ = orc.implicit_run(spec, d, dt, 1, 1 + steps, linsolve=0, scheme=scheme)
        return V

    ref = run(T / 1024, 1)
    err = {s: [float(np.abs(run(T / k, s) - ref).max()) for k in (32, 64, 128)] for s in (0, 1)}
    be, cn = err[0], err[1]
    assert 1.7 < be[0] / be[1] < 2.3 and 1.7 < be[1] / be[2] < 2.3
    assert 3.4 < cn[0] / cn[1] < 4.6 and 3.4 < cn[1] / cn[2] < 4.6
    assert cn[2] < be[2] / 10
