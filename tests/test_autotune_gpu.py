"""Launch shapes on the device: every shape the autotuner searches gives bit for bit the
same trees, and a tuned batch runs with the shape it chose."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

at = importlib.import_module("168861_gb300.autotune")


def problems(pkg, model, hh=True, count=5):
    specs = [model.random_tree(seed=90 + q, n_target=900 + 1733 * q, tspan=1e-3)
             for q in range(count)]
    if not hh:
        specs = [model.myelinated_axon(n_nodes=10 + 4 * q, internode_len=100e-6, dx=2e-6,
                                       node_len=2e-6, tspan=1e-3, dtf=0.8) for q in range(count)]
    out = []
    for sp in specs:
        d = pkg.derive(sp)
        out.append(pkg.ProblemArrays.from_spec(sp, d, 0.8 * d.dT_crit))
    runs = [(1, 1 + 120 + 29 * q, sp.init_time, sp.end_input) for q, sp in enumerate(specs)]
    return out, runs


def states(pkg, probs, runs, precision, overrides, steps=260):
    b = pkg.Batch(probs, mode=0, precision=precision, **overrides)
    b.set_runs(runs)
    b.advance(steps)
    s = [b.get_state(q) for q in range(len(probs))]
    b.close()
    return s


@pytest.mark.parametrize("precision,hh", [("mixed", True), ("mixed", False), ("fp64", True)])
def test_every_shape_gives_the_same_trees(gpu, pkg, model, precision, hh):
    probs, runs = problems(pkg, model, hh)
    ref = states(pkg, probs, runs, precision, {})
    for ov in at.candidates(0, precision):
        got = states(pkg, probs, runs, precision, ov)
        for a, c in zip(ref, got):
            np.testing.assert_array_equal(a.V, c.V, err_msg=str(ov))
            np.testing.assert_array_equal(a.m, c.m, err_msg=str(ov))
            np.testing.assert_array_equal(a.h, c.h, err_msg=str(ov))


def test_tuned_batch(gpu, pkg, model, tmp_path):
    probs, runs = problems(pkg, model, True, count=4)
    cache = str(tmp_path / "tune.json")
    b = pkg.Batch(probs, mode=0, precision="mixed",
                  autotune={"cache": cache, "steps": 16, "warmup": 3})
    t = b.tuning
    assert t["options"] in t["candidates"] and len(t["times"]) == len(t["candidates"])
    assert all(x is None or x > 0 for x in t["times"])
    for k, v in t["options"].items():
        assert getattr(b.options, k) == int(v)
    b.set_runs(runs)
    b.advance(260)
    got = [b.get_state(q) for q in range(len(probs))]
    b.close()
    for a, c in zip(states(pkg, probs, runs, "mixed", {}), got):
        np.testing.assert_array_equal(a.V, c.V)
    # the second batch of this workload takes the cached shape without timing
    b2 = pkg.Batch(probs, mode=0, precision="mixed", autotune={"cache": cache})
    assert b2.tuning["times"] is None and b2.tuning["options"] == t["options"]
    b2.close()


def implicit_states(pkg, probs, runs, overrides, steps=12):
    b = pkg.Batch(probs, mode=1, precision="mixed", restart=20, tol=1e-10, tol_mode="rel",
                  precond="tree", **overrides)
    b.set_runs(runs)
    b.advance(steps)
    s = [b.get_state(q) for q in range(len(probs))]
    b.close()
    return s


def implicit_problems(pkg, model, count=6):
    specs = [model.random_tree(seed=70 + q, n_target=1200 + 2917 * q, tspan=2e-3)
             for q in range(count)]
    probs = [pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs]
    runs = [(1, 1 + 20, sp.init_time, sp.end_input) for sp in specs]
    return probs, runs


def test_implicit_every_shape_gives_the_same_trees(gpu, pkg, model):
    """The implicit batch kernel's CTA counts: each instance stays one CTA's from start to
    end, so every count gives bit for bit the same trees."""
    probs, runs = implicit_problems(pkg, model)
    ref = implicit_states(pkg, probs, runs, {})
    for ov in at.candidates(1, "mixed"):
        got = implicit_states(pkg, probs, runs, ov)
        for a, c in zip(ref, got):
            np.testing.assert_array_equal(a.V, c.V, err_msg=str(ov))
            np.testing.assert_array_equal(a.V_other, c.V_other, err_msg=str(ov))
            np.testing.assert_array_equal(a.n, c.n, err_msg=str(ov))


def test_tuned_implicit_batch(gpu, pkg, model, tmp_path):
    probs, runs = implicit_problems(pkg, model, count=4)
    cache = str(tmp_path / "tune.json")
    b = pkg.Batch(probs, mode=1, precision="mixed", restart=20, tol=1e-10, tol_mode="rel",
                  precond="tree", autotune={"cache": cache, "steps": 4, "warmup": 2})
    t = b.tuning
    assert t["options"] in t["candidates"] and len(t["times"]) == 3
    assert getattr(b.options, "tile_ctas_per_sm") == t["options"]["tile_ctas_per_sm"]
    b.set_runs(runs)
    b.advance(12)
    got = [b.get_state(q) for q in range(len(probs))]
    b.close()
    for a, c in zip(implicit_states(pkg, probs, runs, {}), got):
        np.testing.assert_array_equal(a.V, c.V)
