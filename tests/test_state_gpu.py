"""State export / import (nrt_get_state / nrt_set_state and the batch forms): a run
checkpointed half-way and resumed in a fresh handle ends where the uninterrupted run ends,
bit for bit, in every mode and precision."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def problem(pkg, g):
    d = pkg.Derived(g["eparam"], g["hh_elem"], g["hparam"], float(g["dT_crit"]))
    return pkg.ProblemArrays.from_spec(g["spec"], d, float(g["dT"]))


CASES = [("axon1000_dtf08", pkg_opts) for pkg_opts in (dict(), dict(precision="mixed"))] + \
        [("im_ytree_d3", dict(tol=1e-11, tol_mode="rel")),
         ("im_ytree_d3", dict(precision="mixed", restart=20, tol=1e-10, tol_mode="rel"))]


@pytest.mark.parametrize("name,opts", CASES)
def test_checkpoint_resume_is_exact(gpu, pkg, name, opts):
    g = load_golden(name)
    spec = g["spec"]
    Cls = pkg.SolverIm if g["mode"] == "i" else pkg.SolverEx
    half = 37 if g["mode"] == "i" else 3001
    whole = Cls(problem(pkg, g), **opts)
    whole.run(1, 1 + 2 * half, spec.init_time, spec.end_input)
    want = whole.get_state()
    whole.close()
    a = Cls(problem(pkg, g), **opts)
    a.run(1, 1 + half, spec.init_time, spec.end_input)
    st = a.get_state()
    a.close()
    b = Cls(problem(pkg, g), **opts)
    b.set_state(st)
    np.testing.assert_array_equal(b.get_state().V, st.V)
    b.run(1 + half, 1 + 2 * half, spec.init_time, spec.end_input)
    got = b.get_state()
    b.close()
    np.testing.assert_array_equal(got.V, want.V)
    np.testing.assert_array_equal(got.m, want.m)
    np.testing.assert_array_equal(got.h, want.h)
    np.testing.assert_array_equal(got.n, want.n)


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_instance_moves_between_batches(gpu, pkg, model, mode):
    """Preemption: one tree leaves a batch half-way (its state exported), joins another
    batch, and finishes where it would have finished in the first."""
    specs = [model.random_tree(seed=s, n_target=n, dt=2.5e-5, tspan=2e-3)
             for s, n in [(51, 2000), (52, 5000), (53, 1200)]]
    probs = []
    for sp in specs:
        d = pkg.derive(sp)
        probs.append(pkg.ProblemArrays.from_spec(sp, d, sp.dt_abs if mode else 0.8 * d.dT_crit))
    opts = dict(precision="mixed")
    if mode:
        opts.update(restart=20, tol=1e-10, tol_mode="rel")
    steps = 40 if mode else 400
    full = pkg.Batch(probs, mode=mode, **opts)
    full.set_runs([(1, 1 + steps, sp.init_time, sp.end_input) for sp in specs])
    full.advance(steps)
    want = full.get_state(1)
    full.close()
    first = pkg.Batch(probs, mode=mode, **opts)
    first.set_runs([(1, 1 + steps, sp.init_time, sp.end_input) for sp in specs])
    first.advance(steps // 2)
    st = first.get_state(1)
    first.close()
    # the tree continues in a batch with other company, at the same instance position
    second = pkg.Batch([probs[2], probs[1], probs[0]], mode=mode, **opts)
    second.set_runs([(1, 1 + steps, specs[2].init_time, specs[2].end_input),
                     (1 + steps // 2, 1 + steps, specs[1].init_time, specs[1].end_input),
                     (1, 1 + steps, specs[0].init_time, specs[0].end_input)])
    second.set_state(1, st)
    second.advance(steps)
    got = second.get_state(1)
    second.close()
    # one CTA per instance (implicit) or per element (explicit): the company does not
    # change the tree's arithmetic
    for part in ("V", "m", "h", "n"):
        np.testing.assert_array_equal(getattr(got, part), getattr(want, part))


def test_set_state_general_first_step(gpu, pkg, orc):
    """A V whose terminals do not copy their sources: the next explicit step takes the
    reference's general form, as the oracle does from the same state."""
    g = load_golden("axon1000_dtf08")
    spec = g["spec"]
    s = pkg.SolverEx(problem(pkg, g))
    st = s.get_state()
    V = st.V.copy()
    V[0] += 1e-3
    V[-1] -= 2e-3
    st.V = V
    s.set_state(st)
    s.run(1, 200, spec.init_time, spec.end_input)
    d = orc.derive(spec)
    Vo, _ = orc.explicit_run(spec, d, float(g["dT"]), 1, 200, V=V.copy())
    assert np.abs(s.snapshot() - Vo).max() < 1e-9
    s.close()


def test_snapshot_all_equals_per_instance(gpu, pkg, model):
    specs = [model.random_tree(seed=60 + q, n_target=900 + 700 * q, dt=2.5e-5, tspan=1e-3)
             for q in range(4)]
    probs = [pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs]
    b = pkg.Batch(probs, mode=1, precision="mixed", restart=20, tol=1e-10, tol_mode="rel")
    b.set_runs([(1, 1 + 5 + q, sp.init_time, sp.end_input) for q, sp in enumerate(specs)])
    b.advance(8)
    allv = b.snapshot_all()
    for q in range(len(specs)):
        np.testing.assert_array_equal(allv[q], b.snapshot(q))
    b.close()
