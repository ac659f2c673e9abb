"""Explicit path on the GPU against the reference's own outputs and the oracle.

Plain FP64 must match the reference's FP64 CPU solver within 1e-6 mV (1e-9 V) on every
explicit golden case; mixed precision within 0.1 mV and 0.05 ms spike time.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9          # 1e-6 mV
TOL_MIXED = 1e-4         # 0.1 mV
TOL_SPIKE = 0.05e-3      # 0.05 ms


def problem_from_golden(pkg, g, V0=None):
    d = pkg.Derived(g["eparam"], g["hh_elem"], g["hparam"], float(g["dT_crit"]))
    return pkg.ProblemArrays.from_spec(g["spec"], d, float(g["dT"]), V0=V0)


def run_traced(s, g, i_end=None):
    """Driver loop of src/neurite.cpp:224-236 through nrt_run, recording like the golden."""
    spec = g["spec"]
    rec = int(g["record_every"])
    last = int(g["numStepsT"]) - 1 if i_end is None else i_end
    rows = []
    i = 1
    while i < last:
        nxt = min(last, (i // rec + 1) * rec + 1)
        s.run(i, nxt, spec.init_time, spec.end_input)
        if (nxt - 1) % rec == 0:
            V = s.snapshot()
            rows.append([nxt - 1] + [V[p] for p in g["probes"]])
        i = nxt
    return s.snapshot(), np.array(rows)


def spike_time(t, v, thr=0.0):
    """First upward crossing of thr (linear interpolation), or nan."""
    idx = np.nonzero((v[:-1] < thr) & (v[1:] >= thr))[0]
    if len(idx) == 0:
        return np.nan
    k = idx[0]
    return t[k] + (thr - v[k]) * (t[k + 1] - t[k]) / (v[k + 1] - v[k])


FINITE_CASES = [n for n in golden_names("e") if n != "axon1000_dt1e-3"]


@pytest.mark.parametrize("name", FINITE_CASES)
def test_explicit_fp64_matches_reference(gpu, pkg, name):
    g = load_golden(name)
    s = pkg.SolverEx(problem_from_golden(pkg, g))
    V, trace = run_traced(s, g)
    assert np.abs(V - g["final_V"]).max() < TOL_FP64
    assert trace.shape == g["trace"].shape
    assert np.abs(trace - g["trace"]).max() < TOL_FP64
    m, h, n = s.gates()
    if len(m):
        assert np.abs(np.stack([m, h, n]) - g["final_gates"]).max() < 1e-9
    s.close()


def test_explicit_dropin_loop_equals_device_loop(gpu, pkg):
    """update()/calculate()/snapshot() per step == nrt_run over the same steps (bit-exact)."""
    g = load_golden("axon1000_dtf08")
    spec = g["spec"]
    dT = float(g["dT"])
    a = pkg.SolverEx(problem_from_golden(pkg, g))
    b = pkg.SolverEx(problem_from_golden(pkg, g))
    steps = 700
    for i in range(1, 1 + steps):
        t = i * dT
        a.update(spec.init_time <= t <= spec.end_input)
        a.calculate()
    b.run(1, 1 + steps, spec.init_time, spec.end_input)
    np.testing.assert_array_equal(a.snapshot(), b.snapshot())
    a.close()
    b.close()


def test_explicit_unstable_step_reproduces_reference_blowup(gpu, pkg):
    """dt = 1e-3 ms sits at the reference's critical step: the reference blows up; so
    must we, and the early trace must agree."""
    g = load_golden("axon1000_dt1e-3")
    s = pkg.SolverEx(problem_from_golden(pkg, g))
    V, trace = run_traced(s, g)
    ref = g["trace"]
    early = ref[:, 0] <= 1000  # first ms, before the instability grows
    assert np.abs(trace[early] - ref[early]).max() < TOL_FP64
    assert not np.all(np.isfinite(V)) or np.abs(V).max() > 1.0


def test_explicit_general_initial_state(gpu, pkg, orc):
    """Initial potentials whose terminals differ from their sources take the exact
    two-launch first step; results still match the oracle."""
    g = load_golden("ytree_d3_strain")
    spec = g["spec"]
    rng = np.random.default_rng(1)
    V0 = spec.rest_pot + rng.normal(0, 2e-3, spec.n)
    s = pkg.SolverEx(problem_from_golden(pkg, g, V0=V0))
    s.run(1, 400, spec.init_time, spec.end_input)
    Vg = s.snapshot()
    d = orc.derive(spec)
    Vo, _ = orc.explicit_run(spec, d, float(g["dT"]), 1, 400, V=V0.copy())
    assert np.abs(Vg - Vo).max() < TOL_FP64


def test_explicit_mixed_precision_accuracy(gpu, pkg):
    g = load_golden("axon1000_dtf08")
    s = pkg.SolverEx(problem_from_golden(pkg, g), precision="mixed")
    V, trace = run_traced(s, g)
    assert np.abs(V - g["final_V"]).max() < TOL_MIXED
    assert np.abs(trace[:, 1:] - g["trace"][:, 1:]).max() < TOL_MIXED
    t = g["trace"][:, 0] * float(g["dT"])
    for p in range(1, trace.shape[1]):
        ts_ref = spike_time(t, g["trace"][:, p])
        ts = spike_time(t, trace[:, p])
        if np.isfinite(ts_ref):
            assert abs(ts - ts_ref) < TOL_SPIKE


def test_batch_alone_equals_in_mix(gpu, pkg):
    """Trees of different sizes packed in one batch, each over its own loop range and
    stimulus window, reproduce the reference outputs exactly as when run alone."""
    names = ["ytree_d3_strain", "myelin8", "example8_passive", "axon1000_dtf08"]
    gs = [load_golden(n) for n in names]
    b = pkg.Batch([problem_from_golden(pkg, g) for g in gs])
    runs = [(1, int(g["numStepsT"]) - 1, g["spec"].init_time, g["spec"].end_input) for g in gs]
    b.set_runs(runs)
    b.advance(max(r[1] - r[0] for r in runs))
    assert (b.remaining() == 0).all()
    for k, g in enumerate(gs):
        assert np.abs(b.snapshot(k) - g["final_V"]).max() < TOL_FP64, names[k]
    b.close()


def test_large_tree_against_oracle(gpu, pkg, orc, model):
    """A 2047-branch tree (~2.6e5 elements), a few hundred steps, vs the oracle."""
    spec = model.random_binary_tree(depth=10, seed=2)
    d = orc.derive(spec)
    dT = d.dT_crit * 0.8
    steps = 300
    Vo, _ = orc.explicit_run(spec, d.copy(), dT, 1, 1 + steps)
    dp = pkg.derive(spec)
    s = pkg.SolverEx(pkg.ProblemArrays.from_spec(spec, dp, dT))
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    assert np.abs(s.snapshot() - Vo).max() < TOL_FP64


@pytest.mark.parametrize("count,hh", [(7, True), (3, False)])
def test_tiled_mixed_step_equals_untiled(gpu, pkg, model, count, hh):
    """The TMA-tiled mixed step (bulk-copied element arrays, persistent CTAs) gives bit for
    bit what the one-thread-per-element step gives: uneven trees whose total is no multiple
    of the tile or of 16 bytes, runs that end at different steps, a stimulus window, and
    mostly-passive trees (W dX, K dX staged instead of the gates)."""
    specs = [model.random_tree(seed=70 + q, n_target=700 + 1371 * q, tspan=1e-3)
             for q in range(count)]
    if not hh:
        specs = [model.myelinated_axon(n_nodes=12 + 5 * q, internode_len=120e-6, dx=2e-6,
                                       node_len=2e-6, tspan=1e-3, dtf=0.8) for q in range(count)]
    probs = []
    for sp in specs:
        d = pkg.derive(sp)
        probs.append(pkg.ProblemArrays.from_spec(sp, d, 0.8 * d.dT_crit))
    runs = [(1, 1 + 150 + 37 * q, sp.init_time, sp.end_input) for q, sp in enumerate(specs)]
    out = []
    for tiled in (True, False):
        b = pkg.Batch(probs, mode=0, precision="mixed", tiled=tiled)
        b.set_runs(runs)
        b.advance(300)
        out.append([b.get_state(q) for q in range(count)])
        b.close()
    for a, c in zip(*out):
        np.testing.assert_array_equal(a.V, c.V)
        np.testing.assert_array_equal(a.m, c.m)
        np.testing.assert_array_equal(a.n, c.n)
