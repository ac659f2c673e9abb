"""Device-side recording at probes (nrt_record / nrt_batch_record) against the reference's
traces and the oracle.

The samples of a plain FP64 run are the reference's trace (same loop indices, values
within 1e-6 mV); spike times are the oracle's, computed from its every-step trace with the
same interpolation (oracle.recording), within 1e-6 ms.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9        # 1e-6 mV
TOL_MIXED = 1e-4       # 0.1 mV
TOL_SPIKE = 1e-9       # 1e-6 ms (FP64 paths)


def problem(pkg, g):
    d = pkg.Derived(g["eparam"], g["hh_elem"], g["hparam"], float(g["dT_crit"]))
    return pkg.ProblemArrays.from_spec(g["spec"], d, float(g["dT"]))


def tight(**kw):
    o = dict(tol=1e-11, tol_mode="rel", restart=30, precond="tree")
    o.update(kw)
    return o


def oracle_recording(orc, spec, dT, steps, probes, interval, implicit=False, thresh=0.0):
    """Per probe: the oracle's samples and spike times over loop indices 1 .. steps."""
    import oracle
    d = orc.derive(spec)
    pr = np.asarray(probes, np.int32)
    if implicit:
        _, _, tr, _ = orc.implicit_run(spec, d, dT, 1, 1 + steps, linsolve=0, record_every=1,
                                       probes=pr)
    else:
        _, tr = orc.explicit_run(spec, d, dT, 1, 1 + steps, record_every=1, probes=pr)
    assert len(tr) == steps
    out = []
    for c, p in enumerate(pr):
        smp, spk = oracle.recording(1, spec.rest_pot[p], tr[:, 1 + c], 1, interval, thresh, dT)
        out.append((np.array([smp[k] for k in sorted(smp)]), np.array(spk)))
    return out


@pytest.mark.parametrize("name", [n for n in golden_names("e") if n != "axon1000_dt1e-3"])
def test_explicit_recording_is_the_reference_trace(gpu, pkg, name):
    g = load_golden(name)
    spec = g["spec"]
    rec = int(g["record_every"])
    last = int(g["numStepsT"]) - 1
    s = pkg.SolverEx(problem(pkg, g))
    s.record(g["probes"], interval=rec - 1, capacity=len(g["trace"]) + 5)
    s.run(1, last, spec.init_time, spec.end_input)
    r = s.recording()
    tr = g["trace"]
    for c in range(len(g["probes"])):
        assert r.num_samples[c] == len(tr)
        np.testing.assert_array_equal(r.times[c], tr[:, 0] * float(g["dT"]))
        assert np.abs(r.values[c] - tr[:, 1 + c]).max() < TOL_FP64
    # the reference's trace file, written from the device samples
    line = r.trace_text(0).splitlines()[0].split()
    assert line[0] == "%.20f" % (tr[0, 0] * float(g["dT"]))
    s.close()


def test_explicit_spike_times_match_oracle(gpu, pkg, orc, model):
    """The 1 cm squid axon at 0.8 dT_crit: the action potential starts at the stimulated
    end and passes the first probes (the root terminal, element 1, 2.5 mm) within 10 ms."""
    spec = model.straight_axon(dtf=0.8)
    d = pkg.derive(spec)
    dT = pkg.step_size(spec, d)
    steps = spec.num_steps(dT) - 2
    probes = [0, 1, 250, 500, 750, 1000, 1001]   # both terminals included
    s = pkg.SolverEx(pkg.ProblemArrays.from_spec(spec, d, dT))
    s.record(probes, interval=9, capacity=steps // 10 + 1, max_spikes=4)
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    r = s.recording()
    want = oracle_recording(orc, spec, dT, steps, probes, 9)
    n_spikes = 0
    for c, (smp, spk) in enumerate(want):
        assert r.num_samples[c] == len(smp)
        assert np.abs(r.values[c] - smp).max() < TOL_FP64
        assert r.num_spikes[c] == len(spk)
        if len(spk):
            assert np.abs(r.spikes[c] - spk).max() < TOL_SPIKE
        n_spikes += len(spk)
    assert n_spikes >= 3 and r.num_spikes[0] == r.num_spikes[1] == 1
    s.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_explicit_recording_same_with_and_without_graphs(gpu, pkg, graphs):
    g = load_golden("axon1000_dtf08")
    spec = g["spec"]
    s = pkg.SolverEx(problem(pkg, g), use_graphs=graphs)
    s.record([1, 500, 1000], interval=6, capacity=200)
    s.run(1, 1000, spec.init_time, spec.end_input)
    r = s.recording()
    s.close()
    ref = pkg.SolverEx(problem(pkg, g), use_graphs=not graphs)
    ref.record([1, 500, 1000], interval=6, capacity=200)
    ref.run(1, 1000, spec.init_time, spec.end_input)
    q = ref.recording()
    ref.close()
    for c in range(3):
        np.testing.assert_array_equal(r.values[c], q.values[c])
    assert (r.num_samples == 999 // 7).all()


def test_recording_across_runs_and_capacity(gpu, pkg):
    """Chunked runs continue the counter; samples past capacity and spikes past max_spikes
    are counted but not kept."""
    g = load_golden("axon1000_dtf08")
    spec = g["spec"]
    last = int(g["numStepsT"]) - 1
    whole = pkg.SolverEx(problem(pkg, g))
    whole.record([250, 750], interval=49, capacity=1000)
    whole.run(1, last, spec.init_time, spec.end_input)
    a = whole.recording()
    whole.close()
    part = pkg.SolverEx(problem(pkg, g))
    part.record([250, 750], interval=49, capacity=10, max_spikes=0)
    for i0 in range(1, last, 777):
        part.run(i0, min(last, i0 + 777), spec.init_time, spec.end_input)
    b = part.recording()
    part.close()
    np.testing.assert_array_equal(a.num_samples, b.num_samples)
    np.testing.assert_array_equal(a.num_spikes, b.num_spikes)
    for c in range(2):
        assert len(b.values[c]) == 10 and len(b.spikes[c]) == 0
        np.testing.assert_array_equal(a.values[c][:10], b.values[c])


def test_dropin_loop_is_not_recorded(gpu, pkg):
    g = load_golden("axon1000_dtf08")
    s = pkg.SolverEx(problem(pkg, g))
    s.record([1, 2], interval=0, capacity=10)
    for _ in range(5):
        s.update(True)
        s.calculate()
    assert (s.recording().num_samples == 0).all()
    s.close()


@pytest.mark.parametrize("name", golden_names("i"))
def test_implicit_recording_matches_oracle(gpu, pkg, orc, name):
    g = load_golden(name)
    spec = g["spec"]
    steps = int(g["numStepsT"]) - 2
    probes = list(g["probes"]) + [0, spec.n - 1]
    s = pkg.SolverIm(problem(pkg, g), **tight(max_iter=20000))
    s.record(probes, interval=2, capacity=steps)
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    r = s.recording()
    want = oracle_recording(orc, spec, float(g["dT"]), steps, probes, 2, implicit=True)
    for c, (smp, spk) in enumerate(want):
        assert r.num_samples[c] == len(smp)
        assert np.abs(r.values[c] - smp).max() < TOL_FP64
        assert r.num_spikes[c] == len(spk)
        if len(spk):
            assert np.abs(r.spikes[c] - spk).max() < TOL_SPIKE
    s.close()


def test_implicit_cooperative_recording(gpu, pkg, orc, model):
    """One ~3e4-element tree on the whole-GPU launch, recording every step."""
    spec = model.random_tree(seed=25, n_target=30000, dt=2.5e-5, tspan=2e-3)
    steps = 40
    probes = [1, spec.n // 3, spec.n // 2, spec.n - 2]
    s = pkg.SolverIm(pkg.ProblemArrays.from_spec(spec, pkg.derive(spec)), **tight())
    s.record(probes, interval=0, capacity=steps, threshold=-0.064)
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    r = s.recording()
    want = oracle_recording(orc, spec, spec.dt_abs, steps, probes, 0, implicit=True,
                            thresh=-0.064)
    for c, (smp, spk) in enumerate(want):
        assert np.abs(r.values[c] - smp).max() < TOL_FP64
        assert r.num_spikes[c] == len(spk)
        if len(spk):
            assert np.abs(r.spikes[c] - spk).max() < TOL_SPIKE
    s.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_recording_equals_alone(gpu, pkg, model, mode):
    """Probes on several instances of a mixed-precision batch with uneven runs record what
    each tree records alone; an instance stops recording when its run ends."""
    specs = [model.random_tree(seed=s, n_target=n, dt=2.5e-5, tspan=2e-3)
             for s, n in [(31, 1500), (32, 4000), (33, 900)]]
    probs = []
    for sp in specs:
        d = pkg.derive(sp)
        dT = sp.dt_abs if mode == 1 else 0.8 * d.dT_crit
        probs.append(pkg.ProblemArrays.from_spec(sp, d, dT))
    opts = dict(precision="mixed")
    if mode == 1:
        opts.update(restart=20, tol=1e-10, tol_mode="rel")
    steps = [30, 50, 20] if mode == 1 else [300, 500, 200]
    probes = [(0, 1), (1, specs[1].n // 2), (2, specs[2].n - 2), (1, 1), (0, specs[0].n // 2)]
    b = pkg.Batch(probs, mode=mode, **opts)
    b.set_runs([(1, 1 + k, sp.init_time, sp.end_input) for k, sp in zip(steps, specs)])
    b.record(probes, interval=1, capacity=max(steps), threshold=-0.06)
    b.advance(max(steps))
    r = b.recording()
    b.close()
    Cls = pkg.SolverIm if mode == 1 else pkg.SolverEx
    for c, (q, e) in enumerate(probes):
        alone = Cls(probs[q], **opts)
        alone.record([e], interval=1, capacity=max(steps), threshold=-0.06)
        alone.run(1, 1 + steps[q], specs[q].init_time, specs[q].end_input)
        a = alone.recording()
        alone.close()
        assert r.num_samples[c] == a.num_samples[0] == steps[q] // 2
        np.testing.assert_array_equal(r.times[c], a.times[0])
        assert np.abs(r.values[c] - a.values[0]).max() < TOL_MIXED
        assert r.num_spikes[c] == a.num_spikes[0]


def test_record_rejects_bad_probes(gpu, pkg):
    g = load_golden("axon1000_dtf08")
    s = pkg.SolverEx(problem(pkg, g))
    with pytest.raises(pkg.NeuriteError):
        s.record([5000])
    with pytest.raises(pkg.NeuriteError):
        s.record([1], interval=-1)
    with pytest.raises(pkg.NeuriteError):
        s.recording()          # nothing configured
    s.close()
