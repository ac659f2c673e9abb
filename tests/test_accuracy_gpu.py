"""Mixed precision against the FP64 oracle, per configuration: max |dV| over recorded
compartments and spike-time error (spike = first upward crossing of 0 mV at a recorded
compartment, linearly interpolated between samples).  Bars: 0.1 mV and 0.05 ms.

Run with `-s` to see the per-configuration figures (one ACCURACY line each).

Configurations (seeded, sizes as in the workload definitions, horizons cut where the oracle
would take minutes):
  1. the 1 cm / 1000-compartment squid axon, explicit at 0.8 dT_crit, 10 ms;
  2. the depth-10 random binary tree (2.6e5 compartments), implicit Crank-Nicolson as that
     workload specifies, dt 0.01 ms, 6 ms;
  3. a scaled myelinated axon (6 nodes, 200 um internodes, 20% static strain), explicit,
     20000 steps (nanoseconds of simulated time: the internode step is ~5e-11 s);
  4. six trees spanning the batched population's sizes (1e3 to 1e5 compartments, the
     smallest and the largest included; implicit, dt 0.025 ms) in one batch over the full
     50 ms horizon, probes recorded on the device every step.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_V = 1e-4       # 0.1 mV
TOL_SPIKE = 5e-5   # 0.05 ms


def spike_times(t, trace, thresh=0.0):
    """First upward crossing of `thresh` per column (NaN when none)."""
    out = np.full(trace.shape[1], np.nan)
    for c in range(trace.shape[1]):
        v = trace[:, c]
        up = np.nonzero((v[:-1] < thresh) & (v[1:] >= thresh))[0]
        if len(up):
            k = up[0]
            out[c] = t[k] + (thresh - v[k]) * (t[k + 1] - t[k]) / (v[k + 1] - v[k])
    return out


def report(name, dv, ts_a, ts_b):
    both = ~np.isnan(ts_a) & ~np.isnan(ts_b)
    assert (np.isnan(ts_a) == np.isnan(ts_b)).all(), f"{name}: spikes differ in presence"
    dts = float(np.abs(ts_a[both] - ts_b[both]).max()) if both.any() else None
    print("ACCURACY " + json.dumps({"config": name, "max_dV_mV": dv * 1e3,
                                    "spike_dt_ms": None if dts is None else dts * 1e3,
                                    "spikes_compared": int(both.sum())}))
    assert dv < TOL_V
    if dts is not None:
        assert dts < TOL_SPIKE


def record_gpu(solver, i_end, rec, probes):
    """Runs steps 1 .. i_end-1 in chunks of `rec`, sampling the probes after each chunk."""
    rows, cur = [], 1
    for target in range(rec, i_end, rec):
        solver.run(cur, target + 1, solver.init_time, solver.end_input)
        cur = target + 1
        rows.append(solver.snapshot()[probes])
    if cur < i_end:
        solver.run(cur, i_end, solver.init_time, solver.end_input)
    return np.array(rows)


def explicit_case(pkg, orc, spec, steps, rec, probes, name):
    d = pkg.derive(spec)
    dT = pkg.step_size(spec, d)
    s = pkg.SolverEx(pkg.ProblemArrays.from_spec(spec, d, dT), precision="mixed")
    s.init_time, s.end_input = spec.init_time, spec.end_input
    g = record_gpu(s, 1 + steps, rec, probes)
    Vg = s.snapshot()
    s.close()
    do = orc.derive(spec)
    Vo, tr = orc.explicit_run(spec, do, dT, 1, 1 + steps, record_every=rec, probes=probes)
    tr = tr[: len(g)]
    t = tr[:, 0] * dT
    dv = max(float(np.abs(g - tr[:, 1:]).max()), float(np.abs(Vg - Vo).max()))
    report(name, dv, spike_times(t, g), spike_times(t, tr[:, 1:]))


def test_config1_axon_explicit_mixed(gpu, pkg, orc, model):
    spec = model.straight_axon(dtf=0.8)
    steps = spec.num_steps(pkg.step_size(spec, pkg.derive(spec))) - 2
    explicit_case(pkg, orc, spec, steps, 10, np.array([1, 250, 500, 750, 1000]),
                  "1 axon explicit mixed, 10 ms")


def test_config3_myelinated_explicit_mixed(gpu, pkg, orc, model):
    spec = model.myelinated_axon(n_nodes=6, internode_len=2e-4, strain=0.2, dtf=0.8)
    explicit_case(pkg, orc, spec, 20000, 100, np.array([1, spec.n // 2, spec.n - 2]),
                  "3 myelinated axon explicit mixed, 20000 steps")


def implicit_oracle(orc, spec, steps, rec, probes, scheme=0):
    Vo, _, tr, _ = orc.implicit_run(spec, orc.derive(spec), spec.dt_abs, 1, 1 + steps,
                                    linsolve=0, record_every=rec, probes=probes, scheme=scheme)
    return Vo, tr


def test_config2_binary_tree_implicit_mixed(gpu, pkg, orc, model):
    spec = model.random_binary_tree(depth=10, seed=2, tspan=6e-3)
    steps, probes = 600, np.array([1, 500, spec.n // 2, spec.n - 2])
    s = pkg.SolverIm(pkg.ProblemArrays.from_spec(spec, pkg.derive(spec)), precision="mixed",
                     restart=20, tol=1e-10, tol_mode="rel", precond="tree", scheme="cn")
    s.init_time, s.end_input = spec.init_time, spec.end_input
    g = record_gpu(s, 1 + steps, 1, probes)
    Vg = s.snapshot()
    s.close()
    Vo, tr = implicit_oracle(orc, spec, steps, 1, probes, scheme=1)
    tr = tr[: len(g)]
    t = tr[:, 0] * spec.dt_abs
    dv = max(float(np.abs(g - tr[:, 1:]).max()), float(np.abs(Vg - Vo).max()))
    report("2 binary tree implicit Crank-Nicolson mixed, 6 ms", dv, spike_times(t, g),
           spike_times(t, tr[:, 1:]))


def test_config4_batched_trees_implicit_mixed(gpu, pkg, orc, model):
    sizes = [1000, 100000] + [int(x) for x in model.log_uniform_sizes(4, 1e3, 1e5, 7)]
    specs = [model.random_tree(seed=900 + k, n_target=n) for k, n in enumerate(sizes)]
    steps = specs[0].num_steps(specs[0].dt_abs) - 2  # 50 ms at 0.025 ms
    assert all(sp.dt_abs == specs[0].dt_abs and sp.tspan == 50e-3 for sp in specs)
    probes = [np.array([1, sp.n // 3, sp.n - 2]) for sp in specs]
    b = pkg.Batch([pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs], mode=1,
                  precision="mixed", restart=20, tol=1e-10, tol_mode="rel", precond="tree")
    b.set_runs([(1, 1 + steps, sp.init_time, sp.end_input) for sp in specs])
    b.record([(k, e) for k, pr in enumerate(probes) for e in pr], interval=0, capacity=steps + 1)
    b.advance(steps)
    rec = b.recording()
    finals = [b.snapshot(k) for k in range(len(specs))]
    b.close()
    dv, ta, tb, q = 0.0, [], [], 0
    for k, sp in enumerate(specs):
        g = np.stack([rec.values[q + j] for j in range(len(probes[k]))], axis=1)
        q += len(probes[k])
        Vo, tr = implicit_oracle(orc, sp, steps, 1, probes[k])
        tr = tr[: len(g)]
        assert len(g) == steps and len(tr) == steps
        t = tr[:, 0] * sp.dt_abs
        dv = max(dv, float(np.abs(g - tr[:, 1:]).max()), float(np.abs(finals[k] - Vo).max()))
        ta.append(spike_times(t, g))
        tb.append(spike_times(t, tr[:, 1:]))
    report(f"4 six batched trees of {min(sizes)}-{max(s.n for s in specs)} compartments "
           "implicit mixed, 50 ms", dv, np.concatenate(ta), np.concatenate(tb))
