"""Launch shapes of the explicit time loop that must not change a bit of the results:

- the chunk kernel (nrt_options.step_launch = 1: up to 64 steps per cooperative launch,
  grid barrier between steps) against one launch per step (the default): potentials, gates,
  the probes' samples and spike times and the strained coefficients, over loop ranges that
  end inside a chunk, FP64 and mixed, single trees and batches whose instances finish at
  different steps;
- small FP64 packs' eight lanes per element against one thread per element;

and the library's count of its own kernel launches (nrt_kernel_launches).
"""
import numpy as np
import pytest

from conftest import load_golden
from test_strain_gpu import step_size, strained

pytestmark = pytest.mark.gpu


def golden_axon(pkg):
    g = load_golden("axon1000_dtf08")
    d = pkg.Derived(g["eparam"], g["hh_elem"], g["hparam"], float(g["dT_crit"]))
    return g["spec"], pkg.ProblemArrays.from_spec(g["spec"], d, float(g["dT"])), float(g["dT"])


def built(pkg, spec, dtf=0.8):
    d = pkg.derive(spec)
    dT = dtf * d.dT_crit
    return pkg.ProblemArrays.from_spec(spec, d, dT), dT


def trees(pkg, model):
    """(name, spec, problem, dT): the 1000-compartment golden axon, a myelinated axon (HH
    nodes between passive internodes) and a branched random tree."""
    out = [("axon",) + golden_axon(pkg)]
    for name, spec in (("myelin", model.myelinated_axon(n_nodes=12, internode_len=40e-6,
                                                        tspan=2e-3)),
                       ("tree", model.random_tree(seed=11, n_target=3000, depth_lo=5,
                                                  depth_hi=8, tspan=2e-3))):
        p, dT = built(pkg, spec)
        out.append((name, spec, p, dT))
    return out


def assert_same_state(a, b):
    np.testing.assert_array_equal(a.V, b.V)
    np.testing.assert_array_equal(a.m, b.m)
    np.testing.assert_array_equal(a.h, b.h)
    np.testing.assert_array_equal(a.n, b.n)


def assert_same_recording(r, q):
    np.testing.assert_array_equal(r.num_samples, q.num_samples)
    np.testing.assert_array_equal(r.num_spikes, q.num_spikes)
    for c in range(len(r.values)):
        np.testing.assert_array_equal(r.values[c], q.values[c])
        np.testing.assert_array_equal(r.spikes[c], q.spikes[c])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_chunk_kernel_equals_one_launch_per_step(gpu, pkg, model, precision):
    for name, spec, prob, dT in trees(pkg, model):
        runs = []
        for launch in (0, 1):
            s = pkg.SolverEx(prob, precision=precision, step_launch=launch)
            s.record([1, spec.n // 2, spec.n - 2], interval=4, capacity=400)
            # ranges that end inside a chunk (odd lengths too), then several whole chunks
            s.run(1, 38, spec.init_time, spec.end_input)
            s.run(38, 38 + 77, spec.init_time, spec.end_input)
            s.run(115, 115 + 1000, spec.init_time, spec.end_input)
            runs.append((s.get_state(), s.recording(), s.snapshot()))
            s.close()
        (sa, ra, va), (sb, rb, vb) = runs
        assert_same_state(sa, sb)
        assert_same_recording(ra, rb)
        np.testing.assert_array_equal(va, vb)
        assert np.isfinite(va).all(), name


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_chunk_kernel_with_strain_ramp(gpu, pkg, model, precision):
    """The strained rows are written between the steps of a chunk."""
    spec = model.myelinated_axon(n_nodes=12, internode_len=40e-6, tspan=2e-3)
    seg = strained(spec)
    dT = step_size(pkg, spec, seg, 0.2)
    prob = pkg.ProblemArrays.from_spec(spec, pkg.derive(spec), dT)
    t0, t1 = 30 * dT, 400 * dT
    out = []
    for launch in (0, 1):
        s = pkg.SolverEx(prob, precision=precision, step_launch=launch)
        s.set_strain(spec, seg, 0.0, 0.2, t0, t1)
        s.record([5, spec.n // 2], interval=2, capacity=300)
        s.run(1, 1 + 91, spec.init_time, spec.end_input)
        s.run(92, 92 + 500, spec.init_time, spec.end_input)
        out.append((s.get_state(), s.recording()))
        s.close()
    assert_same_state(out[0][0], out[1][0])
    assert_same_recording(out[0][1], out[1][1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_chunk_kernel_batch_with_unequal_runs(gpu, pkg, model, precision):
    """Instances whose loop ranges end at different steps, inside and between chunks."""
    specs = [model.random_tree(seed=s, n_target=n, depth_lo=4, depth_hi=7, tspan=2e-3)
             for s, n in ((3, 800), (4, 2500), (5, 1200), (6, 400))]
    built_ = [built(pkg, sp) for sp in specs]
    probs = [p for p, _ in built_]
    lengths = [37, 200, 64, 129]
    res = []
    for launch in (0, 1):
        b = pkg.Batch(probs, precision=precision, step_launch=launch)
        b.set_runs([(1, 1 + L, sp.init_time, sp.end_input) for sp, L in zip(specs, lengths)])
        b.record([(q, specs[q].n // 3) for q in range(len(specs))], interval=3, capacity=100)
        b.advance(max(lengths) + 5)
        b.synchronize()
        res.append(([b.get_state(q) for q in range(len(specs))], b.recording(), b.remaining()))
        b.close()
    for q in range(len(specs)):
        assert_same_state(res[0][0][q], res[1][0][q])
    assert_same_recording(res[0][1], res[1][1])
    np.testing.assert_array_equal(res[0][2], res[1][2])
    assert (res[1][2] == 0).all()


def test_chunk_kernel_strides_over_a_large_pack(gpu, pkg, model):
    """A mixed pack larger than the grid's threads (several elements per thread)."""
    specs = [model.random_tree(seed=20 + s, n_target=100000, depth_lo=8, depth_hi=12,
                               tspan=2e-3) for s in range(4)]
    probs = [built(pkg, sp)[0] for sp in specs]
    assert sum(p.num_elem for p in probs) > 155648  # 152 SMs x 1024 threads
    vs = []
    for launch in (0, 1):
        b = pkg.Batch(probs, precision="mixed", step_launch=launch)
        b.set_runs([(1, 1 + 150, sp.init_time, sp.end_input) for sp in specs])
        b.advance(150)
        vs.append(b.snapshot_all())
        b.close()
    for x, y in zip(*vs):
        np.testing.assert_array_equal(x, y)


def test_step_launch_option_is_checked(gpu, pkg):
    spec, prob, dT = golden_axon(pkg)
    with pytest.raises(Exception):
        pkg.SolverEx(prob, step_launch=2)


def test_kernel_launch_counter(gpu, pkg, model):
    """nrt_kernel_launches: a replayed 64-step graph counts its kernel nodes (64 steps and
    the loop-index update), a chunk launch counts itself, an implicit run its persistent
    kernel."""
    specs = [model.random_tree(seed=s, n_target=1500, depth_lo=4, depth_hi=7, tspan=2e-3)
             for s in (7, 8)]
    probs = [built(pkg, sp)[0] for sp in specs]
    counts = {}
    for launch in (0, 1):
        b = pkg.Batch(probs, precision="mixed", step_launch=launch)
        b.set_runs([(1, 1000, sp.init_time, sp.end_input) for sp in specs])
        b.advance(64)  # the exact first step and the graph capture happen here
        b.synchronize()
        l0 = pkg.kernel_launches()
        b.advance(128)
        b.synchronize()
        counts[launch] = pkg.kernel_launches() - l0
        b.close()
    assert counts[0] == 2 * (64 + 1)
    assert counts[1] == 2 * 2  # chunk kernel + loop-index update, twice
    b = pkg.Batch(probs, mode=1, precision="mixed", restart=20, tol=1e-10, tol_mode="rel")
    b.set_runs([(1, 100, sp.init_time, sp.end_input) for sp in specs])
    l0 = pkg.kernel_launches()
    b.advance(10)
    b.synchronize()
    assert pkg.kernel_launches() - l0 == 2  # the persistent kernel + loop-index update
    b.close()


def test_fp64_rate_lanes_equal_one_thread_per_element(gpu, pkg, model):
    """Small FP64 packs step with eight lanes per element (six evaluate one HH rate each,
    lane 0 finishes the element); the result is bit for bit that of one thread per element
    (step_threads set), over the exact first step and graph chunks, single trees and a
    batch."""
    axon = golden_axon(pkg)
    tree = model.random_tree(seed=12, n_target=3000, depth_lo=5, depth_hi=8, tspan=2e-3)
    cases = [[axon[1]], [built(pkg, tree)[0]],
             [built(pkg, model.random_tree(seed=s, n_target=1500, depth_lo=4, depth_hi=7,
                                           tspan=2e-3))[0] for s in (30, 31, 32)]]
    for probs in cases:
        assert sum(p.num_elem for p in probs) <= 8192  # the lanes kernel's range
        states = []
        for shape in ({}, {"step_threads": 64}):
            b = pkg.Batch(probs, precision="fp64", **shape)
            b.set_runs([(1, 1 + 300, 0.0, 3e-4)] * len(probs))
            b.advance(37)
            b.advance(200)
            states.append([b.get_state(q) for q in range(len(probs))])
            b.close()
        for a, c in zip(*states):
            assert_same_state(a, c)
