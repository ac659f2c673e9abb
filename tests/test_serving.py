"""Serving: continuous batching of explicit and implicit requests (nrt_server_*)."""
import time

import numpy as np
import pytest

EX_OPTS = dict(precision="mixed")
IM_OPTS = dict(precision="mixed", restart=20, tol=1e-10, tol_mode="rel", max_iter=2000)


def _requests(pkg, model):
    """Explicit squid axons and implicit random trees of different sizes and lengths."""
    reqs = []
    for k, n in enumerate([200, 600, 300]):
        spec = model.straight_axon(n_comp=n, length=n * 1e-5, dtf=0.8, tspan=2e-3)
        d = pkg.derive(spec)
        dT = pkg.step_size(spec, d)
        reqs.append((pkg.ProblemArrays.from_spec(spec, d, dT), False,
                     (1, 1 + 300 + 150 * k, spec.init_time, spec.end_input)))
    # (25, 30000): above the server's whole-GPU threshold, so it steps on the cooperative
    # launch while the others share block-per-instance batches
    for seed, n, steps in [(21, 1200, 30), (22, 5000, 12), (23, 2500, 45), (24, 800, 20),
                           (25, 30000, 15)]:
        spec = model.random_tree(seed=seed, n_target=n, dt=2.5e-5, tspan=2e-3)
        reqs.append((pkg.ProblemArrays.from_spec(spec, pkg.derive(spec)), True,
                     (1, 1 + steps, spec.init_time, spec.end_input)))
    return reqs


def test_server_rejects_requests_over_budget(pkg, lib, model):
    """Admission control is host logic: a tree larger than the whole budget is refused
    before anything touches a device."""
    spec = model.random_tree(seed=3, n_target=5000)
    p = pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))
    srv = pkg.Server(budget_bytes=1 << 20)
    with pytest.raises(pkg.NeuriteError) as e:
        srv.submit(p, True, 1, 10, 0.0, 1.0)
    assert e.value.status == 6
    assert srv.stats().rejected == 1
    srv.close()


@pytest.mark.gpu
def test_server_results_equal_alone_runs(gpu, pkg, model):
    """Requests that arrive while others run are admitted into new resident batches and
    their results equal each request run alone (within the mixed-precision tolerance)."""
    reqs = _requests(pkg, model)
    srv = pkg.Server(budget_bytes=2 << 30, chunk_steps=16, max_wait_us=0,
                     explicit_opts=EX_OPTS, implicit_opts=IM_OPTS)
    ids = []
    for q, (p, im, run) in enumerate(reqs):
        ids.append(srv.submit(p, im, *run))
        time.sleep(0.002 * (q % 3))  # staggered arrivals
    srv.drain()
    st = srv.stats()
    assert st.completed == len(reqs) and st.rejected == 0
    assert st.batches_created >= 2          # later arrivals joined while others ran
    assert st.p99_ms >= st.p50_ms > 0
    for rid, (p, im, run) in zip(ids, reqs):
        got = srv.result(rid)
        alone = (pkg.SolverIm if im else pkg.SolverEx)(p, **(IM_OPTS if im else EX_OPTS))
        alone.run(*run)
        ref = alone.snapshot()
        assert np.abs(got - ref).max() < 1e-4, (rid, im)
        alone.close()
    srv.close()


@pytest.mark.gpu
def test_server_recording_equals_alone(gpu, pkg, model):
    """Per-request probes in the server record what each request records alone: requests
    with equal settings share batches, a request with other settings gets its own."""
    reqs = _requests(pkg, model)[:6]
    srv = pkg.Server(budget_bytes=2 << 30, chunk_steps=16, max_wait_us=0,
                     explicit_opts=EX_OPTS, implicit_opts=IM_OPTS)
    ids, probes, settings = [], [], []
    for q, (p, im, run) in enumerate(reqs):
        pr = [1, p.num_elem // 2, p.num_elem - 2]
        st = dict(interval=1 + (q == 4), capacity=400, threshold=-0.06, max_spikes=8)
        ids.append(srv.submit(p, im, *run, probes=pr, **st))
        probes.append(pr)
        settings.append(st)
    plain = srv.submit(reqs[0][0], False, *reqs[0][2])   # no probes
    srv.drain()
    # a request submitted without probes has no recording
    assert srv.lib.nrt_server_recording(srv.h, plain, None, None, None, None, None) == 7
    for rid, (p, im, run), pr, st in zip(ids, reqs, probes, settings):
        got = srv.recording(rid)
        alone = (pkg.SolverIm if im else pkg.SolverEx)(p, **(IM_OPTS if im else EX_OPTS))
        alone.record(pr, **st)
        alone.run(*run)
        want = alone.recording()
        alone.close()
        np.testing.assert_array_equal(got.num_samples, want.num_samples)
        np.testing.assert_array_equal(got.num_spikes, want.num_spikes)
        for c in range(len(pr)):
            np.testing.assert_array_equal(got.times[c], want.times[c])
            assert np.abs(got.values[c] - want.values[c]).max() < 1e-4
        assert srv.result(rid) is not None
    srv.close()
