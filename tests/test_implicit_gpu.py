"""Implicit (backward Euler) path on the GPU.

Plain FP64 is held to 1e-6 mV (1e-9 V) against the exact backward-Euler solution of the
reference's own system (the oracle's tree solve of the restated createMatrix, which is
pinned to the reference's src/solverIm-cpu.cpp through its FGMRES run at 1e-12 V); against
the reference's FGMRES output directly, the bound is that solver's own error (1e-5 V, see
test_oracle_golden.py).  Mixed precision is held to 0.1 mV.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
TOL_MIXED = 1e-4


def problem(pkg, g):
    d = pkg.Derived(g["eparam"], g["hh_elem"], g["hparam"], float(g["dT_crit"]))
    return pkg.ProblemArrays.from_spec(g["spec"], d, float(g["dT"]))


def tight(**kw):
    """FP64 solve to a relative residual of 1e-11 (the FP64 floor of b - A x on these
    stiff dx = 1-4 um trees is ~4e-13 ||b||; 1e-11 keeps the error below ~1e-12 V)."""
    o = dict(tol=1e-11, tol_mode="rel", restart=30, precond="segment")
    o.update(kw)
    return o


@pytest.mark.parametrize("name", golden_names("i"))
@pytest.mark.parametrize("precond", ["segment", "jacobi", "tree"])
def test_implicit_fp64_matches_exact_solution(gpu, pkg, orc, name, precond):
    g = load_golden(name)
    spec = g["spec"]
    steps = int(g["numStepsT"]) - 2
    s = pkg.SolverIm(problem(pkg, g), **tight(precond=precond, max_iter=20000))
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    V = s.snapshot()
    d = orc.derive(spec)
    Vo, _, _, _ = orc.implicit_run(spec, d, float(g["dT"]), 1, 1 + steps, linsolve=0)
    assert np.abs(V - Vo).max() < TOL_FP64
    # and the reference's own FGMRES output, within that solver's error
    assert np.abs(V - g["final_V"]).max() < 1e-5
    st = s.stats()
    assert st.nonconverged_steps == 0 and st.krylov_iters > 0
    s.close()


def test_implicit_system_matches_reference_assembly(gpu, pkg, orc):
    """nrt_export_system reproduces createMatrix (src/solverIm-cpu.cpp:29-183)."""
    g = load_golden("im_ytree_d3")
    spec = g["spec"]
    s = pkg.SolverIm(problem(pkg, g), **tight())
    rp, col, val, rhs = s.export_system(True)
    d = orc.derive(spec)
    # the oracle's W, K after the first update() (gates from V^n = rest)
    W = d.eparam[3].copy()
    K = d.eparam[4].copy()
    hp = d.hparam.copy()
    dt = float(g["dT"]) * 1000
    V = spec.rest_pot.copy()
    vna = (V[d.hh_elem] + hp[9] - hp[11]) / 1e-3
    vk = (V[d.hh_elem] + hp[10] - hp[11]) / 1e-3
    am = (2.5 - 0.1 * vna) / (np.exp(2.5 - 0.1 * vna) - 1); bm = 4 * np.exp(-vna / 18)
    ah = 0.07 * np.exp(-vna / 20); bh = 1 / (np.exp(3 - 0.1 * vna) + 1)
    an = (0.1 - 0.01 * vk) / (np.exp(1 - 0.1 * vk) - 1); bn = 0.125 * np.exp(-vk / 80)
    m = hp[0] + dt * (am * (1 - hp[0]) - bm * hp[0])
    h = hp[1] + dt * (ah * (1 - hp[1]) - bh * hp[1])
    n = hp[2] + dt * (an * (1 - hp[2]) - bn * hp[2])
    GNa = hp[3] * m ** 3 * h
    GK = hp[4] * n ** 4
    W[d.hh_elem] = -(GNa + GK + hp[5])
    K[d.hh_elem] = GNa * hp[6] + GK * hp[7] + hp[5] * hp[8]
    rp_o, col_o, val_o, rhs_o = orc.implicit_matrix(spec, d, W, K, spec.input_current,
                                                    float(g["dT"]), V, rhs_in=V.copy())
    np.testing.assert_array_equal(rp, rp_o)
    np.testing.assert_array_equal(col, col_o)
    np.testing.assert_allclose(val, val_o, rtol=1e-13, atol=0)
    np.testing.assert_allclose(rhs, rhs_o, rtol=1e-13, atol=0)
    s.close()


def test_implicit_dropin_loop_equals_device_loop(gpu, pkg):
    g = load_golden("im_axon300")
    spec = g["spec"]
    dT = float(g["dT"])
    a = pkg.SolverIm(problem(pkg, g), **tight())
    b = pkg.SolverIm(problem(pkg, g), **tight())
    steps = 40
    for i in range(1, 1 + steps):
        t = i * dT
        a.update(spec.init_time <= t <= spec.end_input)
        a.calculate()
    b.run(1, 1 + steps, spec.init_time, spec.end_input)
    np.testing.assert_array_equal(a.snapshot(), b.snapshot())


@pytest.mark.parametrize("precond", ["segment", "tree"])
def test_implicit_large_tree_cooperative(gpu, pkg, orc, model, precond):
    """~6.5e4-element tree on the whole-GPU cooperative kernel vs the exact solution."""
    spec = model.random_binary_tree(depth=8, seed=5, dt=2.5e-5, tspan=5e-3)
    steps = 20
    s = pkg.SolverIm(pkg.ProblemArrays.from_spec(spec, pkg.derive(spec)), **tight(precond=precond))
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    d = orc.derive(spec)
    Vo, _, _, _ = orc.implicit_run(spec, d, spec.dt_abs, 1, 1 + steps, linsolve=0)
    assert np.abs(s.snapshot() - Vo).max() < TOL_FP64


def test_config2_fp64_crank_nicolson_full_size(gpu, pkg, orc, model):
    """The Crank-Nicolson workload's tree at full size -- a depth-10 random binary tree
    (2047 branches, about 2.6e5 compartments at dx 1 um, HH everywhere, 2 nA at the root,
    dt 0.01 ms) -- in plain FP64 with that workload's solver settings (GMRES(30), tree
    preconditioner, tolerance 1e-10 relative) against the oracle's exact Crank-Nicolson
    solve, over 600 steps (6 ms: the stimulus and the first spikes), at 1e-9 V."""
    spec = model.random_binary_tree(depth=10, seed=2, tspan=6e-3)
    steps = 600
    s = pkg.SolverIm(pkg.ProblemArrays.from_spec(spec, pkg.derive(spec)), precision="fp64",
                     restart=30, tol=1e-10, tol_mode="rel", precond="tree", max_iter=2000,
                     scheme="cn")
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    V = s.snapshot()
    st = s.stats()
    s.close()
    Vo, _, _, _ = orc.implicit_run(spec, orc.derive(spec), spec.dt_abs, 1, 1 + steps,
                                   linsolve=0, scheme=1)
    assert spec.n > 250000
    assert st.nonconverged_steps == 0
    err = np.abs(V - Vo).max()
    print(f"\nconfig 2 FP64 Crank-Nicolson, n={spec.n}, {steps} steps: max |dV| = {err:.3g} V")
    assert np.nanmax(Vo) > 0.0  # the run spikes
    assert err < TOL_FP64


@pytest.mark.parametrize("steps,advance", [(15, 16), (15, 64), (14, 17)])
def test_cooperative_run_ending_inside_a_launch(gpu, pkg, orc, model, steps, advance):
    """A one-tree batch on the cooperative launch whose run ends before the launch's step
    count leaves its latest V where the host expects it."""
    spec = model.random_tree(seed=25, n_target=30000, dt=2.5e-5, tspan=2e-3)
    p = pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))
    b = pkg.Batch([p], mode=1, **tight())
    b.set_runs([(1, 1 + steps, spec.init_time, spec.end_input)])
    b.advance(advance)
    assert (b.remaining() == 0).all()
    Vo, _, _, _ = orc.implicit_run(spec, orc.derive(spec), spec.dt_abs, 1, 1 + steps, linsolve=0)
    assert np.abs(b.snapshot(0) - Vo).max() < TOL_FP64
    b.close()


def test_implicit_mixed_precision(gpu, pkg, orc):
    g = load_golden("im_ytree_d3")
    spec = g["spec"]
    steps = int(g["numStepsT"]) - 2
    s = pkg.SolverIm(problem(pkg, g), precision="mixed", restart=20, tol=1e-10, tol_mode="rel")
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    d = orc.derive(spec)
    Vo, _, _, _ = orc.implicit_run(spec, d, float(g["dT"]), 1, 1 + steps, linsolve=0)
    assert np.abs(s.snapshot() - Vo).max() < TOL_MIXED
    assert s.stats().nonconverged_steps == 0


@pytest.mark.parametrize("precision,precond", [("fp64", "segment"), ("mixed", "segment"),
                                               ("fp64", "tree"), ("mixed", "tree")])
def test_implicit_batch_alone_equals_in_mix(gpu, pkg, orc, model, precision, precond):
    """Uneven trees in one persistent block-per-instance launch give what each gives alone."""
    specs = [model.random_tree(seed=s, n_target=n, dt=2.5e-5, tspan=1e-3)
             for s, n in [(1, 1500), (2, 6000), (3, 900), (4, 3000)]]
    opts = tight(precond=precond) if precision == "fp64" else dict(
        precision="mixed", restart=20, tol=1e-10, tol_mode="rel", precond=precond)
    probs = [pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs]
    b = pkg.Batch(probs, mode=1, **opts)
    steps = [25, 40, 10, 33]
    b.set_runs([(1, 1 + k, sp.init_time, sp.end_input) for k, sp in zip(steps, specs)])
    b.advance(max(steps))
    assert (b.remaining() == 0).all()
    tol = TOL_FP64 if precision == "fp64" else TOL_MIXED
    for k, sp in enumerate(specs):
        alone = pkg.SolverIm(pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)), **opts)
        alone.run(1, 1 + steps[k], sp.init_time, sp.end_input)
        Va = alone.snapshot()
        Vb = b.snapshot(k)
        assert np.abs(Vb - Va).max() < tol
        d = orc.derive(sp)
        Vo, _, _, _ = orc.implicit_run(sp, d, sp.dt_abs, 1, 1 + steps[k], linsolve=0)
        assert np.abs(Vb - Vo).max() < tol
        alone.close()
    b.close()


def test_implicit_budget_exhaustion_reported(gpu, pkg):
    """A Krylov budget of one iteration cannot reach 1e-11: calculate() reports
    NRT_ENOCONV and the state still advances (the reference would exit(0))."""
    g = load_golden("im_axon300")
    s = pkg.SolverIm(problem(pkg, g), **tight(max_iter=1, precond="none"))
    V0 = s.snapshot()
    s.update(True)
    with pytest.raises(pkg.NeuriteError) as e:
        s.calculate()
    assert e.value.status == 4
    assert not np.array_equal(s.snapshot(), V0)
    assert s.stats().nonconverged_steps == 1


def test_tree_preconditioner_needs_few_iterations(gpu, pkg, model):
    """With the exact tree solve as preconditioner, each FP64 GMRES solve needs about one
    iteration per refinement cycle, whatever the branching."""
    spec = model.random_tree(seed=5, n_target=20000, dt=2.5e-5, tspan=1e-3)
    prob = pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))
    s = pkg.SolverIm(prob, **tight(precond="tree"))
    s.run(1, 21, spec.init_time, spec.end_input)
    st = s.stats()
    assert st.nonconverged_steps == 0
    assert st.krylov_iters <= 20 * 3


@pytest.mark.parametrize("name", golden_names("i"))
@pytest.mark.parametrize("precond", ["segment", "tree"])
def test_bicgstab_fp64_matches_exact_solution(gpu, pkg, orc, name, precond):
    """BiCGSTAB, the reference GPU solver's method (src/solverIm-gpu.cpp:725-843).  Its
    unpreconditioned form (precond="none") does not reach 1e-11 within 20000 iterations on
    these stiff trees; test_bicgstab_unpreconditioned_reports_budget covers that."""
    g = load_golden(name)
    spec = g["spec"]
    steps = int(g["numStepsT"]) - 2
    s = pkg.SolverIm(problem(pkg, g), **tight(krylov="bicgstab", precond=precond, max_iter=20000))
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    d = orc.derive(spec)
    Vo, _, _, _ = orc.implicit_run(spec, d, float(g["dT"]), 1, 1 + steps, linsolve=0)
    assert np.abs(s.snapshot() - Vo).max() < TOL_FP64
    st = s.stats()
    assert st.nonconverged_steps == 0 and st.krylov_iters > 0
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bicgstab_batch_and_cooperative(gpu, pkg, orc, model, precision):
    """BiCGSTAB with the tree preconditioner in a batch and on the whole-GPU launch."""
    opts = tight(krylov="bicgstab", precond="tree") if precision == "fp64" else dict(
        precision="mixed", krylov="bicgstab", restart=20, tol=1e-10, tol_mode="rel", precond="tree")
    tol = TOL_FP64 if precision == "fp64" else TOL_MIXED
    specs = [model.random_tree(seed=s, n_target=n, dt=2.5e-5, tspan=1e-3)
             for s, n in [(11, 2500), (12, 800), (13, 7000)]]
    probs = [pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs]
    b = pkg.Batch(probs, mode=1, **opts)
    b.set_runs([(1, 21, sp.init_time, sp.end_input) for sp in specs])
    b.advance(20)
    for k, sp in enumerate(specs):
        Vo, _, _, _ = orc.implicit_run(sp, orc.derive(sp), sp.dt_abs, 1, 21, linsolve=0)
        assert np.abs(b.snapshot(k) - Vo).max() < tol
    assert b.stats().nonconverged_steps == 0
    b.close()
    spec = model.random_binary_tree(depth=7, seed=3, dt=2.5e-5, tspan=5e-3)
    s = pkg.SolverIm(pkg.ProblemArrays.from_spec(spec, pkg.derive(spec)), **opts)
    s.run(1, 11, spec.init_time, spec.end_input)
    Vo, _, _, _ = orc.implicit_run(spec, orc.derive(spec), spec.dt_abs, 1, 11, linsolve=0)
    assert np.abs(s.snapshot() - Vo).max() < tol
    s.close()


def test_bicgstab_unpreconditioned_reports_budget(gpu, pkg):
    """The reference's unpreconditioned BiCGSTAB stalls on a stiff tree: the step ends at its
    iteration budget with NRT_ENOCONV and a finite state (the reference keeps going silently)."""
    g = load_golden("im_axon300")
    s = pkg.SolverIm(problem(pkg, g), **tight(krylov="bicgstab", precond="none", max_iter=300))
    s.update(True)
    with pytest.raises(pkg.NeuriteError) as e:
        s.calculate()
    assert e.value.status == 4
    assert np.isfinite(s.snapshot()).all()
    assert s.stats().nonconverged_steps == 1
    s.close()


@pytest.mark.parametrize("refinement", ["gmres", "auto"])
def test_pass_counts_follow_the_gmres_structure(gpu, pkg, model, refinement):
    """The kernel's pass counters (used for the bandwidth accounting): one preconditioner
    application per Arnoldi step or Richardson step, one FP64 residual per solution update
    (every update is followed by its residual check), and the basis reads of step j are
    j + 1.  With refinement="auto" (mixed precision, tree preconditioner) every step opens
    with a Richardson step."""
    specs = [model.random_tree(seed=s, n_target=n, dt=2.5e-5, tspan=1e-3)
             for s, n in [(41, 3000), (42, 12000)]]
    b = pkg.Batch([pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs], mode=1,
                  precision="mixed", restart=20, tol=1e-10, tol_mode="rel",
                  refinement=refinement)
    b.set_runs([(1, 21, sp.init_time, sp.end_input) for sp in specs])
    b.advance(20)
    it = b.instance_stats()["iters"]
    pc = b.pass_counts()
    b.close()
    np.testing.assert_array_equal(pc["applies"], it + pc["richardson"])
    np.testing.assert_array_equal(pc["residuals"], pc["xupdates"])
    assert (pc["xupdates"] >= 20).all()            # at least one update per step
    assert (pc["basis"] >= it).all() and (pc["basis"] <= it * (it + 1) // 2).all()
    if refinement == "gmres":
        assert (pc["richardson"] == 0).all() and (it >= 20).all()
    else:
        assert (pc["richardson"] >= 20).all()


def test_richardson_refinement_matches_gmres_cycles(gpu, pkg, model):
    """Mixed precision with the tree preconditioner: Richardson refinement cycles reach the
    same FP64 residual test as GMRES cycles, so both give the backward-Euler solution to
    the tolerance (1e-10 relative here); they differ by far less than the accuracy bar."""
    specs = [model.random_tree(seed=s, n_target=n, dt=2.5e-5, tspan=2e-3)
             for s, n in [(51, 1500), (52, 30000), (53, 90000)]]
    probs = [pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs]
    out = {}
    for refinement in ("gmres", "auto"):
        b = pkg.Batch(probs, mode=1, precision="mixed", restart=20, tol=1e-10, tol_mode="rel",
                      refinement=refinement)
        b.set_runs([(1, 41, sp.init_time, sp.end_input) for sp in specs])
        b.advance(40)
        st = b.instance_stats()
        assert (st["nonconverged"] == 0).all()
        out[refinement] = (b.snapshot_all(), b.pass_counts())
        b.close()
    for x, y in zip(out["gmres"][0], out["auto"][0]):
        assert np.abs(x - y).max() < 1e-8  # 1e-5 mV
    assert (out["auto"][1]["basis"] == 0).all()  # every cycle took the Richardson step


def test_richardson_hands_over_to_gmres_when_it_stalls(gpu, pkg, model):
    """A tolerance below what FP64 rounding of the residual allows: the Richardson steps
    stop lowering the residual tenfold, the rest of each step runs GMRES cycles, and the
    budget ends the step (reported as non-converged)."""
    spec = model.random_tree(seed=54, n_target=5000, dt=2.5e-5, tspan=1e-3)
    b = pkg.Batch([pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))], mode=1,
                  precision="mixed", restart=20, tol=1e-19, tol_mode="rel", max_iter=8)
    b.set_runs([(1, 4, spec.init_time, spec.end_input)])
    b.advance(3)
    st = b.instance_stats()
    pc = b.pass_counts()
    b.close()
    assert pc["richardson"][0] >= 3 and pc["basis"][0] > 0
    assert st["nonconverged"][0] == 3
    assert pc["richardson"][0] + st["iters"][0] == 3 * 8  # the budget counts both kinds


@pytest.mark.parametrize("name", golden_names("i"))
@pytest.mark.parametrize("precond", ["tree", "segment"])
def test_crank_nicolson_fp64_matches_exact_solution(gpu, pkg, orc, name, precond):
    """Crank-Nicolson (not in the reference) against the oracle's restatement, solved
    exactly, at the FP64 bar."""
    g = load_golden(name)
    spec = g["spec"]
    steps = int(g["numStepsT"]) - 2
    s = pkg.SolverIm(problem(pkg, g), scheme="cn", **tight(precond=precond, max_iter=20000))
    s.run(1, 1 + steps, spec.init_time, spec.end_input)
    d = orc.derive(spec)
    Vo, _, _, _ = orc.implicit_run(spec, d, float(g["dT"]), 1, 1 + steps, linsolve=0, scheme=1)
    assert np.abs(s.snapshot() - Vo).max() < TOL_FP64
    Vbe, _, _, _ = orc.implicit_run(spec, d, float(g["dT"]), 1, 1 + steps, linsolve=0)
    assert np.abs(Vo - Vbe).max() > 1e-6   # a different scheme indeed
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_crank_nicolson_batch_and_cooperative(gpu, pkg, orc, model, precision):
    specs = [model.random_tree(seed=s, n_target=n, dt=2.5e-5, tspan=1e-3)
             for s, n in [(81, 2000), (82, 30000)]]
    opts = tight(precond="tree") if precision == "fp64" else dict(
        precision="mixed", restart=20, tol=1e-10, tol_mode="rel")
    tol = TOL_FP64 if precision == "fp64" else TOL_MIXED
    probs = [pkg.ProblemArrays.from_spec(sp, pkg.derive(sp)) for sp in specs]
    steps = [20, 12]
    b = pkg.Batch(probs, mode=1, scheme="cn", **opts)                 # block per instance
    b.set_runs([(1, 1 + k, sp.init_time, sp.end_input) for k, sp in zip(steps, specs)])
    b.advance(max(steps))
    for q, sp in enumerate(specs):
        Vo, _, _, _ = orc.implicit_run(sp, orc.derive(sp), sp.dt_abs, 1, 1 + steps[q],
                                       linsolve=0, scheme=1)
        assert np.abs(b.snapshot(q) - Vo).max() < tol
        if q == 1:  # the large tree alone: the cooperative whole-GPU launch
            s = pkg.SolverIm(probs[q], scheme="cn", **opts)
            s.run(1, 1 + steps[q], sp.init_time, sp.end_input)
            assert np.abs(s.snapshot() - Vo).max() < tol
            s.close()
    b.close()


def test_crank_nicolson_system_matches_oracle(gpu, pkg, orc):
    """nrt_export_system in Crank-Nicolson mode: the oracle's transform of the reference's
    backward-Euler matrix (A + C/dT, 2 b + C/dT V^n - A V^n)."""
    g = load_golden("im_ytree_d3")
    spec = g["spec"]
    be = pkg.SolverIm(problem(pkg, g), **tight())
    cn = pkg.SolverIm(problem(pkg, g), scheme="cn", **tight())
    rp, col, val, rhs = be.export_system(True)
    rp2, col2, val2, rhs2 = cn.export_system(True)
    np.testing.assert_array_equal(rp, rp2)
    np.testing.assert_array_equal(col, col2)
    d = orc.derive(spec)
    n = spec.n
    cdt = d.eparam[0] * d.eparam[2] / float(g["dT"])
    V = spec.rest_pot.copy()
    av = np.array([val[rp[j]:rp[j + 1]] @ V[col[rp[j]:rp[j + 1]]] for j in range(n)])
    ident = (rp[1:] - rp[:-1]) == 1
    want_val = val.copy()
    want_rhs = rhs.copy()
    for j in np.nonzero(~ident)[0]:
        k = rp[j] + int(np.nonzero(col[rp[j]:rp[j + 1]] == j)[0][0])
        want_val[k] += cdt[j]
        want_rhs[j] = 2 * rhs[j] + cdt[j] * V[j] - av[j]
    np.testing.assert_allclose(val2, want_val, rtol=1e-13, atol=0)
    np.testing.assert_allclose(rhs2[~ident], want_rhs[~ident], rtol=1e-12, atol=1e-20)
    be.close()
    cn.close()
