"""nrt_solve_csr_static: the solve for callers that cannot allocate device memory.

Some callers own the whole device memory pool or must not allocate once running, and can
only hand over device buffers they already hold.  This entry point takes the system and
the solution vector in the caller's device memory and keeps every temporary in the
library's static device array.  Here it is checked against the solver handle's own
implicit step (nrt_calculate) on two steps in a row, within the FP64 tolerance of the
implicit tests (1e-9 V), in relative and absolute mode; shown to leave the device's free
memory unchanged once its first call has loaded it; to report a spent budget and a
non-finite system; and to refuse a system larger than its static array.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
ABS, REL = 0, 1
NRT_EINVAL, NRT_ENOCONV, NRT_EBUDGET = 1, 4, 6


class _System:
    """The system's arrays in device memory (allocated by the test, as a caller would)."""

    def __init__(self, torch, rp, col, val, rhs, x0):
        dev = torch.device("cuda", 0)
        self.rp = torch.from_numpy(np.ascontiguousarray(rp, np.int32)).to(dev)
        self.col = torch.from_numpy(np.ascontiguousarray(col, np.int32)).to(dev)
        self.val = torch.from_numpy(np.ascontiguousarray(val, np.float64)).to(dev)
        self.b = torch.from_numpy(np.ascontiguousarray(rhs, np.float64)).to(dev)
        self.x = torch.from_numpy(np.ascontiguousarray(x0, np.float64).copy()).to(dev)
        self.stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()

    def solve(self, lib, restart=16, tol=1e-11, mode=REL, max_iter=0):
        iters = ctypes.c_int32(0)
        res = ctypes.c_double(0)
        rc = lib.nrt_solve_csr_static(len(self.b), self.rp.data_ptr(), self.col.data_ptr(),
                                      self.val.data_ptr(), self.b.data_ptr(), self.x.data_ptr(),
                                      restart, tol, mode, max_iter, self.stream,
                                      ctypes.byref(iters), ctypes.byref(res))
        return rc, iters.value, res.value


def _static_solve(lib, torch, rp, col, val, rhs, x0, restart=16, tol=1e-11, mode=REL,
                  max_iter=0):
    sysm = _System(torch, rp, col, val, rhs, x0)
    rc, its, res = sysm.solve(lib, restart, tol, mode, max_iter)
    return rc, sysm.x.cpu().numpy(), its, res


def _coupled_norm(rp, col, rhs):
    rows = np.repeat(np.arange(len(rhs)), np.diff(rp))
    coupled = np.zeros(len(rhs), bool)
    coupled[rows[col != rows]] = True
    return float(np.linalg.norm(rhs[coupled]))


def _golden_system(pkg, name, active=True):
    g = load_golden(name)
    d = pkg.Derived(g["eparam"], g["hh_elem"], g["hparam"], float(g["dT_crit"]))
    prob = pkg.ProblemArrays.from_spec(g["spec"], d, float(g["dT"]))
    s = pkg.SolverIm(prob, tol=1e-11, tol_mode="rel", restart=30)
    rp, col, val, rhs = s.export_system(active)
    x0 = s.snapshot()
    s.close()
    return rp, col, val, rhs, x0


def _trees(pkg, model):
    for name in ("im_ytree_d3", "im_axon300"):
        g = load_golden(name)
        d = pkg.Derived(g["eparam"], g["hh_elem"], g["hparam"], float(g["dT_crit"]))
        yield name, g["spec"], pkg.ProblemArrays.from_spec(g["spec"], d, float(g["dT"]))
    spec = model.random_tree(seed=17, n_target=30000, dt=2.5e-5, tspan=2e-3)
    yield "rtree30k", spec, pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))


def test_static_solve_matches_handle_step_twice(gpu, pkg, model):
    import torch
    lib = pkg.load()
    for name, spec, prob in _trees(pkg, model):
        s = pkg.SolverIm(prob, tol=1e-11, tol_mode="rel", restart=30)
        for step in (1, 2):  # two calls in a row on the same static array
            t = step * prob.dT
            active = spec.init_time <= t <= spec.end_input
            rp, col, val, rhs = s.export_system(active)
            rc, x, its, res = _static_solve(lib, torch, rp, col, val, rhs, s.snapshot())
            assert rc == 0, (name, step, lib.nrt_last_error())
            assert its > 0
            s.update(active)
            s.calculate()
            ref = s.snapshot()
            err = np.abs(x - ref).max()
            assert err < TOL_FP64, (name, step, err)
        s.close()


def test_static_solve_absolute_tolerance_short_restart(gpu, pkg, model):
    """NRT_TOL_ABS at restart 4 (below the maximum) reaches the handle's step."""
    import torch
    lib = pkg.load()
    for name, spec, prob in _trees(pkg, model):
        s = pkg.SolverIm(prob, tol=1e-11, tol_mode="rel", restart=30)
        active = spec.init_time <= prob.dT <= spec.end_input
        rp, col, val, rhs = s.export_system(active)
        tol_abs = 1e-11 * _coupled_norm(rp, col, rhs)
        rc, x, its, res = _static_solve(lib, torch, rp, col, val, rhs, s.snapshot(), restart=4,
                                        tol=tol_abs, mode=ABS)
        assert rc == 0, (name, lib.nrt_last_error())
        assert res <= tol_abs and its > 0
        s.update(active)
        s.calculate()
        err = np.abs(x - s.snapshot()).max()
        s.close()
        assert err < TOL_FP64, (name, err)


def test_static_solve_budget_and_non_finite(gpu, pkg):
    """A spent budget gives NRT_ENOCONV with x at the last iterate and a finite residual; a
    NaN in the right-hand side gives NRT_EINVAL instead of running the budget out."""
    import torch
    lib = pkg.load()
    rp, col, val, rhs, x0 = _golden_system(pkg, "im_ytree_d3")
    rc, x, its, res = _static_solve(lib, torch, rp, col, val, rhs, x0, tol=1e-30, max_iter=1)
    assert rc == NRT_ENOCONV and its == 1
    assert np.isfinite(res) and res > 0
    assert np.isfinite(x).all() and np.abs(x - x0).max() > 0  # one update was applied
    bad = rhs.copy()
    bad[len(bad) // 2] = np.nan
    rc, x, its, res = _static_solve(lib, torch, rp, col, val, bad, x0)
    assert rc == NRT_EINVAL and its == 0
    assert b"not finite" in lib.nrt_last_error()
    assert np.array_equal(x, x0)


def test_static_solve_leaves_free_memory_unchanged(gpu, pkg):
    """After the first call on the device (which loads the code and with it the static
    array), further calls take no device memory: the free memory the driver reports is the
    same before and after a second call on buffers the caller already holds."""
    import torch
    lib = pkg.load()
    rp, col, val, rhs, x0 = _golden_system(pkg, "im_axon300")
    sysm = _System(torch, rp, col, val, rhs, x0)
    assert sysm.solve(lib)[0] == 0  # the first call (module load, address lookup)
    sysm.x.copy_(torch.from_numpy(x0))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc, its, res = sysm.solve(lib)
    free1, _ = torch.cuda.mem_get_info()
    assert rc == 0 and its > 0
    assert free1 == free0


def test_static_solve_refuses_oversized_systems(gpu, pkg):
    import torch
    lib = pkg.load()
    n = 400_000  # n * (2 * 16 + 6) doubles exceed the 32 MiB static array
    rp = np.arange(n + 1, dtype=np.int32)
    col = np.arange(n, dtype=np.int32)
    val = np.ones(n)
    rc, _, _, _ = _static_solve(lib, torch, rp, col, val, np.ones(n), np.zeros(n))
    assert rc == 6  # NRT_EBUDGET
    assert b"static scratch" in lib.nrt_last_error()
