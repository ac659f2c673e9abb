"""nrt_solve_csr_static: the solve for callers that cannot allocate device memory.

Some callers own the whole device memory pool or must not allocate once running, and can
only hand over device buffers they already hold.  This entry point takes the system and
the solution vector in the caller's device memory and keeps every temporary in the
library's static device array.  Here it is checked against the solver handle's own
implicit step (nrt_calculate) on two steps in a row, within the FP64 tolerance of the
implicit tests (1e-9 V), and shown to refuse a system larger than its static array.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
REL = 1


def _static_solve(lib, torch, rp, col, val, rhs, x0, restart=16, tol=1e-11):
    dev = torch.device("cuda", 0)
    t_rp = torch.from_numpy(np.ascontiguousarray(rp, np.int32)).to(dev)
    t_col = torch.from_numpy(np.ascontiguousarray(col, np.int32)).to(dev)
    t_val = torch.from_numpy(np.ascontiguousarray(val, np.float64)).to(dev)
    t_b = torch.from_numpy(np.ascontiguousarray(rhs, np.float64)).to(dev)
    t_x = torch.from_numpy(np.ascontiguousarray(x0, np.float64).copy()).to(dev)
    torch.cuda.synchronize()
    iters = ctypes.c_int32(0)
    res = ctypes.c_double(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.nrt_solve_csr_static(len(rhs), t_rp.data_ptr(), t_col.data_ptr(), t_val.data_ptr(),
                                  t_b.data_ptr(), t_x.data_ptr(), restart, tol, REL, 0, stream,
                                  ctypes.byref(iters), ctypes.byref(res))
    return rc, t_x.cpu().numpy(), iters.value, res.value


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


def test_static_solve_refuses_oversized_systems(gpu, pkg):
    import torch
    lib = pkg.load()
    n = 400_000  # n * (2 * 16 + 5) doubles exceed the 32 MiB static array
    rp = np.arange(n + 1, dtype=np.int32)
    col = np.arange(n, dtype=np.int32)
    val = np.ones(n)
    rc, _, _, _ = _static_solve(lib, torch, rp, col, val, np.ones(n), np.zeros(n))
    assert rc == 6  # NRT_EBUDGET
    assert b"static scratch" in lib.nrt_last_error()
