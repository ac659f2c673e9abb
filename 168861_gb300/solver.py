"""Host-side mirror of the reference's solver interface over the C ABI.

`SolverEx` / `SolverIm` follow `class Solver` (inc/solver.h:12-24): update(input_active),
calculate(), snapshot().  They are built from the same inputs as the reference solver
constructors (src/solverEx-gpu.cpp:204-439, src/solverIm-gpu.cpp:381-682): the tree and
the per-element values produced by the parameter pipeline (src/init.cpp:235-298), which
`derive()` computes on the host with the library's nrt_derive.

`Batch` packs many trees into one device-resident set of arrays and advances them with
one launch per step (no reference counterpart).
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import _lib, model
from ._lib import check

_PREC = {"fp64": _lib.NRT_FP64, "mixed": _lib.NRT_MIXED}
_KRY = {"gmres": _lib.NRT_GMRES, "bicgstab": _lib.NRT_BICGSTAB}
_PC = {"none": _lib.NRT_PRECOND_NONE, "jacobi": _lib.NRT_PRECOND_JACOBI,
       "segment": _lib.NRT_PRECOND_SEGMENT, "tree": _lib.NRT_PRECOND_TREE}


@dataclasses.dataclass
class Derived:
    """Output of the parameter pipeline: eparam [6][n] = (c_m, r_a, dX, W, K, critical dT),
    hh_elem [num_hh], hparam [12][num_hh] = (m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L,
    LS_Na, LS_K, rest), dT_crit."""
    eparam: np.ndarray
    hh_elem: np.ndarray
    hparam: np.ndarray
    dT_crit: float

    @property
    def num_hh(self) -> int:
        return int(self.hh_elem.shape[0])


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def derive(spec) -> Derived:
    """Runs the reference's parameter pipeline (nrt_derive) for a model.TreeSpec."""
    lib = _lib.load()
    n = spec.n
    nh = int(np.count_nonzero(spec.kind == 1))
    isp = spec.ispec()
    dsp = spec.dspec()
    ep = np.zeros((6, n))
    he = np.zeros(max(nh, 1), np.int32)
    hpar = np.zeros((12, max(nh, 1)))
    nho = ctypes.c_int32(0)
    crit = ctypes.c_double(0)
    check(lib.nrt_derive(n, _p(isp, ctypes.c_int32), _p(dsp, ctypes.c_double), int(spec.myelin),
                         spec.e_max, _p(ep, ctypes.c_double), _p(he, ctypes.c_int32),
                         _p(hpar, ctypes.c_double), ctypes.byref(nho), ctypes.byref(crit)),
          "nrt_derive")
    hparam = np.ascontiguousarray(hpar.reshape(12, max(nh, 1))[:, :nh]) if nh else np.zeros((12, 0))
    return Derived(ep, he[:nh].copy(), hparam, crit.value)


def derive_batch(specs) -> list:
    """The parameter pipeline for many trees in one GPU call (nrt_derive_batch); the same
    results as derive() per tree up to the last bits of the device's math."""
    lib = _lib.load()
    count = len(specs)
    sizes = np.array([sp.n for sp in specs], np.int64)
    off = np.zeros(count + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    T = int(off[-1])
    isp = np.empty((5, T), np.int32)
    dsp = np.empty((12, T))
    rows_i, rows_d = model.ISPEC_ROWS, model.DSPEC_ROWS
    for k, sp in enumerate(specs):  # one copy per row, straight into the packed arrays
        a, b = off[k], off[k + 1]
        for r, name in enumerate(rows_i):
            isp[r, a:b] = getattr(sp, name)
        for r, name in enumerate(rows_d):
            dsp[r, a:b] = getattr(sp, name)
    my = np.array([int(sp.myelin) for sp in specs], np.int32)
    em = np.array([float(sp.e_max) for sp in specs])
    ep = np.empty((6, T))
    hoff = np.zeros(count + 1, np.int64)
    nh = int(sum(int(np.count_nonzero(sp.kind == 1)) for sp in specs))
    he = np.empty(max(nh, 1), np.int32)
    hp = np.empty((12, max(nh, 1)))
    crit = np.empty(count)
    check(lib.nrt_derive_batch(count, _p(off, ctypes.c_int64), _p(isp, ctypes.c_int32),
                               _p(dsp, ctypes.c_double), _p(my, ctypes.c_int32),
                               _p(em, ctypes.c_double), _p(ep, ctypes.c_double),
                               _p(he, ctypes.c_int32), _p(hp, ctypes.c_double),
                               _p(hoff, ctypes.c_int64), _p(crit, ctypes.c_double)),
          "nrt_derive_batch")
    out = []
    for k in range(count):  # views into the packed results
        a, b = int(off[k]), int(off[k + 1])
        h0, h1 = int(hoff[k]), int(hoff[k + 1])
        out.append(Derived(ep[:, a:b], he[h0:h1], hp[:, h0:h1], float(crit[k])))
    return out


def step_size(spec, d: Derived) -> float:
    """dT = dtf * critical dT, or the spec's absolute step (src/neurite.cpp:171-173)."""
    return spec.dt_abs if spec.dt_abs > 0 else d.dT_crit * spec.dtf


def measurement_point(dx, dist_mes: float) -> int:
    """The reference's measurement point (src/init.cpp:339-358) for per-element lengths
    dx (after the strain scaling) and a distance: nrt_measurement_point."""
    lib = _lib.load()
    d = np.ascontiguousarray(dx, dtype=np.float64)
    out = ctypes.c_int32(0)
    check(lib.nrt_measurement_point(len(d), _p(d, ctypes.c_double), float(dist_mes),
                                    ctypes.byref(out)), "nrt_measurement_point")
    return out.value


@dataclasses.dataclass
class Recording:
    """What device-side recording kept, per probe in configuration order: the samples
    (times i*dT and values) and the spike times.  num_samples / num_spikes count every
    sample and crossing, also those past the kept capacity."""
    times: list
    values: list
    num_samples: np.ndarray
    spikes: list
    num_spikes: np.ndarray

    def trace_text(self, probe: int = 0) -> str:
        """One probe's samples in the reference's trace format (src/neurite.cpp:248:
        "%.20f %.20f" of time and potential, one line per sample)."""
        return "".join("%.20f %.20f\n" % (t, v)
                       for t, v in zip(self.times[probe], self.values[probe]))


@dataclasses.dataclass
class State:
    """A tree's state (nrt_get_state): V, the other potential buffer, and the gates of its
    HH elements in HH order."""
    V: np.ndarray
    V_other: np.ndarray
    m: np.ndarray
    h: np.ndarray
    n: np.ndarray


def _state_get(fn, h, args, ne, nh, where):
    st = State(np.empty(ne), np.empty(ne), np.empty(nh), np.empty(nh), np.empty(nh))
    g = [_p(x, ctypes.c_double) if len(x) else None for x in (st.m, st.h, st.n)]
    check(fn(h, *args, _p(st.V, ctypes.c_double), _p(st.V_other, ctypes.c_double), *g), where)
    return st


def _state_set(fn, h, args, st: State, where):
    arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
            for a in (st.V, st.V_other, st.m, st.h, st.n)]
    ptr = [None if a is None or not len(a) else _p(a, ctypes.c_double) for a in arrs]
    check(fn(h, *args, *ptr), where)


def _strain_config(spec_rows, instances, elements, kinds, myelin, e_max, eps0, eps1, t0, t1,
                   keep):
    el = np.ascontiguousarray(elements, dtype=np.int32)
    kd = np.ascontiguousarray(kinds, dtype=np.int32)
    ds = np.ascontiguousarray(spec_rows, dtype=np.float64)
    keep += [el, kd, ds]
    c = _lib.StrainConfig()
    c.num_elem = len(el)
    c.element = _p(el, ctypes.c_int32)
    c.kind = _p(kd, ctypes.c_int32)
    c.dspec = _p(ds, ctypes.c_double)
    if instances is not None:
        ins = np.ascontiguousarray(instances, dtype=np.int32)
        keep.append(ins)
        c.instance = _p(ins, ctypes.c_int32)
    c.myelin, c.e_max = int(myelin), float(e_max)
    c.eps0, c.eps1, c.t0, c.t1 = float(eps0), float(eps1), float(t0), float(t1)
    return c


def strain_rows(spec, elements) -> np.ndarray:
    """The unstrained description of some elements of a tree (nrt_derive's dspec rows)."""
    return np.ascontiguousarray(spec.dspec()[:, np.asarray(elements)])


class _Recorder:
    """nrt_record / nrt_record_read (and the batch forms) for a handle."""

    def _record(self, fn, instances, elements, origin, interval, capacity, threshold,
                max_spikes):
        el = np.ascontiguousarray(elements, dtype=np.int32)
        cfg = _lib.RecordConfig()
        cfg.num_probes = len(el)
        self._rec_keep = [el]
        cfg.element = _p(el, ctypes.c_int32)
        if instances is not None:
            ins = np.ascontiguousarray(instances, dtype=np.int32)
            self._rec_keep.append(ins)
            cfg.instance = _p(ins, ctypes.c_int32)
        cfg.origin = int(origin)
        cfg.interval = int(interval)
        cfg.capacity = int(capacity)
        cfg.threshold = float(threshold)
        cfg.max_spikes = int(max_spikes)
        check(fn(self.h, ctypes.byref(cfg)), fn.__name__)
        self._rec_shape = (len(el), int(capacity), int(max_spikes))

    def _read(self, fn) -> Recording:
        P, cap, ms = getattr(self, "_rec_shape", (0, 0, 0))
        ns = np.zeros(P, np.int64)
        nk = np.zeros(P, np.int32)
        t = np.zeros((P, max(cap, 1)))
        v = np.zeros((P, max(cap, 1)))
        sp = np.zeros((P, max(ms, 1)))
        check(fn(self.h, _p(ns, ctypes.c_int64), _p(t, ctypes.c_double), _p(v, ctypes.c_double),
                 _p(nk, ctypes.c_int32), _p(sp, ctypes.c_double)), fn.__name__)
        kept = np.minimum(ns, cap)
        ks = np.minimum(nk, ms)
        return Recording([t[p, :kept[p]].copy() for p in range(P)],
                         [v[p, :kept[p]].copy() for p in range(P)], ns,
                         [sp[p, :ks[p]].copy() for p in range(P)], nk)


class ProblemArrays:
    """Keeps the numpy arrays of one nrt_problem alive and exposes the C struct."""

    def __init__(self, *, mother, dr, dl, branching, terminals, dx, c_m, r_a, W, K, input,
                 hh_elem, m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L, ls_Na, ls_K, rest, V0,
                 V1=None, dT):
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self.arrays = dict(mother=i32(mother), dr=i32(dr), dl=i32(dl), branching=i32(branching),
                           terminals=i32(terminals), dx=f64(dx), c_m=f64(c_m), r_a=f64(r_a),
                           W=f64(W), K=f64(K), input=f64(input), hh_elem=i32(hh_elem), m=f64(m),
                           h=f64(h), n=f64(n), g_Na=f64(g_Na), g_K=f64(g_K), G_L=f64(G_L),
                           E_Na=f64(E_Na), E_K=f64(E_K), E_L=f64(E_L), ls_Na=f64(ls_Na),
                           ls_K=f64(ls_K), rest=f64(rest), V0=f64(V0))
        if V1 is not None:
            self.arrays["V1"] = f64(V1)
        a = self.arrays
        s = _lib.Problem()
        s.num_elem = len(a["mother"])
        s.num_term = len(a["terminals"])
        s.num_hh = len(a["hh_elem"])
        s.dT = float(dT)
        for k, v in a.items():
            setattr(s, k, _p(v, ctypes.c_int32 if v.dtype == np.int32 else ctypes.c_double))
        self.struct = s
        self.dT = float(dT)

    @property
    def num_elem(self) -> int:
        return int(self.struct.num_elem)

    @classmethod
    def from_spec(cls, spec, d: Derived, dT: float | None = None, V0=None, V1=None,
                  hparam=None):
        """Inputs of the reference solver constructors for a spec after derivation."""
        dT = step_size(spec, d) if dT is None else dT
        hp = d.hparam if hparam is None else hparam
        V0 = spec.rest_pot.copy() if V0 is None else V0  # setting_rest_pot, src/init.cpp:260-267
        e = d.eparam
        return cls(mother=spec.mother, dr=spec.dr, dl=spec.dl, branching=spec.branching,
                   terminals=spec.terminals, dx=e[2], c_m=e[0], r_a=e[1], W=e[3], K=e[4],
                   input=spec.input_current, hh_elem=d.hh_elem, m=hp[0], h=hp[1], n=hp[2],
                   g_Na=hp[3], g_K=hp[4], G_L=hp[5], E_Na=hp[6], E_K=hp[7], E_L=hp[8],
                   ls_Na=hp[9], ls_K=hp[10], rest=hp[11], V0=V0, V1=V1, dT=dT)


def kernel_launches() -> int:
    """Kernels the library has launched in this process so far (nrt_kernel_launches)."""
    return int(_lib.load().nrt_kernel_launches())


def make_options(mode: int, precision: str = "fp64", krylov: str = "gmres",
                 precond: str = "tree", restart: int = 30, tol: float = 1e-14,
                 tol_mode: str = "abs", max_iter: int = 0, use_graphs: bool = True,
                 device: int = -1, schedule: int = 0, tiled: bool = True,
                 scheme: str = "be", tile_ctas_per_sm: int = 0,
                 step_threads: int = 0, inner_tol: float = 0.0,
                 step_launch: int = 0, refinement: str = "auto") -> _lib.Options:
    lib = _lib.load()
    o = _lib.Options()
    check(lib.nrt_options_default(ctypes.byref(o)), "nrt_options_default")
    o.mode = mode
    o.precision = _PREC[precision]
    o.krylov = _KRY[krylov]
    o.precond = _PC[precond]
    o.restart = restart
    o.tol = tol
    o.tol_mode = _lib.NRT_TOL_ABS if tol_mode == "abs" else _lib.NRT_TOL_REL
    o.max_iter = max_iter
    o.use_graphs = int(use_graphs)
    o.device = device
    o.schedule = int(schedule)
    o.tiled = int(bool(tiled))
    o.scheme = {"be": _lib.NRT_BACKWARD_EULER, "cn": _lib.NRT_CRANK_NICOLSON}[scheme]
    o.tile_ctas_per_sm = int(tile_ctas_per_sm)
    o.step_threads = int(step_threads)
    o.inner_tol = float(inner_tol)
    o.step_launch = int(step_launch)
    o.refinement = {"auto": 0, "gmres": 1}[refinement]
    return o


class Solver(_Recorder):
    """inc/solver.h:12-24 over the C ABI."""

    mode = _lib.NRT_EXPLICIT

    def __init__(self, problem: ProblemArrays, **opts):
        self.lib = _lib.load()
        self.problem = problem
        self.options = make_options(self.mode, **opts)
        h = ctypes.c_void_p()
        check(self.lib.nrt_create(ctypes.byref(problem.struct), ctypes.byref(self.options),
                                  ctypes.byref(h)), "nrt_create")
        self.h = h
        self.n = problem.num_elem
        self.num_hh = int(problem.struct.num_hh)

    def update(self, input_active: bool) -> None:
        check(self.lib.nrt_update(self.h, int(bool(input_active))), "nrt_update")

    def calculate(self) -> None:
        check(self.lib.nrt_calculate(self.h), "nrt_calculate")

    def snapshot(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty(self.n) if out is None else out
        check(self.lib.nrt_snapshot(self.h, _p(out, ctypes.c_double)), "nrt_snapshot")
        return out

    def run(self, i_begin: int, i_end: int, init_time: float, end_input: float) -> None:
        """The driver loop of src/neurite.cpp:224-236 for i in [i_begin, i_end)."""
        check(self.lib.nrt_run(self.h, int(i_begin), int(i_end), float(init_time),
                               float(end_input)), "nrt_run")

    def synchronize(self) -> None:
        check(self.lib.nrt_synchronize(self.h), "nrt_synchronize")

    def set_strain(self, spec, elements, eps0: float, eps1: float, t0: float, t1: float) -> None:
        """Strain of `elements` of `spec` (this solver's tree) ramping linearly from eps0 at
        t0 to eps1 at t1 (nrt_set_strain); an empty list stops it."""
        el = np.asarray(elements, dtype=np.int32)
        keep = []
        c = _strain_config(strain_rows(spec, el), None, el, spec.kind[el], spec.myelin,
                           spec.e_max, eps0, eps1, t0, t1, keep)
        check(self.lib.nrt_set_strain(self.h, ctypes.byref(c)), "nrt_set_strain")

    def get_state(self) -> State:
        return _state_get(self.lib.nrt_get_state, self.h, (), self.n, self.num_hh, "nrt_get_state")

    def set_state(self, st: State) -> None:
        _state_set(self.lib.nrt_set_state, self.h, (), st, "nrt_set_state")

    def record(self, elements, interval: int = 0, origin: int = 1, capacity: int = 4096,
               threshold: float = 0.0, max_spikes: int = 64) -> None:
        """Records V at `elements` on the device during run(): a sample every
        interval + 1 loop iterations counted from `origin` (the reference driver's rule),
        and upward crossings of `threshold` (V).  Replaces any earlier recording."""
        self._record(self.lib.nrt_record, None, elements, origin, interval, capacity,
                     threshold, max_spikes)

    def recording(self) -> Recording:
        return self._read(self.lib.nrt_record_read)

    def stream(self) -> int:
        """The handle's cudaStream_t as an integer (for timing events on it)."""
        v = ctypes.c_void_p()
        check(self.lib.nrt_get_stream(self.h, ctypes.byref(v)), "nrt_get_stream")
        return int(v.value or 0)

    def gates(self):
        nh = self.num_hh
        m, h, n = np.empty(nh), np.empty(nh), np.empty(nh)
        if nh:
            check(self.lib.nrt_get_gates(self.h, _p(m, ctypes.c_double), _p(h, ctypes.c_double),
                                         _p(n, ctypes.c_double)), "nrt_get_gates")
        return m, h, n

    def stats(self) -> _lib.Stats:
        st = _lib.Stats()
        check(self.lib.nrt_get_stats(self.h, ctypes.byref(st)), "nrt_get_stats")
        return st

    def export_system(self, input_active: bool):
        n = self.n
        cap = 4 * n + 2
        rp = np.zeros(n + 1, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        rhs = np.zeros(n)
        nnz = ctypes.c_int32(0)
        check(self.lib.nrt_export_system(self.h, int(bool(input_active)), _p(rp, ctypes.c_int32),
                                         _p(col, ctypes.c_int32), _p(val, ctypes.c_double),
                                         _p(rhs, ctypes.c_double), ctypes.byref(nnz)),
              "nrt_export_system")
        k = nnz.value
        return rp, col[:k].copy(), val[:k].copy(), rhs

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.nrt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class SolverEx(Solver):
    """Replaces SolverExGPU / SolverExCPU (explicit forward Euler)."""
    mode = _lib.NRT_EXPLICIT


class SolverIm(Solver):
    """Replaces SolverImGPU / SolverImCPU (implicit backward Euler)."""
    mode = _lib.NRT_IMPLICIT_BE


class Batch(_Recorder):
    """Many independent trees advanced together (one launch per step for all of them)."""

    def __init__(self, problems: list[ProblemArrays], mode: int = _lib.NRT_EXPLICIT,
                 autotune=False, **opts):
        """opts: make_options keywords.  autotune: True, or a dict of autotune.tune
        keywords (cache, steps, sample_elements, restarts ...), picks the launch shape by
        timing the candidates on this workload (cached per device and workload size);
        options given here win over the tuned ones.  The choice is in self.tuning."""
        self.lib = _lib.load()
        self.problems = problems
        self.tuning = None
        if autotune:
            from .autotune import tune
            kw = dict(autotune) if isinstance(autotune, dict) else {}
            rest = {k: v for k, v in opts.items() if k != "precision"}
            self.tuning = tune(problems, mode, opts.get("precision", "fp64"), **kw, **rest)
            for k, v in self.tuning["options"].items():
                opts.setdefault(k, v)
        arr = (_lib.Problem * len(problems))(*[p.struct for p in problems])
        self._arr = arr
        self.options = make_options(mode, **opts)
        h = ctypes.c_void_p()
        check(self.lib.nrt_batch_create(arr, len(problems), ctypes.byref(self.options),
                                        ctypes.byref(h)), "nrt_batch_create")
        self.h = h
        self.count = len(problems)

    def set_runs(self, runs) -> None:
        """runs: iterable of (i_begin, i_end, init_time, end_input)."""
        arr = (_lib.InstanceRun * self.count)(*[_lib.InstanceRun(int(a), int(b), float(c), float(d))
                                                  for a, b, c, d in runs])
        check(self.lib.nrt_batch_set_runs(self.h, arr), "nrt_batch_set_runs")

    def advance(self, steps: int) -> None:
        check(self.lib.nrt_batch_advance(self.h, int(steps)), "nrt_batch_advance")

    def synchronize(self) -> None:
        check(self.lib.nrt_batch_synchronize(self.h), "nrt_batch_synchronize")

    def set_strain(self, i: int, spec, elements, eps0: float, eps1: float, t0: float,
                   t1: float) -> None:
        """As Solver.set_strain, for `elements` of instance i (whose tree is `spec`)."""
        el = np.asarray(elements, dtype=np.int32)
        keep = []
        c = _strain_config(strain_rows(spec, el), np.full(len(el), int(i), np.int32), el,
                           spec.kind[el], spec.myelin, spec.e_max, eps0, eps1, t0, t1, keep)
        check(self.lib.nrt_batch_set_strain(self.h, ctypes.byref(c)), "nrt_batch_set_strain")

    def get_state(self, i: int) -> State:
        p = self.problems[i]
        return _state_get(self.lib.nrt_batch_get_state, self.h, (int(i),), p.num_elem,
                          int(p.struct.num_hh), "nrt_batch_get_state")

    def set_state(self, i: int, st: State) -> None:
        _state_set(self.lib.nrt_batch_set_state, self.h, (int(i),), st, "nrt_batch_set_state")

    def record(self, probes, interval: int = 0, origin: int = 1, capacity: int = 4096,
               threshold: float = 0.0, max_spikes: int = 64) -> None:
        """As Solver.record, for probes given as (instance, element) pairs."""
        pr = np.asarray(probes, dtype=np.int32).reshape(-1, 2)
        self._record(self.lib.nrt_batch_record, pr[:, 0], pr[:, 1], origin, interval, capacity,
                     threshold, max_spikes)

    def recording(self) -> Recording:
        return self._read(self.lib.nrt_batch_record_read)

    def stream(self) -> int:
        v = ctypes.c_void_p()
        check(self.lib.nrt_batch_get_stream(self.h, ctypes.byref(v)), "nrt_batch_get_stream")
        return int(v.value or 0)

    def snapshot(self, i: int) -> np.ndarray:
        out = np.empty(self.problems[i].num_elem)
        check(self.lib.nrt_batch_snapshot(self.h, i, _p(out, ctypes.c_double)), "nrt_batch_snapshot")
        return out

    def snapshot_all(self) -> list:
        """Latest potential of every instance, from one device-to-host copy."""
        sizes = [p.num_elem for p in self.problems]
        out = np.empty(sum(sizes))
        check(self.lib.nrt_batch_snapshot_all(self.h, _p(out, ctypes.c_double)),
              "nrt_batch_snapshot_all")
        return np.split(out, np.cumsum(sizes)[:-1])

    def remaining(self) -> np.ndarray:
        out = np.zeros(self.count, np.int64)
        check(self.lib.nrt_batch_remaining(self.h, _p(out, ctypes.c_int64)), "nrt_batch_remaining")
        return out

    def stats(self) -> _lib.Stats:
        st = _lib.Stats()
        check(self.lib.nrt_batch_get_stats(self.h, ctypes.byref(st)), "nrt_batch_get_stats")
        return st

    def instance_stats(self) -> dict:
        """Per-instance Krylov statistics (implicit): iters, last_iters, nonconverged,
        last_residual."""
        it = np.zeros(self.count, np.int64)
        li = np.zeros(self.count, np.int32)
        nc = np.zeros(self.count, np.int32)
        lr = np.zeros(self.count)
        check(self.lib.nrt_batch_instance_stats(self.h, _p(it, ctypes.c_int64),
                                                _p(li, ctypes.c_int32), _p(nc, ctypes.c_int32),
                                                _p(lr, ctypes.c_double)), "nrt_batch_instance_stats")
        return dict(iters=it, last_iters=li, nonconverged=nc, last_residual=lr)

    def pass_counts(self) -> dict:
        """Per-instance counts of the implicit kernel's passes over the rows (GMRES):
        residuals, applies, xupdates, basis, and Richardson refinement steps (richardson)."""
        out = {k: np.zeros(self.count, np.int64) for k in ("residuals", "applies", "xupdates",
                                                          "basis", "richardson")}
        check(self.lib.nrt_batch_pass_counts(self.h, *[_p(out[k], ctypes.c_int64) for k in out]),
              "nrt_batch_pass_counts")
        return out

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.nrt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop (nrt_server_*): requests are admitted by device
    memory budget, packed per admission into resident batches that advance concurrently,
    and returned as each finishes."""

    def __init__(self, budget_bytes: int, chunk_steps: int = 64, max_batch: int = 4096,
                 max_wait_us: int = 200, explicit_opts: dict | None = None,
                 implicit_opts: dict | None = None):
        self.lib = _lib.load()
        cfg = _lib.ServerConfig(int(budget_bytes), int(chunk_steps), int(max_batch),
                                int(max_wait_us))
        self.ex = make_options(_lib.NRT_EXPLICIT, **(explicit_opts or {}))
        self.im = make_options(_lib.NRT_IMPLICIT_BE, **(implicit_opts or {}))
        h = ctypes.c_void_p()
        check(self.lib.nrt_server_create(ctypes.byref(cfg), ctypes.byref(self.ex),
                                         ctypes.byref(self.im), ctypes.byref(h)),
              "nrt_server_create")
        self.h = h
        self.sizes = {}
        self.rec_shape = {}

    def submit(self, problem: ProblemArrays, implicit: bool, i_begin: int, i_end: int,
               init_time: float, end_input: float, probes=None, interval: int = 0,
               origin: int = 1, capacity: int = 4096, threshold: float = 0.0,
               max_spikes: int = 64) -> int:
        """Queues a request; with `probes` (elements of this tree) its samples and spike
        times are recorded on the device (nrt_server_submit_recorded)."""
        run = _lib.InstanceRun(int(i_begin), int(i_end), float(init_time), float(end_input))
        rid = ctypes.c_int64(0)
        if probes is None:
            check(self.lib.nrt_server_submit(self.h, ctypes.byref(problem.struct),
                                             int(bool(implicit)), ctypes.byref(run),
                                             ctypes.byref(rid)), "nrt_server_submit")
        else:
            el = np.ascontiguousarray(probes, dtype=np.int32)
            cfg = _lib.RecordConfig()
            cfg.num_probes = len(el)
            cfg.element = _p(el, ctypes.c_int32)
            cfg.origin, cfg.interval, cfg.capacity = int(origin), int(interval), int(capacity)
            cfg.threshold, cfg.max_spikes = float(threshold), int(max_spikes)
            check(self.lib.nrt_server_submit_recorded(self.h, ctypes.byref(problem.struct),
                                                      int(bool(implicit)), ctypes.byref(run),
                                                      ctypes.byref(cfg), ctypes.byref(rid)),
                  "nrt_server_submit_recorded")
            self.rec_shape[rid.value] = (len(el), int(capacity), int(max_spikes))
        self.sizes[rid.value] = problem.num_elem
        return rid.value

    def recording(self, rid: int):
        """The recording of a finished request (before result()), or None while it runs."""
        P, cap, ms = self.rec_shape[rid]
        ns = np.zeros(P, np.int64)
        nk = np.zeros(P, np.int32)
        t = np.zeros((P, max(cap, 1)))
        v = np.zeros((P, max(cap, 1)))
        sp = np.zeros((P, max(ms, 1)))
        rc = self.lib.nrt_server_recording(self.h, int(rid), _p(ns, ctypes.c_int64),
                                           _p(t, ctypes.c_double), _p(v, ctypes.c_double),
                                           _p(nk, ctypes.c_int32), _p(sp, ctypes.c_double))
        if rc == _lib.NRT_ENOTREADY:
            return None
        check(rc, "nrt_server_recording")
        kept, ks = np.minimum(ns, cap), np.minimum(nk, ms)
        return Recording([t[p, :kept[p]].copy() for p in range(P)],
                         [v[p, :kept[p]].copy() for p in range(P)], ns,
                         [sp[p, :ks[p]].copy() for p in range(P)], nk)

    def result(self, rid: int):
        """Final potential of a finished request, or None while it runs."""
        out = np.empty(self.sizes[rid])
        rc = self.lib.nrt_server_result(self.h, int(rid), _p(out, ctypes.c_double))
        if rc == _lib.NRT_ENOTREADY:
            return None
        check(rc, "nrt_server_result")
        del self.sizes[rid]
        return out

    def drain(self) -> None:
        check(self.lib.nrt_server_drain(self.h), "nrt_server_drain")

    def stats(self) -> _lib.ServerStats:
        st = _lib.ServerStats()
        check(self.lib.nrt_server_get_stats(self.h, ctypes.byref(st)), "nrt_server_get_stats")
        return st

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.nrt_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simulate(spec, mode: str = "explicit", steps: int | None = None, **opts):
    """Runs the reference driver loop (src/neurite.cpp:171-236) for a spec; returns
    (final V, solver).  steps limits the loop to i in [1, 1 + steps)."""
    d = derive(spec)
    dT = step_size(spec, d)
    prob = ProblemArrays.from_spec(spec, d, dT)
    cls = SolverEx if mode == "explicit" else SolverIm
    s = cls(prob, **opts)
    ns = spec.num_steps(dT)
    i_end = ns - 1 if steps is None else min(ns - 1, 1 + steps)
    s.run(1, i_end, spec.init_time, spec.end_input)
    return s.snapshot(), s
