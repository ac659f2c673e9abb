"""Python access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

* `Oracle` wraps oracle/_build/libneurite_oracle.so (the C restatement, neurite_oracle.c).
* `write_spec` / `run_reference` / `read_reference_output` drive oracle/_ref/ref_harness,
  the reference's own CPU code compiled from source, to make golden fixtures.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libneurite_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")
REF_BIN_IM = os.path.join(HERE, "_ref", "ref_harness_im")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

EPARAM_ROWS = ("c_m", "r_a", "dX", "W", "K", "crit")
HPARAM_ROWS = ("m", "h", "n", "g_Na", "g_K", "G_L", "E_Na", "E_K", "E_L", "LS_Na", "LS_K", "rest")


def build(ref_dir: str | None = None, with_ref: bool = False) -> None:
    """Builds the C restatement (and, if asked and present, the reference harness)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if with_ref:
        env = dict(os.environ)
        args = ["make", "-s", "-C", HERE, "ref", "ref_im"]
        if ref_dir:
            args.append(f"REF={ref_dir}")
        subprocess.run(args, check=True, env=env)


class Derived:
    """Parameters after the reference's pipeline: eparam [6][n], hparam [12][num_hh]."""

    def __init__(self, eparam, hh_elem, hparam, dT_crit):
        self.eparam = eparam
        self.hh_elem = hh_elem
        self.hparam = hparam
        self.dT_crit = dT_crit

    @property
    def num_hh(self):
        return int(self.hh_elem.shape[0])

    def copy(self):
        return Derived(self.eparam.copy(), self.hh_elem.copy(), self.hparam.copy(), self.dT_crit)


class Oracle:
    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        c_int, c_double = ctypes.c_int, ctypes.c_double
        lib.nro_derive.argtypes = [c_int, _i32p, _f64p, c_int, c_double, _f64p, _i32p, _f64p,
                                   ctypes.POINTER(c_int), ctypes.POINTER(c_double)]
        lib.nro_explicit_run.argtypes = [c_int, _i32p, _f64p, _f64p, c_int, _i32p, c_int, _i32p,
                                         _f64p, c_double, c_int, c_int, c_double, c_double, _f64p,
                                         c_int, c_int, _i32p, _f64p, ctypes.POINTER(c_int)]
        lib.nro_implicit_run.argtypes = [c_int, _i32p, _f64p, _f64p, c_int, _i32p, _f64p, c_double,
                                         c_int, c_int, c_double, c_double, _f64p, _f64p, c_int,
                                         c_int, c_int, _i32p, _f64p, ctypes.POINTER(c_int),
                                         ctypes.POINTER(ctypes.c_longlong), c_int]
        lib.nro_implicit_matrix.argtypes = [c_int, _i32p, _f64p, _f64p, _f64p, _f64p, c_double,
                                            _f64p, _i32p, _i32p, _f64p, _f64p, ctypes.POINTER(c_int)]
        lib.nro_tree_solve.argtypes = [c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        lib.nro_gmres.argtypes = [c_int, _i32p, _i32p, _f64p, _f64p, _f64p, c_int, c_double, c_int,
                                  ctypes.POINTER(c_int)]
        self.lib = lib

    def derive(self, spec) -> Derived:
        n = spec.n
        num_hh = int(np.count_nonzero(spec.kind == 1))
        eparam = np.zeros((6, n))
        hh_elem = np.zeros(max(num_hh, 1), np.int32)
        hparam = np.zeros((12, max(num_hh, 1)))
        nh = ctypes.c_int(0)
        crit = ctypes.c_double(0)
        rc = self.lib.nro_derive(n, spec.ispec(), spec.dspec(), int(spec.myelin), spec.e_max,
                                 eparam, hh_elem, hparam, ctypes.byref(nh), ctypes.byref(crit))
        if rc:
            raise RuntimeError(f"nro_derive failed: {rc}")
        return Derived(eparam, hh_elem[:num_hh].copy(), np.ascontiguousarray(hparam[:, :num_hh]),
                       crit.value)

    def explicit_run(self, spec, d: Derived, dT: float, i_begin: int, i_end: int, V=None,
                     record_every: int = 0, probes=()):
        """Runs steps [i_begin, i_end) in place on (V, d.hparam); returns (V, trace)."""
        n = spec.n
        V = np.ascontiguousarray(spec.rest_pot.copy() if V is None else V, dtype=np.float64)
        probes = np.asarray(probes, np.int32) if len(probes) else np.zeros(1, np.int32)
        nprobe = len(probes) if record_every else 0
        cap = (i_end - i_begin) // record_every + 1 if record_every else 1
        trace = np.zeros((cap, nprobe + 1))
        nrec = ctypes.c_int(0)
        rc = self.lib.nro_explicit_run(
            n, spec.ispec(), d.eparam, np.ascontiguousarray(spec.input_current, dtype=np.float64),
            len(spec.terminals), spec.terminals.astype(np.int32), d.num_hh,
            d.hh_elem if d.num_hh else np.zeros(1, np.int32),
            d.hparam if d.num_hh else np.zeros((12, 1)), dT, i_begin, i_end, spec.init_time,
            spec.end_input, V, record_every, nprobe, probes, trace, ctypes.byref(nrec))
        if rc:
            raise RuntimeError(f"nro_explicit_run failed: {rc}")
        return V, trace[: nrec.value]

    def implicit_run(self, spec, d: Derived, dT: float, i_begin: int, i_end: int, V=None,
                     Vother=None, linsolve: int = 0, record_every: int = 0, probes=(),
                     scheme: int = 0):
        """Implicit steps [i_begin, i_end): backward Euler (scheme 0, the reference's) or
        Crank-Nicolson (scheme 1); returns (V, Vother, trace, krylov_iters)."""
        n = spec.n
        V = np.ascontiguousarray(spec.rest_pot.copy() if V is None else V, dtype=np.float64)
        Vo = np.ascontiguousarray(spec.rest_pot.copy() if Vother is None else Vother, dtype=np.float64)
        probes = np.asarray(probes, np.int32) if len(probes) else np.zeros(1, np.int32)
        nprobe = len(probes) if record_every else 0
        cap = (i_end - i_begin) // record_every + 1 if record_every else 1
        trace = np.zeros((cap, nprobe + 1))
        nrec = ctypes.c_int(0)
        kit = ctypes.c_longlong(0)
        rc = self.lib.nro_implicit_run(
            n, spec.ispec(), d.eparam, np.ascontiguousarray(spec.input_current, dtype=np.float64),
            d.num_hh, d.hh_elem if d.num_hh else np.zeros(1, np.int32),
            d.hparam if d.num_hh else np.zeros((12, 1)), dT, i_begin, i_end, spec.init_time,
            spec.end_input, V, Vo, linsolve, record_every, nprobe, probes, trace,
            ctypes.byref(nrec), ctypes.byref(kit), int(scheme))
        if rc:
            raise RuntimeError(f"nro_implicit_run failed: {rc}")
        return V, Vo, trace[: nrec.value], kit.value

    def implicit_matrix(self, spec, d: Derived, W, K, input_, dT, Vprev, rhs_in=None):
        n = spec.n
        cap = 4 * n + 2
        row_ptr = np.zeros(n + 1, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        rhs = np.ascontiguousarray(np.zeros(n) if rhs_in is None else rhs_in, dtype=np.float64).copy()
        nnz = ctypes.c_int(0)
        rc = self.lib.nro_implicit_matrix(n, spec.ispec(), d.eparam, np.ascontiguousarray(W),
                                          np.ascontiguousarray(K), np.ascontiguousarray(input_),
                                          dT, np.ascontiguousarray(Vprev), row_ptr, col, val, rhs,
                                          ctypes.byref(nnz))
        if rc:
            raise RuntimeError(f"nro_implicit_matrix failed: {rc}")
        k = nnz.value
        return row_ptr, col[:k].copy(), val[:k].copy(), rhs

    def tree_solve(self, row_ptr, col, val, b):
        x = np.zeros_like(b)
        rc = self.lib.nro_tree_solve(len(b), row_ptr, col, val, np.ascontiguousarray(b), x)
        if rc:
            raise RuntimeError(f"nro_tree_solve failed: {rc}")
        return x


# ---------------------------------------------------------------- recording

def measurement_point(dX, dist_mes: float) -> int:
    """The reference's measurement point (src/init.cpp:339-358): the first element k at
    which the running sum of dX (after the strain scaling) reaches dist_mes.  Not found,
    or found at element 0, gives int(numStepsX / 2)."""
    temp = 0.0
    point = 0
    for k in range(len(dX)):
        temp = temp + float(dX[k])
        if temp >= dist_mes:
            point = k
            break
    if point == 0:
        point = len(dX) // 2
    return point


def recording(i_first: int, v_before, steps, origin: int, interval: int, thresh: float,
              dT: float):
    """What device-side recording keeps for one probe, from its value before loop index
    i_first and after every step i_first, i_first + 1, ... (`steps`, one per loop index).

    Samples follow the reference driver's counter (src/neurite.cpp:241-248: a snapshot when
    `++GL_cont > interval`, the loop starting at i = origin): loop index i is sampled when
    (i - origin + 1) is a positive multiple of interval + 1.  Spikes are upward crossings
    of `thresh` between consecutive steps, timed by linear interpolation between
    t = (i - 1) dT and i dT.  Returns ({slot: value}, [spike times])."""
    samples, spikes = {}, []
    prev = float(v_before)
    for k, v in enumerate(steps):
        i = i_first + k
        v = float(v)
        if prev < thresh <= v:
            t0, t1 = (i - 1) * dT, i * dT
            spikes.append(t0 + (thresh - prev) * (t1 - t0) / (v - prev))
        q = i - origin + 1
        if q > 0 and q % (interval + 1) == 0:
            samples[q // (interval + 1) - 1] = v
        prev = v
    return samples, spikes


# ---------------------------------------------------------------- reference harness I/O

def spec_dT(spec, dT_crit: float) -> float:
    """dT as src/neurite.cpp:171-173 picks it (or the spec's absolute step)."""
    return spec.dt_abs if spec.dt_abs > 0 else dT_crit * spec.dtf


def write_spec(spec, path: str, record_every: int = 0, probes=()) -> None:
    """Writes the text tree description that oracle/ref_harness.cpp reads."""
    n = spec.n
    with open(path, "w") as f:
        f.write("NEURITE_SPEC 1\n")
        f.write(f"num_elem {n}\n")
        f.write(f"num_term {len(spec.terminals)}\n")
        f.write("terminals " + " ".join(str(int(t)) for t in spec.terminals) + "\n")
        f.write(f"dt_abs {spec.dt_abs!r}\ndtf {spec.dtf!r}\ntspan {spec.tspan!r}\n")
        f.write(f"init_time {spec.init_time!r}\nend_input {spec.end_input!r}\n")
        f.write(f"e_max {spec.e_max!r}\nmyelin {int(spec.myelin)}\n")
        f.write(f"record_every {int(record_every)}\n")
        f.write(f"num_probes {len(probes)}\n")
        f.write("probes " + " ".join(str(int(p)) for p in probes) + "\n")
        f.write("elements\n")
        I = spec.ispec()
        D = spec.dspec()
        for i in range(n):
            f.write(" ".join(str(int(v)) for v in I[:, i]) + " " +
                    " ".join(repr(float(v)) for v in D[:, i]) + "\n")


def read_reference_output(path: str) -> dict:
    with open(path) as f:
        tok = f.read().split()
    pos = 0

    def nxt():
        nonlocal pos
        v = tok[pos]
        pos += 1
        return v

    out = {}
    while pos < len(tok):
        key = nxt()
        if key in ("dT_crit", "dT"):
            out[key] = float(nxt())
        elif key == "numStepsT":
            out[key] = int(nxt())
        elif key == "measurement_points":
            k = int(nxt())
            rows = [(float(nxt()), int(nxt())) for _ in range(k)]
            out["mp_dist"] = np.array([r[0] for r in rows])
            out["mp_index"] = np.array([r[1] for r in rows], np.int32)
        elif key == "elem_params":
            n = int(nxt())
            out["eparam"] = np.array([float(nxt()) for _ in range(6 * n)]).reshape(n, 6).T.copy()
        elif key == "hh_params":
            k = int(nxt())
            rows = np.array([float(nxt()) for _ in range(13 * k)]).reshape(k, 13)
            out["hh_elem"] = rows[:, 0].astype(np.int32)
            out["hparam"] = rows[:, 1:].T.copy()
        elif key == "trace":
            r, p = int(nxt()), int(nxt())
            out["trace"] = np.array([float(nxt()) for _ in range(r * (p + 1))]).reshape(r, p + 1)
        elif key == "final_V":
            n = int(nxt())
            out["final_V"] = np.array([float(nxt()) for _ in range(n)])
        elif key == "final_gates":
            k = int(nxt())
            out["final_gates"] = np.array([float(nxt()) for _ in range(3 * k)]).reshape(k, 3).T.copy()
        else:
            raise ValueError(f"unexpected token {key!r} in {path}")
    return out


def run_reference(spec, workdir: str, mode: str = "e", record_every: int = 0, probes=()) -> dict:
    """Runs the compiled reference (oracle/_ref) on spec; returns the parsed output."""
    os.makedirs(workdir, exist_ok=True)
    sp = os.path.join(workdir, "spec.txt")
    op = os.path.join(workdir, "out.txt")
    write_spec(spec, sp, record_every, probes)
    exe = REF_BIN if mode == "e" else REF_BIN_IM
    subprocess.run([exe, sp, op, mode], check=True, stdout=subprocess.DEVNULL)
    return read_reference_output(op)
