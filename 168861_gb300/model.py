"""Tree descriptions ("specs") in the reference's element numbering.

A spec holds, per element, what the reference's geometry builders put into
`Cable` / `Hodgkin_Huxley` objects before the parameter pipeline runs
(src/space.cpp, e.g. without_branching_CT_HH at src/space.cpp:650-798):
kind, mother, DR, DL, branching flag, unstrained dX and diameter, strain, injected
current and the material constants, plus the run's time window.

Numbering convention (src/space.cpp:106,135; src/init.cpp:309):
  * element 0 is a fictitious sealed root (mother -1, DR 1) and terminals[0] == 0;
  * elements are numbered depth-first along the right child, so DR == j + 1 inside a
    branch and a branch point's DL is the first element of its left sub-branch
    (a later index);
  * a terminal has DR == itself and is a ghost that copies its mother (explicit) or is
    an identity row (implicit); the last element is a terminal;
  * the stimulus is a point current on element 1.

Every builder here emits that convention; `validate()` checks it.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# Reference defaults, src/discretization.cpp:19-39 and :78-97 (SI units).
DEFAULT_DIAMETER = 3e-6
DEFAULT_THICKNESS = 4e-9
DEFAULT_RO_A = 1.87
DEFAULT_RO_M = 2.5e9
DEFAULT_PER_M = 4e-11
DEFAULT_REST = -0.0655
SIGMA_NA = 4.8e-6
SIGMA_K = 1.44e-6
SIGMA_L = 1.2e-8

KIND_CABLE = 0
KIND_HH = 1

ISPEC_ROWS = ("kind", "mother", "dr", "dl", "branching")
DSPEC_ROWS = ("dX", "diameter", "epsilon", "input_current", "ro_a", "ro_m", "per_m",
              "thickness", "rest_pot", "sigma_Na", "sigma_K", "sigma_L")


@dataclasses.dataclass
class TreeSpec:
    kind: np.ndarray
    mother: np.ndarray
    dr: np.ndarray
    dl: np.ndarray
    branching: np.ndarray
    dX: np.ndarray
    diameter: np.ndarray
    epsilon: np.ndarray
    input_current: np.ndarray
    ro_a: np.ndarray
    ro_m: np.ndarray
    per_m: np.ndarray
    thickness: np.ndarray
    rest_pot: np.ndarray
    sigma_Na: np.ndarray
    sigma_K: np.ndarray
    sigma_L: np.ndarray
    terminals: np.ndarray
    myelin: bool = False          # cable_init_constants flag (src/init.cpp:180-198)
    e_max: float = 1.0            # maximum microscopic strain (src/neurite.cpp:136)
    dt_abs: float = 0.0           # absolute dT in s; 0 -> dtf * critical dT
    dtf: float = 1.0
    tspan: float = 0.0            # simulated time in s
    init_time: float = 0.0        # stimulus window [init_time, end_input] in s
    end_input: float = 0.0
    name: str = ""

    @property
    def n(self) -> int:
        return int(self.kind.shape[0])

    def ispec(self) -> np.ndarray:
        return np.ascontiguousarray(np.stack([getattr(self, r).astype(np.int32) for r in ISPEC_ROWS]))

    def dspec(self) -> np.ndarray:
        return np.ascontiguousarray(np.stack([getattr(self, r).astype(np.float64) for r in DSPEC_ROWS]))

    _SCALARS = ("myelin", "e_max", "dt_abs", "dtf", "tspan", "init_time", "end_input")

    def to_arrays(self, prefix: str = "spec_") -> dict:
        d = {prefix + "ispec": self.ispec(), prefix + "dspec": self.dspec(),
             prefix + "terminals": self.terminals.astype(np.int32),
             prefix + "scalars": np.array([float(getattr(self, k)) for k in self._SCALARS]),
             prefix + "name": np.array(self.name)}
        return d

    @classmethod
    def from_arrays(cls, d, prefix: str = "spec_") -> "TreeSpec":
        isp, dsp = d[prefix + "ispec"], d[prefix + "dspec"]
        kw = {r: isp[k].astype(np.int32).copy() for k, r in enumerate(ISPEC_ROWS)}
        kw.update({r: dsp[k].astype(np.float64).copy() for k, r in enumerate(DSPEC_ROWS)})
        s = cls(terminals=np.asarray(d[prefix + "terminals"], np.int32).copy(), **kw)
        for k, v in zip(cls._SCALARS, d[prefix + "scalars"]):
            setattr(s, k, bool(v) if k == "myelin" else float(v))
        s.name = str(d[prefix + "name"]) if prefix + "name" in d else ""
        return s

    def num_steps(self, dT: float) -> int:
        """numStepsT = int(tspan / dT), src/neurite.cpp:176-177."""
        return int(self.tspan / dT)

    def validate(self) -> None:
        """Checks the reference numbering convention (raises ValueError)."""
        n = self.n
        if n < 4:
            raise ValueError("a tree needs at least 4 elements")
        m, dr, dl, br = self.mother, self.dr, self.dl, self.branching
        if m[0] != -1 or dr[0] != 1:
            raise ValueError("element 0 must be the fictitious root (mother -1, DR 1)")
        t = np.asarray(self.terminals)
        if t[0] != 0 or t[-1] != n - 1:
            raise ValueError("terminals[0] must be 0 and the last element a terminal")
        if np.any(m[1:] < 0) or np.any(m[1:] >= np.arange(1, n)):
            raise ValueError("every mother must precede its child")
        term = np.zeros(n, bool)
        term[t[1:]] = True
        if np.any(dr[term] != np.nonzero(term)[0]):
            raise ValueError("terminals must have DR == themselves")
        nt = np.nonzero(~term)[0][1:]
        if np.any(dr[nt] != nt + 1):
            raise ValueError("non-terminal elements must have DR == j + 1")
        if np.any(m[nt + 1] != nt):
            raise ValueError("the right child's mother must be the element")
        b = np.nonzero(br)[0]
        if np.any(dl[b] <= b) or np.any(m[dl[b]] != b):
            raise ValueError("a branch point's DL must be a later element whose mother it is")
        if np.any(dl[~br.astype(bool)] != 0):
            raise ValueError("DL must be 0 off branch points")
        if np.any(term[1:3]) or br[1]:
            raise ValueError("the root branch needs at least two compartments")


def _blank(n: int) -> dict:
    return dict(
        kind=np.zeros(n, np.int32), mother=np.zeros(n, np.int32), dr=np.zeros(n, np.int32),
        dl=np.zeros(n, np.int32), branching=np.zeros(n, np.int32),
        dX=np.zeros(n), diameter=np.full(n, DEFAULT_DIAMETER), epsilon=np.zeros(n),
        input_current=np.zeros(n), ro_a=np.full(n, DEFAULT_RO_A), ro_m=np.full(n, DEFAULT_RO_M),
        per_m=np.full(n, DEFAULT_PER_M), thickness=np.full(n, DEFAULT_THICKNESS),
        rest_pot=np.full(n, DEFAULT_REST), sigma_Na=np.full(n, SIGMA_NA),
        sigma_K=np.full(n, SIGMA_K), sigma_L=np.full(n, SIGMA_L))


def _from_segments(segs, root_dx, root_diam, **mat) -> TreeSpec:
    """Lays out segments in reference order.

    segs: list of dicts in depth-first, right-first order, each with keys
      'parent' (index into segs or -1), 'side' ('R'/'L'), 'ncomp', 'dx', 'diam', 'kind'
      (array-like or scalar), and optional per-compartment arrays 'epsilon', 'sigma_scale',
      'per_m', 'ro_m'.  Leaves get one ghost terminal element appended.
    """
    children = {i: [] for i in range(len(segs))}
    for i, s in enumerate(segs):
        if s["parent"] >= 0:
            children[s["parent"]].append(i)
    n = 1 + sum(s["ncomp"] + (0 if children[i] else 1) for i, s in enumerate(segs))
    a = _blank(n)
    for k, v in mat.items():
        a[k][:] = v
    a["mother"][0] = -1
    a["dr"][0] = 1
    a["dX"][0] = root_dx
    a["diameter"][0] = root_diam
    first = {}
    last = {}
    pos = 1
    terminals = [0]
    order = []

    def emit(si):
        nonlocal pos
        s = segs[si]
        nc = s["ncomp"]
        idx = np.arange(pos, pos + nc)
        first[si] = pos
        for key in ("dx", "diam"):
            pass
        a["dX"][idx] = s["dx"]
        a["diameter"][idx] = s["diam"]
        a["kind"][idx] = s.get("kind", KIND_HH)
        for key in ("epsilon", "per_m", "ro_m", "input_current"):
            if key in s:
                a[key][idx] = s[key]
        if "sigma_scale" in s:
            sc = np.asarray(s["sigma_scale"], float)
            a["sigma_Na"][idx] = SIGMA_NA * sc
            a["sigma_K"][idx] = SIGMA_K * sc
            a["sigma_L"][idx] = SIGMA_L * sc
        a["mother"][idx[1:]] = idx[:-1]
        a["dr"][idx] = idx + 1
        pos += nc
        last[si] = pos - 1
        order.append(si)
        ch = children[si]
        if not ch:
            g = pos  # ghost terminal copying its mother
            a["mother"][g] = g - 1
            a["dr"][g] = g
            a["dX"][g] = s["dx"]
            a["diameter"][g] = s["diam"]
            a["kind"][g] = KIND_CABLE
            terminals.append(g)
            pos += 1
            return
        right = [c for c in ch if segs[c]["side"] == "R"]
        left = [c for c in ch if segs[c]["side"] == "L"]
        for c in right:
            a["mother"][pos] = last[si]
            emit(c)
        for c in left:
            bp = last[si]
            a["branching"][bp] = 1
            a["dl"][bp] = pos
            a["mother"][pos] = bp
            emit(c)

    a["mother"][1] = 0
    emit(0)
    assert pos == n
    spec = TreeSpec(terminals=np.asarray(terminals, np.int32), **a)
    return spec


def straight_axon(n_comp: int = 1000, length: float = 1e-2, diameter: float = 2e-6,
                  ro_a: float = 1.0, rest: float = -0.065, i_amp: float = 1e-9,
                  pulse: float = 0.5e-3, dt: float = 1e-6, tspan: float = 10e-3,
                  dtf: float = 0.0) -> TreeSpec:
    """Unmyelinated squid-HH axon: n_comp HH compartments between two fictitious ends.

    Defaults are the 1 cm, 2 um axon at dx = 10 um with a 1 nA, 0.5 ms pulse at x = 0.
    With dtf > 0 the step is dtf * critical dT instead of `dt`.
    """
    dx = length / n_comp
    seg = dict(parent=-1, side="R", ncomp=n_comp, dx=dx, diam=diameter, kind=KIND_HH)
    s = _from_segments([seg], dx, diameter, ro_a=ro_a, rest_pot=rest)
    s.input_current[1] = i_amp
    s.myelin = True   # the reference applies its myelin model to cables whenever HH is on
    s.dt_abs = 0.0 if dtf > 0 else dt
    s.dtf = dtf if dtf > 0 else 1.0
    s.tspan = tspan
    s.init_time = 0.0
    s.end_input = pulse
    s.name = f"straight_axon_{n_comp}"
    s.validate()
    return s


def random_binary_tree(depth: int = 10, seed: int = 2, len_lo: float = 50e-6,
                       len_hi: float = 200e-6, root_diam: float = 4e-6, dx: float = 1e-6,
                       ro_a: float = 1.0, rest: float = -0.065, i_amp: float = 2e-9,
                       dt: float = 1e-5, tspan: float = 20e-3) -> TreeSpec:
    """Full binary tree of 2**(depth+1)-1 branches, HH everywhere, Rall 3/2 taper.

    Branch lengths ~ U(len_lo, len_hi); equal daughters get d * 2**(-2/3).  A step
    current of i_amp is applied at element 1 for the whole run.
    """
    rng = np.random.default_rng(seed)
    segs = []

    def add(parent, side, level, diam):
        L = rng.uniform(len_lo, len_hi)
        nc = max(2, int(round(L / dx)))
        si = len(segs)
        segs.append(dict(parent=parent, side=side, ncomp=nc, dx=dx, diam=diam, kind=KIND_HH))
        if level < depth:
            cd = diam * 2.0 ** (-2.0 / 3.0)
            add(si, "R", level + 1, cd)
            add(si, "L", level + 1, cd)

    add(-1, "R", 0, root_diam)
    s = _from_segments(segs, dx, root_diam, ro_a=ro_a, rest_pot=rest)
    s.input_current[1] = i_amp
    s.myelin = True
    s.dt_abs = dt
    s.tspan = tspan
    s.init_time = 0.0
    s.end_input = tspan
    s.name = f"binary_tree_d{depth}_s{seed}"
    s.validate()
    return s


def random_tree(seed: int, n_target: int, depth_lo: int = 4, depth_hi: int = 12,
                p_lo: float = 0.6, p_hi: float = 0.9, dx: float = 1e-6, root_diam: float = 4e-6,
                ro_a: float = 1.0, rest: float = -0.065, i_amp: float | None = None,
                strain: float | None = None, dt: float = 2.5e-5, tspan: float = 50e-3) -> TreeSpec:
    """Seeded random dendritic tree of about n_target elements, HH everywhere.

    Depth ~ U{depth_lo..depth_hi}; each branch splits with probability
    p ~ U(p_lo, p_hi) until the depth limit; branch lengths are scaled so the total
    is close to n_target compartments.  Stimulus ~ U(0.5, 3) nA and static strain
    ~ U(0, 0.15) unless given.
    """
    rng = np.random.default_rng(seed)
    depth = int(rng.integers(depth_lo, depth_hi + 1))
    p = rng.uniform(p_lo, p_hi)
    shape = []

    def grow(parent, side, level):
        si = len(shape)
        shape.append([parent, side, level, rng.uniform(0.5, 1.5)])
        if level < depth and (level == 0 or rng.random() < p):
            grow(si, "R", level + 1)
            grow(si, "L", level + 1)

    grow(-1, "R", 0)
    w = np.array([x[3] for x in shape])
    nseg = len(shape)
    nleaf = sum(1 for i in range(nseg) if not any(x[0] == i for x in shape))
    budget = max(n_target - 1 - nleaf, 2 * nseg)
    ncomp = np.maximum(2, np.round(w / w.sum() * budget)).astype(int)
    segs = []
    for i, (parent, side, level, _) in enumerate(shape):
        segs.append(dict(parent=parent, side=side, ncomp=int(ncomp[i]), dx=dx,
                         diam=root_diam * 2.0 ** (-2.0 * level / 3.0), kind=KIND_HH))
    s = _from_segments(segs, dx, root_diam, ro_a=ro_a, rest_pot=rest)
    amp = rng.uniform(0.5e-9, 3e-9) if i_amp is None else i_amp
    eps = rng.uniform(0.0, 0.15) if strain is None else strain
    s.input_current[1] = amp
    s.epsilon[:] = eps
    s.myelin = True
    s.dt_abs = dt
    s.tspan = tspan
    s.init_time = 0.0
    s.end_input = tspan
    s.name = f"random_tree_s{seed}"
    s.validate()
    return s


def myelinated_axon(n_nodes: int = 200, node_len: float = 1e-6, internode_len: float = 1e-3,
                    dx: float = 1e-6, diameter: float = 2e-6, node_density: float = 10.0,
                    internode_cm: float = 0.005e-2, internode_rm_scale: float = 1000.0,
                    ro_a: float = 1.0, rest: float = -0.065, i_amp: float = 1e-9,
                    pulse: float = 0.5e-3, strain: np.ndarray | float = 0.0, dtf: float = 0.8,
                    tspan: float = 10e-3) -> TreeSpec:
    """Myelinated axon: n_nodes HH nodes of Ranvier separated by passive internodes.

    Internodes carry Cm = internode_cm F/m^2 and Rm = internode_rm_scale * (ro_m * th) of
    the reference membrane, given directly (no 45-layer myelin model); nodes carry HH
    at node_density times the squid channel densities.  `strain` is a scalar or a
    per-element static strain.
    """
    th = DEFAULT_THICKNESS
    n_node_c = max(1, int(round(node_len / dx)))
    n_int_c = max(1, int(round(internode_len / dx)))
    kinds = []
    for k in range(n_nodes):
        kinds += [KIND_HH] * n_node_c
        if k < n_nodes - 1:
            kinds += [KIND_CABLE] * n_int_c
    kinds = np.asarray(kinds, np.int32)
    nc = len(kinds)
    per_m = np.where(kinds == KIND_HH, DEFAULT_PER_M, internode_cm * th)
    ro_m = np.where(kinds == KIND_HH, DEFAULT_RO_M, DEFAULT_RO_M * internode_rm_scale)
    scale = np.where(kinds == KIND_HH, node_density, 1.0)
    seg = dict(parent=-1, side="R", ncomp=nc, dx=dx, diam=diameter, kind=kinds, per_m=per_m,
               ro_m=ro_m, sigma_scale=scale)
    s = _from_segments([seg], dx, diameter, ro_a=ro_a, rest_pot=rest)
    s.per_m[0] = s.per_m[1]
    s.per_m[-1] = s.per_m[-2]
    s.epsilon[:] = strain
    s.input_current[1] = i_amp
    s.myelin = False
    s.dt_abs = 0.0
    s.dtf = dtf
    s.tspan = tspan
    s.init_time = 0.0
    s.end_input = pulse
    s.name = f"myelinated_axon_{n_nodes}"
    s.validate()
    return s


def from_neurite_txt(text: str, hh: bool = True, i_amp: float = 0.8e-9, ro_a: float = 1.0,
                     rest: float = -0.065, dt: float = 1e-6, tspan: float = 5e-3) -> TreeSpec:
    """Reads the reference's segmented-neuron format (src/space.cpp:37-183).

    Columns per row: me mother dR branching dL diameter_um length_um (src/space.cpp:69).
    Row k becomes element k (the reference's refining == 1 case); element 0 is the
    fictitious root built from row 1's geometry; a row with me == dR is a terminal.
    """
    rows = [r.split() for r in text.strip().splitlines() if r.strip()]
    me = np.array([int(r[0]) for r in rows])
    mom = np.array([int(r[1]) for r in rows])
    dR = np.array([int(r[2]) for r in rows])
    br = np.array([int(r[3]) for r in rows])
    dL = np.array([int(r[4]) for r in rows])
    diam = np.array([float(r[5]) for r in rows]) * 1e-6
    length = np.array([float(r[6]) for r in rows]) * 1e-6
    n = len(rows) + 1
    a = _blank(n)
    a["ro_a"][:] = ro_a
    a["rest_pot"][:] = rest
    a["mother"][0] = -1
    a["dr"][0] = 1
    a["dX"][0] = length[0]
    a["diameter"][0] = diam[0]
    a["kind"][0] = KIND_CABLE
    a["mother"][me] = mom
    a["dr"][me] = dR
    a["branching"][me] = br
    a["dl"][me] = np.where(br != 0, dL, 0)
    a["dX"][me] = length
    a["diameter"][me] = diam
    a["kind"][me] = KIND_HH if hh else KIND_CABLE
    term = [0] + [int(x) for x in me[me == dR]]
    a["kind"][np.asarray(term[1:], int)] = KIND_CABLE
    s = TreeSpec(terminals=np.asarray(term, np.int32), **a)
    s.input_current[1] = i_amp
    s.myelin = True
    s.dt_abs = dt
    s.tspan = tspan
    s.init_time = 0.0
    s.end_input = 3e-3
    s.name = "neurite_txt"
    return s


def log_uniform_sizes(count: int, lo: float, hi: float, seed: int) -> np.ndarray:
    """Per-instance compartment targets, log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size=count)).astype(int)
