"""Regenerates the golden fixtures in this folder from the reference's own CPU code.

Run in a container where the reference tree exists (default /root/reference):

    python tests/golden/make_golden.py [--ref /root/reference]

It builds oracle/_ref/ref_harness (src/solverEx-cpu.cpp & co. compiled unmodified, see
oracle/Makefile and oracle/ref_harness.cpp) and oracle/_ref/ref_harness_im (plus
src/solverIm-cpu.cpp with the RCI shim), runs them on each case below and stores, per
case, the tree description and the reference outputs: derived parameters, critical and
chosen dT, a probe trace, the final potential and gates, and the reference's measurement
point (src/init.cpp:339-358) for a few distances along the tree.  loader_example8.npz holds
what the reference's own loader (src/space.cpp:37-183) builds from its example-8 neuron file.
The GPU tests and the oracle tests read only these .npz files, so nothing at test time needs
the reference tree.
"""
from __future__ import annotations

import argparse
import importlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

model = importlib.import_module("168861_gb300.model")
import oracle as O  # noqa: E402


def cases(ref_dir: str):
    """(name, spec, mode, record_every, probes, max_loop_index or None)."""
    out = []
    s = model.straight_axon(dtf=0.8)
    out.append(("axon1000_dtf08", s, "e", 50, [1, 250, 500, 750, 1000], None))
    s = model.straight_axon()  # dt = 1e-3 ms exactly, at the critical step: unstable
    out.append(("axon1000_dt1e-3", s, "e", 50, [1, 250, 500, 750, 1000], None))
    s = model.random_binary_tree(depth=3, seed=7, len_lo=20e-6, len_hi=60e-6, dx=4e-6,
                                 root_diam=3e-6, dt=0.0, tspan=4e-3)
    s.dt_abs, s.dtf = 0.0, 0.8
    s.epsilon[:] = 0.08
    s.e_max = 0.1
    out.append(("ytree_d3_strain", s, "e", 400, [1, s.n // 3, s.n // 2, s.n - 2], 20000))
    s = model.myelinated_axon(n_nodes=8, internode_len=60e-6, dx=2e-6, node_len=2e-6,
                              tspan=1.0e-3, dtf=0.8)
    out.append(("myelin8", s, "e", 200, [1, s.n // 2, s.n - 2], 20000))
    s = model.random_tree(seed=11, n_target=1500, depth_lo=4, depth_hi=6, dt=0.0, tspan=2e-3,
                          strain=0.05)
    s.dt_abs, s.dtf = 0.0, 0.7
    out.append(("rtree1500", s, "e", 400, [1, s.n // 2, s.n - 2], 20000))
    path = os.path.join(ref_dir, "applications", "example_8", "neuron_for_neurite.txt")
    with open(path) as f:
        s = model.from_neurite_txt(f.read(), hh=False, tspan=2e-3)
    s.myelin = False
    s.dt_abs, s.dtf = 0.0, 0.8
    s.name = "example8_passive"
    out.append(("example8_passive", s, "e", 400, [1, 100, 400, 877], 20000))
    # implicit (backward Euler): reference createMatrix + its FGMRES driver over the shim
    s = model.straight_axon(n_comp=300, length=3e-3, tspan=2e-3, dt=2.5e-5)
    out.append(("im_axon300", s, "i", 4, [1, 100, 200, 300], None))
    s = model.random_binary_tree(depth=3, seed=3, len_lo=20e-6, len_hi=60e-6, dx=4e-6,
                                 root_diam=3e-6, dt=2e-5, tspan=2e-3)
    out.append(("im_ytree_d3", s, "i", 5, [1, s.n // 2, s.n - 2], None))
    return out


def loader_golden(ref_dir: str) -> None:
    """loader_example8.npz: the reference's own loader (src/space.cpp:37-183, through the
    harness's mode L) on applications/example_8/neuron_for_neurite.txt.  Stores the file's
    seven columns as numbers (the input) and the elements the reference built from them."""
    import shutil
    import subprocess
    src = os.path.join(ref_dir, "applications", "example_8", "neuron_for_neurite.txt")
    text = open(src).read()
    rows = [r.split() for r in text.strip().splitlines() if r.strip()]
    ints = np.array([[int(x) for x in r[:5]] for r in rows], np.int32)
    flts = np.array([[float(x) for x in r[5:7]] for r in rows], np.float64)
    with tempfile.TemporaryDirectory() as td:
        shutil.copy(src, os.path.join(td, "neuron_for_neurite.txt"))
        out = os.path.join(td, "elements.txt")
        subprocess.run([O.REF_BIN, td, out, "L"], check=True, capture_output=True)
        lines = open(out).read().splitlines()
    n, nterm = (int(x) for x in lines[0].split())
    terms = np.array([int(x) for x in lines[1].split()], np.int32)
    el = [ln.split() for ln in lines[2:2 + n]]
    np.savez_compressed(
        os.path.join(HERE, "loader_example8.npz"),
        rows_int=ints, rows_float=flts, num_terminals=np.array(nterm), terminals=terms,
        mother=np.array([int(e[0]) for e in el], np.int32),
        dr=np.array([int(e[1]) for e in el], np.int32),
        dl=np.array([int(e[2]) for e in el], np.int32),
        branching=np.array([int(e[3]) for e in el], np.int32),
        dX=np.array([float(e[4]) for e in el]), diameter=np.array([float(e[5]) for e in el]),
        input_current=np.array([float(e[6]) for e in el]))
    print(f"loader_example8: n={n} terminals={nterm}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("NEURITE_REFERENCE", "/root/reference"))
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    O.build(ref_dir=args.ref, with_ref=True)
    if args.only in ("", "loader_example8"):
        loader_golden(args.ref)
    for name, spec, mode, rec, probes, cap in cases(args.ref):
        if args.only and args.only != name:
            continue
        if cap is not None:
            d = O.Oracle().derive(spec)
            dT = O.spec_dT(spec, d.dT_crit)
            spec.tspan = min(spec.tspan, (cap + 2) * dT)
        with tempfile.TemporaryDirectory() as td:
            out = O.run_reference(spec, td, mode, rec, probes)
        arrays = spec.to_arrays()
        arrays.update({
            "mode": np.array(mode), "record_every": np.array(rec),
            "probes": np.asarray(probes, np.int32), "dT_crit": np.array(out["dT_crit"]),
            "dT": np.array(out["dT"]), "numStepsT": np.array(out["numStepsT"]),
            "eparam": out["eparam"], "hh_elem": out["hh_elem"], "hparam": out["hparam"],
            "trace": out["trace"], "final_V": out["final_V"], "final_gates": out["final_gates"],
            "mp_dist": out["mp_dist"], "mp_index": out["mp_index"],
        })
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        fin = out["final_V"]
        print(f"{name}: n={spec.n} steps={out['numStepsT']} dT={out['dT']:.4g} "
              f"Vmax(trace)={np.nanmax(out['trace'][:, 1:]) * 1e3:.3f} mV "
              f"finite={np.isfinite(fin).all()}")


if __name__ == "__main__":
    main()
