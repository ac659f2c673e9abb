"""The C++ drop-in adapter (include/neurite_gb300_solver.hpp) used the way the reference's
driver uses its solvers (src/neurite.cpp:185-255): `Solver *s = new SolverExGB300(...)`."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

DROPIN = os.path.join(ROOT, "tests", "dropin")
REF_INC = os.path.join(os.environ.get("NEURITE_REFERENCE", "/root/reference"), "inc")


def _compile(lib, out):
    libdir = os.path.dirname(lib._name)
    cmd = ["g++", "-std=gnu++98", "-O2", "-Wall", "-I", DROPIN, "-I", os.path.join(ROOT, "include"),
           os.path.join(DROPIN, "dropin_main.cpp"), "-o", out, "-L", libdir, "-lneurite_gb300",
           f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_adapter_builds_as_cpp98_and_links(lib, tmp_path):
    _compile(lib, str(tmp_path / "dropin"))


@pytest.mark.skipif(not os.path.isdir(REF_INC), reason="reference headers not present")
def test_adapter_compiles_against_reference_headers(tmp_path):
    """The adapter against the reference's own class definitions (inc/*.h), in the
    reference's language level (-std=gnu++98)."""
    src = tmp_path / "tu.cpp"
    src.write_text('#include "configuration.h"\n#include "discretization.h"\n#include "solver.h"\n'
                   '#include "neurite_gb300_solver.hpp"\n'
                   'Solver *make(double dT, double **p, int nt, int *t, int nh, Hodgkin_Huxley **hh,'
                   ' int n, discretization **e, bool im) {\n'
                   '  if (im) return new SolverImGB300(dT, p, nt, t, 0, nh, hh, n, e);\n'
                   '  return new SolverExGB300(dT, p, nt, t, 0, nh, hh, n, e); }\n')
    subprocess.run(["g++", "-std=gnu++98", "-DDEBUG=0", "-c", "-I", REF_INC, "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(tmp_path / "tu.o")],
                   check=True, capture_output=True, text=True)


def _write_case(path, g, mode, steps, V0=None):
    spec = g["spec"]
    e = g["eparam"]
    hp = g["hparam"]
    V0 = spec.rest_pot if V0 is None else V0
    r = lambda x: repr(float(x))  # plain decimal text (numpy 2 reprs carry a type prefix)
    with open(path, "w") as f:
        f.write(f"{mode} {spec.n} {len(spec.terminals)} {steps} {r(g['dT'])} "
                f"{r(spec.init_time)} {r(spec.end_input)}\n")
        f.write(" ".join(str(int(t)) for t in spec.terminals) + "\n")
        f.write(f"{len(g['hh_elem'])} " + " ".join(str(int(x)) for x in g["hh_elem"]) + "\n")
        for i in range(spec.n):
            f.write(f"{int(spec.mother[i])} {int(spec.dr[i])} {int(spec.dl[i])} "
                    f"{int(spec.branching[i])} {r(e[2, i])} {r(e[0, i])} {r(e[1, i])} "
                    f"{r(e[3, i])} {r(e[4, i])} {r(spec.input_current[i])} {r(V0[i])}\n")
        for k in range(len(g["hh_elem"])):
            f.write(" ".join(r(hp[q, k]) for q in range(12)) + "\n")


@pytest.mark.gpu
@pytest.mark.parametrize("name,mode", [("axon1000_dtf08", 0), ("rtree1500", 0), ("im_ytree_d3", 1)])
def test_dropin_adapter_runs_reference_loop(gpu, lib, orc, tmp_path, name, mode):
    g = load_golden(name)
    exe = str(tmp_path / "dropin")
    _compile(lib, exe)
    steps = int(g["numStepsT"]) - 2
    case = str(tmp_path / "case.txt")
    _write_case(case, g, mode, steps)
    out = str(tmp_path / "V.txt")
    subprocess.run([exe, case, out], check=True, capture_output=True, text=True, timeout=600)
    V = np.loadtxt(out)
    if mode == 0:
        assert np.abs(V - g["final_V"]).max() < 1e-9
    else:
        # default implicit options: ||r||_2 <= 1e-14 absolute, like the reference
        assert np.abs(V - g["final_V"]).max() < 1e-5
