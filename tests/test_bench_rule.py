"""The algorithmic-bytes rule behind every `roofline` figure of bench.py, pinned to its
worked figures:

- the uniform 1 cm squid axon, HH everywhere: 68 B per compartment-step in FP64 (V r/w 16,
  gates r/w 48, parent index 4) and 44 B in mixed precision (FP32 gates);
- the myelinated axon's passive internodes: 36 B FP64 / 28 B mixed (V 16, index 4, and the
  two coefficients dT/(c_m dX), 1/(r_a dX), because the geometry differs between nodes and
  internodes);
- the implicit rule: assembly plus, per Krylov iteration, a CSR SpMV of 36 B and the
  orthogonalisation's 4 (2 (j + 1) + 1) B per row.

Variation is judged over the compartments a step computes; the fictitious root and the
sealed ends are copies of their neighbours and do not make a uniform tree look varied.
"""
import numpy as np
import pytest

import bench


@pytest.fixture(scope="module")
def axon(pkg, model):
    spec = model.straight_axon(dtf=0.8)
    return pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))


@pytest.fixture(scope="module")
def myelin(pkg, model):
    spec = model.myelinated_axon(n_nodes=12, internode_len=40e-6)
    return pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))


@pytest.mark.parametrize("precision,per_hh", [("fp64", 68), ("mixed", 44)])
def test_uniform_axon(axon, precision, per_hh):
    n, n_hh = axon.num_elem, int(axon.struct.num_hh)
    assert (n, n_hh) == (1002, 1000)
    # the two fictitious ends are passive: potential and index only
    assert bench.algorithmic_bytes_explicit([axon], precision) == n_hh * per_hh + (n - n_hh) * 20


@pytest.mark.parametrize("precision,fb,per_cable,per_node",
                         [("fp64", 8, 36, 84), ("mixed", 4, 28, 52)])
def test_myelinated_axon(myelin, precision, fb, per_cable, per_node):
    n, n_hh = myelin.num_elem, int(myelin.struct.num_hh)
    assert n_hh == 12
    ph, pp = bench._param_bytes(myelin, fb)
    assert (ph, pp) == (2 * fb, 2 * fb)  # geometry varies; channels and W, K do not
    total = bench.algorithmic_bytes_explicit([myelin], precision)
    assert total == n_hh * per_node + (n - n_hh) * per_cable


def test_implicit_rule(axon):
    n, n_hh = axon.num_elem, int(axon.struct.num_hh)
    steps, iters, basis = 10, 30.0, 45.0  # per run: 3 iterations and 4.5 basis vectors a step
    counts = {"basis": [basis], "residuals": [20.0], "applies": [30.0], "xupdates": [20.0]}
    rule, passes = bench.algorithmic_bytes_implicit([axon], steps, [iters], counts)
    asm = n_hh * (24 + 24) + (n - n_hh) * 24  # uniform tree: no varying parameters
    assert rule == pytest.approx(asm + n * (36 * iters + 4 * (2 * basis + iters)) / steps)
    per_run = 37 * 20 + 38 * 30 + (17 + 8 + 4) * iters + 8 * basis + 17 * 20
    assert passes == pytest.approx(n_hh * 85 + (n - n_hh) * 77 + n * 29 + n * per_run / steps)


def test_implicit_rule_richardson_steps(axon):
    """Richardson refinement steps: no Krylov iteration, one FP64 SpMV (56 B) each under the
    rule; their applications, updates and residuals are counted passes as before."""
    n, n_hh = axon.num_elem, int(axon.struct.num_hh)
    steps = 10
    counts = {"basis": [0.0], "residuals": [20.0], "applies": [20.0], "xupdates": [20.0],
              "richardson": [20.0]}
    rule, passes = bench.algorithmic_bytes_implicit([axon], steps, [0.0], counts)
    asm = n_hh * (24 + 24) + (n - n_hh) * 24
    assert rule == pytest.approx(asm + n * 56 * 20 / steps)
    per_run = 37 * 20 + 38 * 20 + 17 * 20
    assert passes == pytest.approx(n_hh * 85 + (n - n_hh) * 77 + n * 29 + n * per_run / steps)


def test_varied_geometry_is_charged(pkg, model):
    """A random tree (diameter set per branch level) pays for both coefficients."""
    spec = model.random_tree(seed=4, n_target=800)
    p = pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))
    ph, _ = bench._param_bytes(p, 8)
    assert ph >= 16
    assert np.isfinite(bench.algorithmic_bytes_explicit([p], "fp64"))
