"""Host-side checks that need no GPU: the C ABI library loads and exports every declared
symbol, the host parameter pipeline matches the reference, input validation rejects bad
trees before touching a device, and the tree builders emit the reference numbering."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(nrt_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(lib, pkg):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(pkg._lib.EXPORTS)


@pytest.mark.parametrize("name", golden_names())
def test_library_derivation_matches_reference(pkg, lib, name):
    g = load_golden(name)
    d = pkg.derive(g["spec"])
    assert d.dT_crit == g["dT_crit"]
    np.testing.assert_array_equal(d.hh_elem, g["hh_elem"])
    np.testing.assert_allclose(d.eparam, g["eparam"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(d.hparam, g["hparam"], rtol=1e-14, atol=1e-300)


def _problem(pkg, g):
    return pkg.ProblemArrays.from_spec(g["spec"], pkg.Derived(g["eparam"], g["hh_elem"],
                                                              g["hparam"], float(g["dT_crit"])),
                                       float(g["dT"]))


def test_status_strings(lib):
    assert lib.nrt_status_string(0) == b"ok"
    assert b"topology" in lib.nrt_status_string(2)


@pytest.mark.parametrize("mode", [0, 1])
def test_create_rejects_bad_topology_without_device(pkg, lib, mode):
    g = load_golden("ytree_d3_strain")
    p = _problem(pkg, g)
    p.arrays["mother"][5] = p.num_elem + 7   # out of range
    opts = pkg.solver.make_options(mode)
    h = ctypes.c_void_p()
    rc = lib.nrt_create(ctypes.byref(p.struct), ctypes.byref(opts), ctypes.byref(h))
    assert rc == 2 and not h.value
    assert b"range" in lib.nrt_last_error()


def test_create_rejects_bad_options_without_device(pkg, lib):
    g = load_golden("ytree_d3_strain")
    p = _problem(pkg, g)
    for field, val in [("restart", 0), ("restart", 999), ("tol", -1.0), ("precision", 7),
                       ("step_threads", 48), ("step_threads", 512), ("step_threads", -32),
                       ("tile_ctas_per_sm", -1), ("tile_ctas_per_sm", 65)]:
        opts = pkg.solver.make_options(1)
        setattr(opts, field, val)
        h = ctypes.c_void_p()
        assert lib.nrt_create(ctypes.byref(p.struct), ctypes.byref(opts), ctypes.byref(h)) == 1


def test_options_struct_matches_the_header(pkg, lib):
    """The Python mirror of nrt_options has the C layout: nrt_options_default fills every
    field the header documents, and the launch-shape fields sit where the header puts them."""
    import ctypes as ct
    o = pkg._lib.Options()
    ct.memset(ct.byref(o), 0x7f, ct.sizeof(o))
    assert lib.nrt_options_default(ct.byref(o)) == 0
    assert ct.sizeof(o) == 4 * 6 + 8 + 4 * 8 + 8 + 4 * 2  # 6 ints, tol, 8 ints, inner_tol, 2 ints
    assert (o.tiled, o.use_graphs, o.tile_ctas_per_sm, o.step_threads) == (1, 1, 0, 0)
    assert o.inner_tol == 0.0
    assert (o.step_launch, o.refinement) == (0, 0)


def test_implicit_requires_reference_numbering(pkg, lib, model):
    # a branch point whose DL child is not a later element: fine for the explicit gather
    # formulation, rejected for the reference's implicit assembly
    g = load_golden("im_ytree_d3")
    p = _problem(pkg, g)
    b = int(np.nonzero(p.arrays["branching"])[0][0])
    p.arrays["dl"][b] = b - 1
    h = ctypes.c_void_p()
    rc = lib.nrt_create(ctypes.byref(p.struct), ctypes.byref(pkg.solver.make_options(1)),
                        ctypes.byref(h))
    assert rc == 2


def test_builders_follow_reference_numbering(model):
    model.straight_axon().validate()
    s = model.random_binary_tree(depth=10, seed=2)
    s.validate()
    assert 2.0e5 < s.n < 3.2e5 and len(s.terminals) == 1 + 2 ** 10
    s = model.random_tree(seed=3, n_target=5000)
    s.validate()
    assert 3000 < s.n < 8000
    m = model.myelinated_axon(n_nodes=5, internode_len=50e-6, dx=1e-6, node_len=1e-6)
    m.validate()
    assert int((m.kind == 1).sum()) == 5


def test_neurite_txt_loader_round_trip(model):
    g = load_golden("example8_passive")
    s = g["spec"]
    rows = []
    for me in range(1, s.n):
        rows.append(f"{me} {s.mother[me]} {s.dr[me]} {s.branching[me]} {s.dl[me]} "
                    f"{s.diameter[me] * 1e6:.6f} {s.dX[me] * 1e6:.6f}")
    t = model.from_neurite_txt("\n".join(rows), hh=False)
    np.testing.assert_array_equal(t.mother, s.mother)
    np.testing.assert_array_equal(t.dr, s.dr)
    np.testing.assert_array_equal(t.dl, s.dl)
    np.testing.assert_array_equal(t.terminals, s.terminals)
    # the reference's loader (src/space.cpp:37-183) yields exactly this numbering
    assert len(s.terminals) == 59 and s.n == 879


def test_spec_serialisation_round_trip(model):
    s = model.random_tree(seed=4, n_target=2000)
    t = model.TreeSpec.from_arrays(s.to_arrays())
    for k in model.ISPEC_ROWS + model.DSPEC_ROWS:
        np.testing.assert_array_equal(getattr(s, k), getattr(t, k))
    assert t.tspan == s.tspan and t.myelin == s.myelin
