"""The segmented-neuron loader (model.from_neurite_txt) against the reference's own loader.

tests/golden/loader_example8.npz holds the seven columns of the reference's example-8 neuron
file (applications/example_8/neuron_for_neurite.txt: me mother dR branching dL diameter_um
length_um, read as numbers) and the elements the reference's loading_neuron_passive_dendritic_tree
(src/space.cpp:37-183, selected by simulation=CT_segmented_neuron at src/init.cpp:120-121)
built from them, through oracle/ref_harness.cpp's mode L.  The file is written back as text
(every number round-trips exactly) and read by the package's loader; the element arrays must
agree bit for bit."""
import numpy as np

from conftest import GOLDEN


def _text(g):
    lines = []
    for ints, flts in zip(g["rows_int"], g["rows_float"]):
        lines.append(" ".join(str(int(x)) for x in ints) + " " + " ".join(repr(float(x)) for x in flts))
    return "\n".join(lines) + "\n"


def test_loader_matches_reference_loader(model):
    g = np.load(f"{GOLDEN}/loader_example8.npz")
    spec = model.from_neurite_txt(_text(g), hh=False)
    n = len(g["mother"])
    assert spec.n == n
    assert np.array_equal(spec.mother, g["mother"])
    assert np.array_equal(spec.dr, g["dr"])
    assert np.array_equal(spec.dl, g["dl"])
    assert np.array_equal(spec.branching.astype(np.int32), g["branching"])
    assert np.array_equal(spec.dX, g["dX"])            # bit for bit
    assert np.array_equal(spec.diameter, g["diameter"])
    assert np.array_equal(spec.input_current, g["input_current"])
    assert np.array_equal(spec.terminals, g["terminals"])
    assert len(spec.terminals) == int(g["num_terminals"])


def test_loader_golden_is_the_example_neuron():
    """The fixture is the 878-row example neuron: every non-terminal row continues to the
    next element (the reference ignores the file's dR there and uses me + 1), branch rows
    name a later element as DL, and the reference's element 0 copies row 1's geometry."""
    g = np.load(f"{GOLDEN}/loader_example8.npz")
    rows = g["rows_int"]
    assert rows.shape == (878, 5)
    me, dR, br, dL = rows[:, 0], rows[:, 2], rows[:, 3], rows[:, 4]
    term = me == dR
    assert np.array_equal(g["dr"][me[~term]], me[~term] + 1)
    assert (dL[br != 0] > me[br != 0]).all()
    assert g["dX"][0] == g["rows_float"][0, 1] * 1e-6
