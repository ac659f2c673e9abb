"""Recording on the host side: the measurement point against the reference's own output,
the sample counter against the reference driver's, and the trace text format."""
import numpy as np
import pytest

from conftest import golden_names, load_golden


@pytest.mark.parametrize("name", golden_names())
def test_measurement_point_matches_reference(pkg, lib, orc, name):
    """nrt_measurement_point and the oracle's restatement give the index the reference's
    measurement_point (src/init.cpp:339-358) returned for each distance in the fixture:
    zero, the first element's dX (its 'found at 0' case), fractions of the length, the
    whole length and twice it (never reached)."""
    import oracle
    g = load_golden(name)
    dx = g["eparam"][2]
    for dist, want in zip(g["mp_dist"], g["mp_index"]):
        assert oracle.measurement_point(dx, float(dist)) == want
        assert pkg.measurement_point(dx, float(dist)) == want


def test_measurement_point_rejects_bad_arguments(pkg, lib):
    import ctypes
    out = ctypes.c_int32(0)
    d = np.ones(3)
    assert lib.nrt_measurement_point(0, d.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1.0,
                                     ctypes.byref(out)) == 1
    assert lib.nrt_measurement_point(3, None, 1.0, ctypes.byref(out)) == 1


def reference_counter(i_first, i_last, interval):
    """The reference driver's sampling (src/neurite.cpp:241-242) restated as its loop:
    GL_cont starts at 0 and a snapshot is taken when ++GL_cont > interval."""
    cont, out = 0, []
    for i in range(i_first, i_last):
        cont += 1
        if cont > interval:
            cont = 0
            out.append(i)
    return out


@pytest.mark.parametrize("interval", [0, 1, 4, 49, 399])
def test_sample_rule_is_the_reference_counter(interval):
    import oracle
    steps = np.zeros(1200)
    samples, _ = oracle.recording(1, 0.0, steps, 1, interval, 0.5, 1.0)
    rule = [1 + (k + 1) * (interval + 1) - 1 for k in sorted(samples)]
    assert rule == reference_counter(1, 1 + len(steps), interval)


@pytest.mark.parametrize("name", golden_names())
def test_golden_traces_follow_the_sample_rule(name):
    """The fixtures' traces (sampled where i % record_every == 0 from i = 1) are the
    samples of origin 1, interval record_every - 1."""
    import oracle
    g = load_golden(name)
    rec = int(g["record_every"])
    n_loop = int(g["trace"][-1, 0]) if len(g["trace"]) else 0
    samples, _ = oracle.recording(1, 0.0, np.zeros(n_loop), 1, rec - 1, 0.5, 1.0)
    rows = [1 + (k + 1) * rec - 1 for k in sorted(samples)]
    assert rows == [int(i) for i in g["trace"][:, 0]]


def test_spike_interpolation():
    import oracle
    steps = [-0.06, -0.01, 0.02, 0.03, -0.02, 0.01]
    _, spikes = oracle.recording(5, -0.07, steps, 1, 0, 0.0, 2.0)
    # crossings between i=6 -> 7 and i=9 -> 10
    assert spikes == pytest.approx([12.0 + 0.01 / 0.03 * 2.0, 18.0 + 0.02 / 0.03 * 2.0])


def test_trace_text_format(pkg):
    r = pkg.Recording([np.array([1e-6, 2e-6])], [np.array([-0.065, 0.0123])],
                      np.array([2]), [np.array([])], np.array([0]))
    lines = r.trace_text(0).splitlines()
    assert lines == ["%.20f %.20f" % (1e-6, -0.065), "%.20f %.20f" % (2e-6, 0.0123)]
    assert lines[0].split()[0] == "0.00000100000000000000"
