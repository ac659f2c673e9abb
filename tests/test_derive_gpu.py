"""The parameter pipeline on the GPU for many trees at once (nrt_derive_batch) against the
host pipeline (nrt_derive, pinned bit for bit to the reference's own code) and the
reference's outputs in the golden fixtures."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

RTOL = 1e-13   # device exp / pow / sqrt and fused multiply-adds vs the host's


def test_derive_batch_matches_golden(gpu, pkg):
    gs = [load_golden(n) for n in golden_names()]
    out = pkg.derive_batch([g["spec"] for g in gs])
    for g, d in zip(gs, out):
        np.testing.assert_array_equal(d.hh_elem, g["hh_elem"])
        np.testing.assert_allclose(d.eparam, g["eparam"], rtol=RTOL, atol=0)
        np.testing.assert_allclose(d.hparam, g["hparam"], rtol=RTOL, atol=1e-300)
        assert d.dT_crit == pytest.approx(float(g["dT_crit"]), rel=RTOL)


def test_derive_batch_matches_host_on_a_population(gpu, pkg, model):
    specs = [model.random_tree(seed=400 + k, n_target=int(n), strain=0.1)
             for k, n in enumerate(model.log_uniform_sizes(24, 1e3, 3e4, 5))]
    specs.append(model.myelinated_axon(n_nodes=9, internode_len=80e-6, dtf=0.8))
    specs.append(model.straight_axon(dtf=0.8))
    out = pkg.derive_batch(specs)
    for sp, d in zip(specs, out):
        h = pkg.derive(sp)
        np.testing.assert_array_equal(d.hh_elem, h.hh_elem)
        np.testing.assert_allclose(d.eparam, h.eparam, rtol=RTOL, atol=0)
        np.testing.assert_allclose(d.hparam, h.hparam, rtol=RTOL, atol=1e-300)
        assert d.dT_crit == pytest.approx(h.dT_crit, rel=RTOL)
