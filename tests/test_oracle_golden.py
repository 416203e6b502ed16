"""The oracle reproduces its committed FP64 golden fixtures (regression)."""
import os

import numpy as np
import pytest

from mocassin_gb300 import nebula
from oracle import runner
from tests.golden import make_golden

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "transport_small_fp64.npz"))


@pytest.mark.parametrize("spec", nebula.small_cases(), ids=lambda s: s.name)
def test_oracle_matches_golden(spec):
    neb = nebula.build(spec)
    js, _, es, st = runner.run(neb, precision="fp64", seed=make_golden.SEED)
    counts = np.array([st[k] for k in make_golden.KEYS])
    np.testing.assert_array_equal(counts, GOLDEN[spec.name + "/counts"])
    np.testing.assert_allclose(js.sum(0), GOLDEN[spec.name + "/j_cell"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(js.sum(1), GOLDEN[spec.name + "/j_nu"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(es.sum(1), GOLDEN[spec.name + "/esc_nu"], rtol=1e-12, atol=0)


def test_fp32_oracle_agrees_with_fp64_within_noise():
    """The FP32 restatement (the reference's `real`) and the FP64 one agree on
    the band-integrated J of the whole grid within 4 sigma of packet noise."""
    spec = nebula.small_cases()[1]
    neb = nebula.build(spec)
    tot = {"fp64": [], "fp32": []}
    for seed in range(1, 9):
        for prec in ("fp64", "fp32"):
            js, _, _, _ = runner.run(neb, n_packets=2000, precision=prec, seed=seed)
            tot[prec].append(js.sum())
    a, b = np.array(tot["fp64"]), np.array(tot["fp32"])
    sig = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    assert abs(a.mean() - b.mean()) < 4 * sig
