"""Stochastic parity of the GPU Lambda iteration with the CPU oracle's.

A small, fully ionised clumpy nebula (13^3 full grid over +/-3e18 cm,
lognormal nH with median 30 cm^-3, 60 kK star of 5e37 erg/s, 600 bins,
1e5 packets per iteration) is iterated five times from the same initial
state by

- the GPU: the frequency-sorted FP32 march in a CUDA graph, the cell update
  (FP64, or FP32 in the chosen form), the opacity rebuild on the tensor cores
  (split BF16) and the emission CDFs on the GPU (iterate.LambdaIteration),
  and
- the CPU oracle: the FP64 transport, FP64 update, FP64 opacity and FP64
  emission CDFs (oracle/lambda_oracle.py),

each over 6 independent seed sets.  After the fifth iteration, per cell Te,
the main ionic fractions, and the forbidden-line luminosity of each line ion
(sum of emissivity x Hden x dV over the grid, outputGas,
output_mod.f90:455-520) are compared through the z-score of the difference
of the two sides' means (its standard error from the seed-to-seed spread):

- the GPU with the FP64 cell update (FP32 march, split-BF16 opacity, FP32
  emission CDFs) agrees with the oracle within 3 sigma of the packet noise on
  all three, for >= 95 % of the entries, with a mean squared z-score near 1;
- the chosen form (FP32 cell update) agrees within 3 sigma on Te and the
  ionic fractions.  Its line luminosities carry a systematic error: the FP32
  secant stops at another Te inside the reference's 1 % balance tolerance
  (update_mod.f90:391-491) and forbidden lines amplify a Te error several
  times, so for them the test bounds the error against the FP64 oracle (the
  mean over seeds) instead: median below 2 %, every line ion above 1e-3 of
  the brightest within 10 %.

The differences of the means against the FP64 oracle are printed for every
result.
"""
import numpy as np
import pytest

from mocassin_gb300 import iterate, nebula
from oracle import lambda_oracle

pytestmark = pytest.mark.gpu

SEEDS = 6
ITERATIONS = 5
PACKETS = 100000


def _spec():
    return nebula.NebulaSpec("clumpy13_ionised", 13, 3.0e18, False,
                             [nebula.Star(60000.0, 50.0, (0, 0, 0), PACKETS)],
                             nh_median=30.0, sigma_ln=1.0, smooth_cells=1.5, seed=1)


def _z(a, b):
    """z-scores of the difference of the means of samples a and b (axis 0)."""
    se = np.sqrt(a.var(0, ddof=1) / len(a) + b.var(0, ddof=1) / len(b))
    return (a.mean(0) - b.mean(0)), se


def _check(name, a, b, mask, sigma_gate=True):
    d, se = _z(a, b)
    ok = mask & (se > 0)
    z = d[ok] / se[ok]
    rel = np.abs(d[ok]) / np.abs(b.mean(0)[ok])
    print("%s: %d entries, |z|<3 for %.1f %%, mean z^2 %.2f, |GPU - oracle| / oracle median %.2e, 95th %.2e, max %.2e"
          % (name, ok.sum(), 100 * np.mean(np.abs(z) < 3), np.mean(z ** 2), np.median(rel), np.percentile(rel, 95),
             rel.max()))
    assert ok.sum() > 0
    if sigma_gate:
        assert np.mean(np.abs(z) < 3.0) >= 0.95, name
        assert 0.4 < np.mean(z ** 2) < 2.0, name
    return rel


def _gpu_runs(neb, update):
    te_, x_, lum = [], [], []
    for s in range(SEEDS):
        li = iterate.LambdaIteration(neb, form="graph", update=update)
        for it in range(ITERATIONS):
            li.step(seed=100 * s + it + 1)
        te, ne, X, _, _, _ = li.state()
        li.close()
        te_.append(te[1:])
        x_.append(X[1:])
        lum.append(lambda_oracle.line_luminosities(neb, te, ne, X))
    return np.array(te_), np.array(x_), np.array(lum)


_ORACLE = {}


def _oracle_runs(neb):
    if "runs" not in _ORACLE:
        te_, x_, lum = [], [], []
        for s in range(SEEDS):
            lo = lambda_oracle.OracleLambda(neb)
            for it in range(ITERATIONS):
                lo.step(seed=100 * s + 50 + it + 1)
            te_.append(lo.te[1:])
            x_.append(lo.X[1:])
            lum.append(lambda_oracle.line_luminosities(neb, lo.te, lo.ne, lo.X))
        _ORACLE["runs"] = (np.array(te_), np.array(x_), np.array(lum))
    return _ORACLE["runs"]


# H+, He+, He++, O+, O++, N+, Ne++, S+ and S++
IONS = [(0, 2), (1, 2), (1, 3), (4, 2), (4, 3), (3, 2), (5, 3), (6, 2), (6, 3)]


def _compare(neb, update, line_sigma_gate):
    gte, gx, glum = _gpu_runs(neb, update)
    ote, ox, olum = _oracle_runs(neb)
    _check("Te (%s update)" % update, gte, ote, np.ones(gte.shape[1], bool))
    ga = np.stack([gx[:, :, e, s] for e, s in IONS], axis=2)
    oa = np.stack([ox[:, :, e, s] for e, s in IONS], axis=2)
    _check("ionic fractions (%s update)" % update, ga, oa, (oa.mean(0) > 1e-3) & (ga.mean(0) > 1e-3))
    big = olum.mean(0) > 1e-3 * olum.mean(0).max()
    return _check("line luminosities (%s update)" % update, glum, olum, big, sigma_gate=line_sigma_gate)


def test_lambda_iteration_with_the_fp64_update_matches_the_oracle_within_3_sigma(gpu_lib):
    _compare(nebula.build(_spec()), "fp64", True)


def test_chosen_lambda_iteration_matches_the_oracle(gpu_lib):
    rel = _compare(nebula.build(_spec()), "fp32", False)
    assert np.median(rel) < 0.02 and rel.max() < 0.10
