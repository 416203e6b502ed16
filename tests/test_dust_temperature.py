"""Grain temperatures from radiative balance (getDustT) on the GPU, against the
CPU oracle, and the Kirchhoff known answer: grains in a blackbody field of
temperature T0 (J_nu = pi B_nu, the estimator's units) come out at T0."""
import ctypes as C
import ctypes.util

import numpy as np
import pytest

from mocassin_gb300 import dust, nebula, transport
from oracle import dust_oracle


def _blackbody_jste(nu, t0):
    """Normalised Jste per bin of an isotropic blackbody field: 4 pi h B/h(nu, T0) fr1Ryd widFlx."""
    b = dust.planck_over_h(nu.astype(np.float64), t0)
    return 4.0 * np.pi * dust.HPLANCK * b * dust.FR1RYD * nebula.wid_flx(nu).astype(np.float64)


@pytest.mark.parametrize("t0", [20.0, 57.0, 140.0, 800.0])
def test_oracle_kirchhoff(t0):
    neb = nebula.build(nebula.small_cases()[3])
    xs, w, _ = dust.grains(neb.nu)
    em = dust.emission_table(xs, neb.nu)
    j = _blackbody_jste(neb.nu, t0)
    absorbed = (xs / np.pi) @ j
    for k in range(len(w)):
        assert abs(dust_oracle.temperature(em[k], absorbed[k]) - t0) < 1e-6 * t0


def test_locate_rules():
    xa = np.array([1.0, 2.0, 4.0, 8.0])
    assert dust_oracle.locate(xa, 0.5) == 0 and dust_oracle.locate(xa, 9.0) == 4
    assert dust_oracle.locate(xa, 1.0) == 1 and dust_oracle.locate(xa, 3.0) == 2 and dust_oracle.locate(xa, 4.0) == 3
    assert dust_oracle.locate(xa, 8.0) == 1   # no entry exceeds it: minloc of an empty mask


def _cudart():
    for name in ("cudart", "cudart64"):
        p = ctypes.util.find_library(name)
        if p:
            return C.CDLL(p)
    return C.CDLL("libcudart.so")


@pytest.mark.gpu
@pytest.mark.parametrize("case", [3, 4], ids=["full11_dust_iso", "full9_dust_hg"])
def test_gpu_matches_oracle(gpu_lib, case):
    neb = nebula.build(nebula.small_cases()[case])
    ctx = transport.TransportContext(neb)
    ctx.run(seed=4, precision="fp64")
    js, _, _ = ctx.download()
    xs, w, _ = dust.grains(neb.nu)
    em = dust.emission_table(xs, neb.nu)
    wab = dust.absorption_weights(xs)
    td, ms = ctx.dust_temperatures(wab, em, w, 1e-9)
    ctx.close()
    absorbed = wab.T.astype(np.float64) @ (js * 1e-9)
    hit = (js > 0).any(0)
    ref = dust_oracle.dust_temperatures(absorbed, em.astype(np.float32).astype(np.float64), w, hit)
    c = np.nonzero(hit[1:])[0] + 1
    assert len(c) > 10
    # FP32 tensor-core moments (3e-5) against FP64 sums: T ~ A^(1/6) moves by ~1e-5
    np.testing.assert_allclose(td[:, c], ref[:, c], rtol=2e-4)
    assert np.all(td[:, np.nonzero(~hit)[0]] == 0)


@pytest.mark.gpu
def test_gpu_kirchhoff(gpu_lib):
    neb = nebula.build(nebula.small_cases()[3])
    ctx = transport.TransportContext(neb)
    t0 = 75.0
    j = np.tile(_blackbody_jste(neb.nu, t0)[:, None], (1, neb.ncells + 1)) / 1e-9
    jd, _, _ = ctx.device_estimators()
    rt = _cudart()
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    jj = np.ascontiguousarray(j)
    assert rt.cudaMemcpy(C.c_void_p(jd), jj.ctypes.data_as(C.c_void_p), jj.nbytes, 1) == 0
    xs, w, _ = dust.grains(neb.nu)
    td, _ = ctx.dust_temperatures(dust.absorption_weights(xs), dust.emission_table(xs, neb.nu), w, 1e-9)
    ctx.close()
    np.testing.assert_allclose(td[1:, 1:], t0, rtol=5e-4)
    np.testing.assert_allclose(td[0, 1:], t0, rtol=5e-4)
