"""Host side of the grain temperatures (getDustT, source/update_mod.f90:1836-1945).

The grains of the dusty workloads are one silicate-like species in 10 MRN
size bins (mocassin_gb300.nebula._dust_kappa).  Per size bin a the
reference forms, for every cell,
    absorbed(a) = sum_i xSecAbs(a, i) Jste(i) / pi             (:1858-1866)
on the normalised Jste, and finds the temperature whose emission
    dustEmIntegral(a, T) = 4 h sum_i xSecAbs(a, i) B(nu_i, T) fr1Ryd widFlx(i),
    T = 1 .. 3000 K                                             (dust_mod.f90:150-178)
equals it, by `locate` and a linear step (:1899-1915).  The absorbed
integrals are moments of Jste (the tensor-core moment kernel); this module
builds their weights and the emission table.
"""
import numpy as np

from . import nebula

NTEMPS = 3000                      # constants_mod.f90:55
GRAIN_VN = 0.588                   # grainVn [Ryd] of the silicate of dustData/sil-dlee.nk
GRAIN_MSURF = 20.077               # MsurfAtom of the same file (ph_mod.f90:910-911)
HPLANCK = 6.6262e-27               # constants_mod.f90:14
FR1RYD = 3.28984e15                # constants_mod.f90:13
HCRYD_K = 157893.94                # continuum_mod.f90:10


def grains(nu):
    """(xs_abs [nsizes, nbins] cm^2 per grain, number weights [nsizes], radii [nsizes] cm)."""
    a = np.logspace(np.log10(0.005e-4), np.log10(0.25e-4), 10)
    w = a ** -3.5 * np.gradient(a)
    w = w / w.sum()
    lam = 2.9979250e10 / (nu.astype(np.float64) * FR1RYD)
    x = 2.0 * np.pi * a[:, None] / lam[None, :]
    qa = 1.0 - np.exp(-0.5 * x)
    return np.pi * a[:, None] ** 2 * qa, w, a


def planck_over_h(energy, t):
    """getFlux(energy [Ryd], T, 'blackbody') (continuum_mod.f90:359-394), FP64."""
    constant = 0.5250229 / HPLANCK
    e = np.asarray(energy, dtype=np.float64)
    u = HCRYD_K * e / t
    out = np.empty_like(u)
    big = u > 86.0
    out[big] = constant * e[big] ** 3 * np.exp(-u[big])
    den = np.expm1(u[~big])
    small = den <= 0
    val = constant * e[~big] ** 3 / np.where(small, 1.0, den)
    val[small] = (3.32154e-6 * e[~big] ** 2 * t / HPLANCK)[small]
    out[~big] = val
    return out


def emission_table(xs_abs, nu):
    """dustEmIntegral [nsizes, NTEMPS] for T = 1 .. NTEMPS K."""
    wf = nebula.wid_flx(nu).astype(np.float64)
    nu64 = nu.astype(np.float64)
    tab = np.zeros((xs_abs.shape[0], NTEMPS))
    for k in range(NTEMPS):
        b = planck_over_h(nu64, float(k + 1))
        tab[:, k] = (xs_abs * (b * FR1RYD * wf)[None, :]).sum(1)
    return tab * HPLANCK * 4.0


def absorption_weights(xs_abs):
    """Moment weights [nbins, nsizes]: xSecAbs / pi."""
    return np.ascontiguousarray((xs_abs / np.pi).T.astype(np.float32))


def grain_opacity(nu):
    """Per size bin the extinction (abs + sca) and scattering cross-sections
    per grain [nsizes, nbins] cm^2 (FP32) and the number weights [nsizes] of
    the synthetic MRN mix whose sums are the workloads' dust opacity
    (nebula._dust_kappa: Q_abs = 1 - exp(-x/2), Q_sca = 0.9 x^4 / (1 + x^4))."""
    xs_abs, w, a = grains(nu)
    lam = 2.9979250e10 / (nu.astype(np.float64) * FR1RYD)
    x = 2.0 * np.pi * a[:, None] / lam[None, :]
    xs_sca = np.pi * a[:, None] ** 2 * (0.9 * x ** 4 / (1.0 + x ** 4))
    return (np.ascontiguousarray((xs_abs + xs_sca).astype(np.float32)), np.ascontiguousarray(xs_sca.astype(np.float32)),
            w.astype(np.float32))


def grain_physics(neb, abundance=1.0):
    """The grains of the photoelectric and gas-grain collision terms of the
    cell update (setGrainPotential, setPhotoelHeatCool,
    setDustGasCollHeatCool, source/update_mod.f90:527-930): the absorption
    cross-sections per grain [nsizes][nbins] (FP32, as the opacity and the
    grain temperatures use them), radii [um], number weights, the species
    abundance, grainVn and MsurfAtom, the frequency grid and the threshold
    of every balance ion (the first bin with a nonzero cross-section, the
    same IP as the heating sums), and Ndust per cell."""
    from . import balance
    xs, w, a = grains(neb.nu)
    ions = [tuple(int(v) for v in r) for r in nebula.atomic_table()["ions"]]
    return {"xs_abs": np.ascontiguousarray(xs.astype(np.float32)), "radius_um": a * 1e4, "weight": w,
            "abundance": float(abundance), "vn": GRAIN_VN, "msurf": GRAIN_MSURF,
            "nu": neb.nu.astype(np.float64), "ion_nu": balance.ion_thresholds(neb.xs, neb.nu, ions),
            "ndust": np.ascontiguousarray(neb.ndust, dtype=np.float32)}
