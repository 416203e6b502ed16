"""Synthetic nebulae in mocassin's own grid layout.

Builds, for one transport iteration, every array the packet transport reads,
laid out as the Fortran side holds it (column-major, so the numpy arrays are
``(nbins, Nc+1)`` C-order == ``opacity(0:Nc, 1:nbins)`` cell fastest):

* axes            grid_mod.f90:530-601 (symmetricXYZ / full odd grid), FP32
* active map      grid_mod.f90:1225-1294: numbering loops x outer, z inner;
                  cells outside R_in / R_out, or without gas and dust, are 0
* geoCorr         grid_mod.f90:807-820
* star cell       setStarPosition, grid_mod.f90:3569-3649 with ``locate``
                  (interpolation_mod.f90:48-81)
* initial ions    grid_mod.f90:1562-1600 (H0 = 1e-5 start) or a two-zone
                  ionised/neutral structure for absorption-heavy cases
* stellar CDF     getFlux (blackbody) + setProbDen, continuum_mod.f90:359-474;
                  deltaE = L/N, continuum_mod.f90:303-343
* opacity         the dense form of addOpacity (ionization_mod.f90:349-484):
                  den[cell, ion] @ XS[ion, nu] plus the dust term of
                  iteration_mod.f90:166-227

The emission CDFs (recPDF, totalLines) that emission_mod builds from the full
recombination physics are synthetic here: a Milne-relation recombination
continuum of each ion plus a free-free tail (and a grain thermal term when
dust is present), and a constant line fraction.  They are inputs consumed
identically by the GPU path and the oracle.
"""
from __future__ import annotations

import dataclasses
import os
from typing import List, Optional

import numpy as np

f32 = np.float32
HCRYD_K = 157893.94          # h c Ryd / k  [K]   continuum_mod.f90:10
HPLANCK = 6.6262e-27         # constants_mod.f90:14
RADIO_4P9GHZ = 1.489434e-6

# number abundances relative to H of the benchmark sets
ABUNDANCES = {1: 1.0, 2: 0.1, 6: 2.2e-4, 7: 4.0e-5, 8: 3.3e-4, 10: 5.0e-5, 16: 9.0e-6}

FLAG_SYMMETRIC_XYZ = 1 << 0
FLAG_GAS = 1 << 1
FLAG_DUST = 1 << 2
FLAG_ISOTROPIC = 1 << 3
FLAG_DEBUG = 1 << 4
FLAG_MULTISTARS = 1 << 5

_TABLE = None


def atomic_table():
    """Frequency grid (600 bins, 1e-5..24.5 Ryd), XS[ion, nu] [cm^2], ions."""
    global _TABLE
    if _TABLE is None:
        d = np.load(os.path.join(os.path.dirname(__file__), "data", "atomic_table.npz"))
        _TABLE = {k: d[k] for k in d.files}
    return _TABLE


def locate(xa: np.ndarray, x) -> int:
    """interpolation_mod.f90:48-81 (1-based result)."""
    x = f32(x)
    n = len(xa)
    if x > xa[n - 1]:
        return n
    if x < xa[0]:
        return 0
    diff = xa - x
    mask = diff > 0
    if not mask.any():
        return 1  # minloc of an empty mask is 0 -> max(0 - 1, 1)
    idx = int(np.argmin(np.where(mask, diff, np.inf))) + 1
    return max(idx - 1, 1)


def axis_cell(xa: np.ndarray, x) -> int:
    """Cell of coordinate x: locate + half-cell step (grid_mod.f90:3590-3593)."""
    p = locate(xa, x)
    if p < len(xa):
        if f32(x) > (xa[p - 1] + xa[p]) / f32(2):
            p += 1
    return p


def make_axis(n: int, extent: float, symmetric: bool) -> np.ndarray:
    a = np.zeros(n, dtype=f32)
    for i in range(1, n + 1):
        if symmetric:
            v = f32(i - 1) / f32(n - 1)
        else:
            v = f32(2) * f32(i - 1) / f32(n - 1) - f32(1)
        a[i - 1] = v * f32(extent)
    return a


def wid_flx(nu: np.ndarray) -> np.ndarray:
    w = np.empty_like(nu)
    w[0] = nu[1] - nu[0]
    w[1:-1] = (nu[2:] - nu[:-2]) / f32(2)
    w[-1] = nu[-1] - nu[-2]
    return w


def blackbody_cdf(nu: np.ndarray, t_star: float) -> np.ndarray:
    """inSpectrumProbDen(iStar, :) of a blackbody (continuum_mod.f90:370-474)."""
    nbins = len(nu)
    const = f32(0.5250229) / f32(HPLANCK)
    flux = np.zeros(nbins, dtype=f32)
    for i in range(nbins):
        e = f32(nu[i])
        arg = f32(HCRYD_K) * e / f32(t_star)
        if arg > f32(86):
            flux[i] = f32(const * e * e * e * np.exp(-np.float64(arg)))
            continue
        den = f32(np.exp(arg) - f32(1))
        if den <= 0:
            flux[i] = f32(3.32154e-6) * e * e * f32(t_star) / f32(HPLANCK)
            continue
        flux[i] = const * e * e * e / den
    w = wid_flx(nu).astype(np.float64)
    s = flux.astype(np.float64)
    norm = float(np.sum(s * w))
    cdf = np.zeros(nbins, dtype=f32)
    cdf[0] = f32(s[0] * w[0] / norm)
    for i in range(1, nbins):
        cdf[i] = f32(np.float64(cdf[i - 1]) + s[i] * w[i] / norm)
    cdf[cdf >= cdf.max()] = f32(1)
    return cdf


def cdf_rows(weights: np.ndarray) -> np.ndarray:
    """Row-wise cumulative distribution, FP32, last entry forced to 1."""
    c = np.cumsum(weights, axis=1)
    tot = c[:, -1:]
    tot[tot <= 0] = 1.0
    c = (c / tot).astype(f32)
    c[:, -1] = f32(1)
    return c


def smooth_gaussian_periodic(field: np.ndarray, sigma: float) -> np.ndarray:
    """Separable periodic Gaussian filter (FFT), sigma in cells."""
    out = field.astype(np.float64)
    for ax in range(field.ndim):
        n = field.shape[ax]
        k = np.fft.rfftfreq(n)
        kern = np.exp(-2.0 * (np.pi * k * sigma) ** 2)
        shape = [1] * field.ndim
        shape[ax] = len(k)
        out = np.fft.irfft(np.fft.rfft(out, axis=ax) * kern.reshape(shape), n=n, axis=ax)
    return out


@dataclasses.dataclass
class Star:
    t_star: float           # K
    lum: float              # L [1e36 erg/s]
    frac_pos: tuple         # position as fractions of the axis maxima (starPosition input)
    n_packets: int


@dataclasses.dataclass
class NebulaSpec:
    name: str
    n: int                      # nx = ny = nz
    extent: float               # axis maximum [cm]
    symmetric: bool
    stars: List[Star]
    nh_median: float
    sigma_ln: float = 0.0       # lognormal width (0 = uniform)
    smooth_cells: float = 3.0
    seed: int = 1
    r_in: float = -1.0
    r_out: float = 0.0
    te: float = 10000.0
    ionisation: str = "start"   # "start" (H0 = 1e-5) | "stromgren"
    stromgren_radius: float = 0.5  # fraction of the extent (ionisation="stromgren")
    dust: bool = False
    isotropic: bool = True
    hg_g: float = 0.0           # constant HG asymmetry when not isotropic
    dust_to_gas: float = 0.01
    line_fraction: float = 0.6
    nbins_stride: int = 1       # keep every k-th bin of the 600-bin grid
    views: tuple = ()           # viewing angles ((theta, phi) rad, at most 2; phi < 0 = no phi)
    n_theta_bins: int = 0       # totAngleBinsTheta (0 = 10)
    n_phi_bins: int = 0         # totAngleBinsPhi (0 = 20)


@dataclasses.dataclass
class Nebula:
    spec: NebulaSpec
    nx: int
    ny: int
    nz: int
    ncells: int
    nbins: int
    x_axis: np.ndarray
    y_axis: np.ndarray
    z_axis: np.ndarray
    active: np.ndarray          # (nz, ny, nx) C-order == active(nx,ny,nz) Fortran
    hden: np.ndarray            # (Nc+1,)
    nu: np.ndarray
    xs: np.ndarray              # (nion, nbins)
    ion_den: np.ndarray         # (Nc+1, nion) ion number densities [cm^-3]
    opacity: np.ndarray         # (nbins, Nc+1) C-order == opacity(0:Nc,1:nbins)
    sca_opac: Optional[np.ndarray]
    dust_kappa: Optional[np.ndarray]   # (nbins,) per unit Ndust (abs + sca)
    ndust: Optional[np.ndarray]        # (Nc+1,)
    rec_pdf: np.ndarray
    total_lines: np.ndarray
    g_sca: Optional[np.ndarray]
    geo_corr: tuple
    r_out: float
    ion_edge1: float
    flags: int
    star_pos: list              # [(x,y,z)] FP32 cm
    star_cell: list             # [(xP,yP,zP)] 1-based
    spec_cdf: list              # [np.ndarray(nbins)]
    delta_e: list               # [deltaE] FP32
    n_packets: list


def _ion_fractions(spec: NebulaSpec, ions, r_node):
    """Fractional ion abundances per active node (nc, nion)."""
    nion = len(ions)
    frac = np.zeros((len(r_node), nion), dtype=np.float64)
    if spec.ionisation == "start":
        h0 = 1.0e-5
        for j, (z, st) in enumerate(ions):
            if z == 1:
                frac[:, j] = h0 if st == 1 else 0.0
            elif z == 2:
                frac[:, j] = h0 if st == 1 else (1.0 - h0 if st == 2 else 0.0)
            else:
                frac[:, j] = h0 if st == 1 else 0.0
        return frac
    # two-zone structure: ionised inside the Stromgren radius, neutral outside
    rs = spec.stromgren_radius * spec.extent
    inside = r_node < rs
    for j, (z, st) in enumerate(ions):
        if z == 1:
            frac[:, j] = np.where(inside, 1.0e-3, 0.9) if st == 1 else 0.0
        elif z == 2:
            frac[:, j] = np.where(inside, 1.0e-2, 0.9) if st == 1 else np.where(inside, 0.9, 0.1) if st == 2 else 0.0
        else:
            if st == 1:
                frac[:, j] = np.where(inside, 1.0e-3, 0.9)
            elif st == 2:
                frac[:, j] = np.where(inside, 0.6, 0.1)
            elif st == 3:
                frac[:, j] = np.where(inside, 0.4, 0.0)
    return frac


def _dust_kappa(nu: np.ndarray):
    """Per-grain-number opacity [cm^2] (abs, sca) of an MRN silicate-like mix:
    10 log-spaced sizes 0.005-0.25 um, n(a) ~ a^-3.5, smooth synthetic
    efficiencies Q_abs = 1 - exp(-x/2), Q_sca = 0.9 x^4 / (1 + x^4), x = 2 pi a / lambda."""
    a = np.logspace(np.log10(0.005e-4), np.log10(0.25e-4), 10)       # cm
    w = a ** -3.5 * np.gradient(a)
    w = w / w.sum()
    lam = 2.9979250e10 / (nu.astype(np.float64) * 3.28984e15)         # cm
    x = 2.0 * np.pi * a[None, :] / lam[:, None]
    qa = 1.0 - np.exp(-0.5 * x)
    qs = 0.9 * x ** 4 / (1.0 + x ** 4)
    geo = np.pi * a ** 2 * w
    mean_mass = float(np.sum(w * 4.0 / 3.0 * np.pi * a ** 3 * 3.5))   # g (3.5 g/cm^3)
    return (qa * geo).sum(1), (qs * geo).sum(1), mean_mass


def build(spec: NebulaSpec) -> Nebula:
    tab = atomic_table()
    nu = tab["nu"][:: spec.nbins_stride].astype(f32)
    xs = tab["xs"][:, :: spec.nbins_stride].astype(f32)
    ions = [tuple(int(v) for v in r) for r in tab["ions"]]
    edges = tab["edges"]
    nbins = len(nu)
    n = spec.n
    sym = spec.symmetric
    if not sym and n % 2 == 0:
        raise ValueError("a non-symmetric automatic grid needs odd n (grid_mod.f90:563-579)")
    xa = make_axis(n, spec.extent, sym)
    ya, za = xa.copy(), xa.copy()

    # density at nodes, indexed [i, j, k] (x, y, z)
    if spec.sigma_ln > 0:
        rng = np.random.default_rng(spec.seed)
        g = rng.standard_normal((n, n, n))
        g = smooth_gaussian_periodic(g, spec.smooth_cells)
        g = (g - g.mean()) / g.std()
        nh = spec.nh_median * np.exp(spec.sigma_ln * g)
    else:
        nh = np.full((n, n, n), spec.nh_median)
    nh = nh.astype(f32)

    # active numbering: i (x) outer, j, k (z) inner (grid_mod.f90:1224-1290)
    xi, yj, zk = np.meshgrid(xa, ya, za, indexing="ij")
    e10 = f32(1e10)
    radius = e10 * np.sqrt((xi / e10) * (xi / e10) + (yj / e10) * (yj / e10) + (zk / e10) * (zk / e10))
    ok = np.ones((n, n, n), dtype=bool)
    ok &= ~(radius < f32(spec.r_in))
    if spec.r_out > 0:
        ok &= ~(radius > f32(spec.r_out))
    ok &= nh > 0
    act_ijk = np.zeros((n, n, n), dtype=np.int32)
    flat = ok.reshape(-1)                       # C order over (i, j, k): k fastest
    act_ijk.reshape(-1)[flat] = np.arange(1, int(flat.sum()) + 1, dtype=np.int32)
    nc = int(flat.sum())
    active = np.ascontiguousarray(act_ijk.transpose(2, 1, 0))  # (z, y, x): x fastest in memory

    cells_ijk = np.argwhere(ok)                 # ordered by cell number
    hden = np.zeros(nc + 1, dtype=f32)
    hden[1:] = nh[ok]
    r_node = radius[ok].astype(np.float64)

    frac = _ion_fractions(spec, ions, r_node)
    ab = np.array([ABUNDANCES[z] for (z, st) in ions])
    ion_den = np.zeros((nc + 1, len(ions)), dtype=f32)
    ion_den[1:] = (frac * ab[None, :] * hden[1:, None].astype(np.float64)).astype(f32)

    # bound-free opacity: den @ XS (FP64 sum, stored FP32 like `real`)
    opac = ion_den.astype(np.float64) @ xs.astype(np.float64)       # (Nc+1, nbins)
    flags = FLAG_GAS
    sca = None
    dk = None
    ndust = None
    gsca = None
    if spec.dust:
        flags |= FLAG_DUST
        ka, ks, mass = _dust_kappa(nu)
        ndust = np.zeros(nc + 1, dtype=f32)
        ndust[1:] = (spec.dust_to_gas * 1.4 * 1.6726e-24 * hden[1:].astype(np.float64) / mass).astype(f32)
        dk = (ka + ks).astype(f32)
        sca_d = ndust[:, None].astype(np.float64) * ks[None, :]
        opac = opac + ndust[:, None].astype(np.float64) * (ka + ks)[None, :]
        sca = np.ascontiguousarray(sca_d.T.astype(f32))
        if spec.isotropic:
            flags |= FLAG_ISOTROPIC
        else:
            gsca = np.full(nbins, spec.hg_g, dtype=f32)
    opacity = np.ascontiguousarray(opac.T.astype(f32))               # (nbins, Nc+1)

    # synthetic emission CDFs (recPDF rows for cells 1..Nc; row 0 unused)
    te = spec.te
    wf = wid_flx(nu).astype(np.float64)
    nu64 = nu.astype(np.float64)
    thr = np.array([nu64[np.argmax(xs[j] > 0)] if (xs[j] > 0).any() else np.inf for j in range(len(ions))])
    up = np.zeros_like(frac)
    # recombining stage of ion j is stage j+1 of the same element
    for j, (z, st) in enumerate(ions):
        nxt = [k for k, (z2, st2) in enumerate(ions) if z2 == z and st2 == st + 1]
        up[:, j] = (frac[:, nxt[0]] if nxt else (1.0 - frac[:, j])) * ab[j]
    milne = (nu64[None, :] ** 3 * xs.astype(np.float64) / 6.3e-18 *
             np.exp(-HCRYD_K * np.clip(nu64[None, :] - thr[:, None], 0, None) / te))   # (nion, nbins)
    rec = up @ milne                                                                   # (nc, nbins)
    ff = 0.5 * np.exp(-HCRYD_K * nu64 / te)
    w_gas = (rec + ff[None, :]) * wf[None, :]
    if spec.dust:
        bnu = nu64 ** 3 / np.expm1(np.clip(HCRYD_K * nu64 / 60.0, 1e-30, 700))
        w_d = (ka * bnu * wf)[None, :]
        w_gas = w_gas / w_gas.sum(1, keepdims=True) + w_d / w_d.sum()
    rec_rows = np.zeros((nc + 1, nbins), dtype=f32)
    rec_rows[1:] = cdf_rows(w_gas)
    rec_rows[0] = f32(1)
    rec_pdf = np.ascontiguousarray(rec_rows.T)                                         # (nbins, Nc+1)
    total_lines = np.full(nc + 1, f32(spec.line_fraction), dtype=f32)
    total_lines[0] = f32(0)

    geo = (f32((xa[-1] - xa[-2]) / f32(2)), f32((ya[-1] - ya[-2]) / f32(2)), f32((za[-1] - za[-2]) / f32(2)))
    star_pos, star_cell, cdfs, des, nps = [], [], [], [], []
    for st in spec.stars:
        p = (f32(st.frac_pos[0]) * xa[-1], f32(st.frac_pos[1]) * ya[-1], f32(st.frac_pos[2]) * za[-1])
        c = (axis_cell(xa, p[0]), axis_cell(ya, p[1]), axis_cell(za, p[2]))
        star_pos.append(p)
        star_cell.append(c)
        cdfs.append(blackbody_cdf(nu, st.t_star))
        des.append(f32(f32(st.lum) / f32(st.n_packets)))
        nps.append(int(st.n_packets))
    if len(spec.stars) > 1:
        flags |= FLAG_MULTISTARS
    if sym:
        flags |= FLAG_SYMMETRIC_XYZ
    return Nebula(spec=spec, nx=n, ny=n, nz=n, ncells=nc, nbins=nbins, x_axis=xa, y_axis=ya, z_axis=za,
                  active=active, hden=hden, nu=nu, xs=xs, ion_den=ion_den, opacity=opacity, sca_opac=sca,
                  dust_kappa=dk, ndust=ndust, rec_pdf=rec_pdf, total_lines=total_lines, g_sca=gsca,
                  geo_corr=geo, r_out=float(f32(spec.r_out)), ion_edge1=float(edges[0]), flags=flags,
                  star_pos=star_pos, star_cell=star_cell, spec_cdf=cdfs, delta_e=des, n_packets=nps)


# ---- the workloads -------------------------------------------------------

def octant21(n_packets: int = 1_000_000) -> NebulaSpec:
    """One-octant 21^3 grid over 0..3e18 cm, nH = 100, 40 kK star of 1e37 erg/s."""
    return NebulaSpec("octant21_uniform", 21, 3.0e18, True, [Star(40000.0, 10.0, (0, 0, 0), n_packets)],
                      nh_median=100.0, r_in=0.0)


def clumpy61(n_packets: int = 20_000_000) -> NebulaSpec:
    """Full 61^3 grid over +/-5e18 cm, lognormal nH (median 300, sigma_ln 1,
    3-cell Gaussian correlation, seed 1), 60 kK star of 5e37 erg/s."""
    return NebulaSpec("clumpy61_lognormal", 61, 5.0e18, False, [Star(60000.0, 50.0, (0, 0, 0), n_packets)],
                      nh_median=300.0, sigma_ln=1.0, smooth_cells=3.0, seed=1)


def dusty81(n_packets: int = 50_000_000) -> NebulaSpec:
    """Full 81^3 grid over +/-5e18 cm, uniform nH = 1e3, MRN dust at a
    dust-to-gas mass ratio of 0.01 with isotropic scattering, 60 kK star of 5e37 erg/s."""
    return NebulaSpec("dusty81_uniform", 81, 5.0e18, False, [Star(60000.0, 50.0, (0, 0, 0), n_packets)],
                      nh_median=1000.0, dust=True, isotropic=True)


def twostar101(n_packets: int = 100_000_000) -> NebulaSpec:
    """Full 101^3 grid over +/-5e18 cm, lognormal nH (median 1e3), stars of
    50 kK and 80 kK (1e37 erg/s each) at x = -/+1e18 cm."""
    half = n_packets // 2
    return NebulaSpec("twostar101_lognormal", 101, 5.0e18, False,
                      [Star(50000.0, 10.0, (-0.2, 0, 0), half), Star(80000.0, 10.0, (0.2, 0, 0), n_packets - half)],
                      nh_median=1000.0, sigma_ln=1.0, smooth_cells=3.0, seed=1)


def batch64(n_models: int = 64, seed: int = 1, packets_total: int = 200_000_000, n_min: int = 17,
            n_max: int = 65) -> List[NebulaSpec]:
    """Independent nebulae for batched serving: grid sizes odd and uniform in
    n_min..n_max, star temperatures uniform in 30-100 kK, log nH uniform in
    [1, 4], outer radius uniform in 1e18-1e19 cm (the grid spans +/- the
    outer radius), the abundances of the other workloads, packets in
    proportion to the cell count (packets_total over all models)."""
    rng = np.random.default_rng(seed)
    ns = rng.choice(np.arange(n_min, n_max + 1, 2), n_models)
    tstar = rng.uniform(30000.0, 100000.0, n_models)
    lognh = rng.uniform(1.0, 4.0, n_models)
    rout = rng.uniform(1.0e18, 1.0e19, n_models)
    cells = ns.astype(np.float64) ** 3 * (np.pi / 6.0)   # the sphere inside the cube
    npk = np.maximum((packets_total * cells / cells.sum()).astype(np.int64), 1000)
    specs = []
    for i in range(n_models):
        specs.append(NebulaSpec("batch%02d_n%d" % (i, ns[i]), int(ns[i]), float(rout[i]), False,
                                [Star(float(tstar[i]), 10.0, (0, 0, 0), int(npk[i]))],
                                nh_median=float(10.0 ** lognh[i]), r_out=float(rout[i]), r_in=0.0))
    return specs


def small_cases():
    """Small grids the oracle finishes in seconds: every branch of the march."""
    return [
        NebulaSpec("sym9_start", 9, 3.0e18, True, [Star(40000.0, 10.0, (0, 0, 0), 4000)], nh_median=100.0, r_in=0.0),
        NebulaSpec("sym11_stromgren", 11, 3.0e18, True, [Star(40000.0, 10.0, (0, 0, 0), 3000)], nh_median=300.0,
                   r_in=0.0, ionisation="stromgren", stromgren_radius=0.45),
        NebulaSpec("full9_lognormal_rout", 9, 5.0e18, False, [Star(60000.0, 50.0, (0, 0, 0), 3000)],
                   nh_median=300.0, sigma_ln=1.0, smooth_cells=1.5, r_out=4.6e18, r_in=1.0e18,
                   ionisation="stromgren", stromgren_radius=0.6),
        NebulaSpec("full11_dust_iso", 11, 5.0e18, False, [Star(60000.0, 50.0, (0, 0, 0), 2000)],
                   nh_median=1000.0, dust=True, isotropic=True, ionisation="stromgren", stromgren_radius=0.5),
        NebulaSpec("full9_dust_hg", 9, 5.0e18, False, [Star(60000.0, 50.0, (0, 0, 0), 2000)],
                   nh_median=1000.0, dust=True, isotropic=False, hg_g=0.6, ionisation="stromgren",
                   stromgren_radius=0.5),
        NebulaSpec("full9_twostar", 9, 5.0e18, False,
                   [Star(50000.0, 10.0, (-0.3, 0.1, 0), 1500), Star(80000.0, 10.0, (0.3, 0, -0.1), 1500)],
                   nh_median=300.0, ionisation="stromgren", stromgren_radius=0.7),
    ]
