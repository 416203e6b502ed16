"""CPU oracle of the diffuse-emission CDF (test infrastructure only): the
recPDF row and totalLines of every cell from its Te, Ne and ionic fractions,
restating emissionDriver / fb_ff / twoPhoton / RecLinesEmission / forLines /
setDiffusePDF (source/emission_mod.f90:32-1311) for a gas-only grid, in FP64,
vectorised over cells.  Each step follows the reference loop it cites;
inputs are the committed emission tables (data/emission_tables.npz, written
from the reference's data files by make_emission_tables.py), the frequency
grid and the cross-section matrix of atomic_table.npz, and the forbidden-line
totals of update_oracle.cpp (oracle_forbidden_lines).

Deviations, stated once:
* gauntFF is evaluated at every cell's own Te.  The reference recomputes it
  in BoltGaunt (ionization_mod.f90:165-172) only when Te moved by more than
  10 % from the Te it was last computed at, so its value depends on the
  order cells are visited in.
* The HI, HeI-singlet and HeII ground-state cross-sections of the Milne
  relation are the H0, He0 and He+ rows of the cross-section matrix (Verner
  fits), not mocassin's hydrogenic xSecArray entries.
* A row whose emission sums to zero is written as a step at the first bin
  (the reference divides by zero there).
"""
import os

import numpy as np

from mocassin_gb300 import balance, nebula
from oracle import update_runner

HCRYD_K = 157893.94
HCRYD = 2.1799153e-11
CRYD = 3.2898423e15
HPLANCK = 6.6262e-27
PI = 3.141592654
FOURPI = 4.0 * PI
HIONPOT = 0.99946


def tables():
    d = np.load(os.path.join(os.path.dirname(nebula.__file__), "data", "emission_tables.npz"))
    return {k: d[k] for k in d.files}


def locate(xa, x):
    """locate (interpolation_mod.f90:48-81), 1-based."""
    return nebula.locate(xa, x)


def edge_pointers(nu, nu_gamma):
    """HINuEdgeP & co. (initGammaCont, ph_mod.f90:135-197), 1-based."""
    nb = len(nu)
    p = np.zeros(len(nu_gamma), dtype=np.int64)
    for i, v in enumerate(nu_gamma):
        k = locate(nu, v)
        if k < nb and np.float32(v) > (nu[k - 1] + nu[k]) / np.float32(2):
            k += 1
        p[i] = k
    p[0] = 1
    return p


def gaunt(z_log, log10te, log10nu, dd):
    """getGauntFF (ionization_mod.f90:193-330) for one Te and all bins."""
    d = dd.reshape(11, 8).T  # d(8, 11), column-major reshape of dd(88)
    if log10te < 2.5:
        xlrkt = 5.1983649 - 2.5
    elif log10te > 8.0:
        xlrkt = 5.1983649 - 8.0
    else:
        xlrkt = 5.1983649 - log10te
    txg = 0.66666667 * (2.0 * z_log + xlrkt)
    gamma2 = 10 ** (txg * 1.5)
    con = 0.72727273 * xlrkt + 0.90909091
    c = np.zeros(8)
    for j in range(8):
        b = np.zeros(13)
        b[11] = d[j, 10]
        b[10] = txg * b[11] + d[j, 9]
        for ir in range(9, 0, -1):
            b[ir] = txg * b[ir + 1] - b[ir + 2] + d[j, ir - 1]
        c[j] = 0.25 * (b[1] - b[3])
    xlf = np.asarray(log10nu, dtype=np.float64)
    txu = 0.72727273 * xlf + con
    u = 10 ** ((txu - 0.90909091) / 0.72727273)
    bb = np.zeros((10, len(xlf)))
    bb[8] = c[7]
    bb[7] = txu * bb[8] + c[6]
    for ir in range(6, 0, -1):
        bb[ir] = txu * bb[ir + 1] - bb[ir + 2] + c[ir - 1]
    g = np.zeros(len(xlf))
    lu = np.log10(u)
    cheb = np.abs(txu) <= 2.0
    low = ~cheb & (lu < -4.0)
    high = ~cheb & ~low & (txu > 2.0)
    g[cheb] = (bb[1] - bb[3])[cheb]
    if gamma2 < 0.3:
        g[low] = 0.551329 * np.log(2.24593 / u[low])
    else:
        g[low] = 0.551329 * np.log(0.944931 / u[low] / np.sqrt(gamma2))
    if np.log10(gamma2) < -3.0:
        g[high] = np.sqrt(0.9549297 / u[high])
    elif np.log10(gamma2) < 0.0:
        slope = (np.sqrt(12 * gamma2 / u[high]) - np.sqrt(0.9549297 / u[high])) / 3.0
        g[high] = np.sqrt(12 * gamma2 / u[high]) + slope * np.log10(gamma2)
    else:
        g[high] = np.minimum(1.05, np.sqrt(12.0 * gamma2 / u[high]))
    return g


def two_photon_ay(y):
    """Nussbaumer & Schmutz (1984) two-photon distribution A(y) of hydrogen
    [1/s] (hydro2phot, emission_mod.f90:595-596)."""
    q = 4 * y * (1 - y)
    return 202.0 * (y * (1 - y) * (1 - q ** 0.8) + 0.88 * ((y * (1 - y)) ** 1.53) * q ** 0.8)


def planck_over_h(nu, t):
    """getFlux(energy, T, 'blackbody') (continuum_mod.f90:359-394), FP64,
    for a frequency vector at one temperature."""
    constant = 0.5250229 / HPLANCK
    u = HCRYD_K * nu / t
    out = np.empty_like(u)
    big = u > 86.0
    out[big] = constant * nu[big] ** 3 * np.exp(-u[big])
    den = np.expm1(u[~big])
    rj = den <= 0
    out[~big] = np.where(rj, 3.32154e-6 * nu[~big] ** 2 * t / HPLANCK, constant * nu[~big] ** 3 / np.where(rj, 1, den))
    return out


def grain_emission(tdust, xs_abs, gw, t_sub, nu, positive):
    """sum over size bins of xSecAbs B(nu, Tdust) widFlx grainWeight grainAbun
    [n][nbins] (sumDiffuseDust, emission_mod.f90:1042-1105; setDustPDF
    :1329-1367 also requires Tdust > 0)."""
    nu64 = nu.astype(np.float64)
    wid = nebula.wid_flx(nu).astype(np.float64)
    out = np.zeros((len(tdust), len(nu)))
    for c in range(len(tdust)):
        for a in range(xs_abs.shape[0]):
            t = float(tdust[c][a])
            if t < t_sub and (t > 0 or not positive):
                if t <= 0:
                    continue  # the Planck function of 0 K is 0
                out[c] += xs_abs[a].astype(np.float64) * planck_over_h(nu64, t) * wid * gw[a]
    return out


def dust_pdf(tdust, xs_abs, gw, t_sub, nu=None):
    """dustPDF rows [n][nbins] of a dust-only grid (setDustPDF, :1313-1387)."""
    nu = nebula.atomic_table()["nu"] if nu is None else nu
    s = grain_emission(tdust, xs_abs, gw, t_sub, nu, True)
    cdf = np.cumsum(s, axis=1)
    last = cdf[:, -1].copy()
    ok = last > 0
    cdf[ok] = cdf[ok] / last[ok, None]
    cdf[~ok] = 1.0
    cdf[:, -1] = 1.0
    return cdf


def diffuse_pdf(te, ne, X, abund, forb, T=None, nu=None, xs=None, ions=None, dust=None):
    """recPDF rows [n][nbins] (cumulative, normalised) and totalLines [n] of
    n cells: te, ne [n], X [n][7][8] (elements H He C N O Ne S, stage 1..7),
    abund [7], forb [n][ncel] from update_runner.forbidden_lines.  dust: None
    or a dict with tdust [n][nsizes], xs_abs [nsizes][nbins], gw [nsizes],
    t_sub and ndust_over_hden [n] for the thermal grain emission."""
    T = tables() if T is None else T
    at = nebula.atomic_table()
    nu = at["nu"] if nu is None else nu
    xs = at["xs"] if xs is None else xs
    ions = [tuple(int(v) for v in r) for r in at["ions"]] if ions is None else ions
    nb = len(nu)
    nu64 = nu.astype(np.float64)
    wid = nebula.wid_flx(nu).astype(np.float64)
    te = np.asarray(te, dtype=np.float64)
    ne = np.maximum(np.asarray(ne, dtype=np.float64), 1e-5)   # emissionDriver :86-88
    n = len(te)
    sq = np.sqrt(te)
    log10te = np.log10(te)
    abH, abHe = abund[0], abund[1]
    xH2, xHe2, xHe3 = X[:, 0, 2], X[:, 1, 2], X[:, 1, 3]
    tk = T["tk"].astype(np.float64)

    def gamma_series(lg, nu_g):
        """below-limit gammas (fb_ff :311-410): Te interpolation in log-log,
        then linear in nu between the edge pairs, 10**."""
        ep = edge_pointers(nu, nu_g)
        out = np.zeros((n, nb))
        for c in range(n):
            t = te[c]
            if t <= tk[0]:
                loc = lg[0].astype(np.float64)
            elif t >= tk[-1]:
                loc = lg[-1].astype(np.float64)
            else:
                k = locate(T["tk"], t) - 1
                fac = np.log10(t / tk[k])
                afit = (lg[k + 1].astype(np.float64) - lg[k]) / np.log10(tk[k + 1] / tk[k])
                loc = lg[k] + afit * fac
            for i in range(len(nu_g) // 2):
                iup, ilow = ep[2 * i + 1], ep[2 * i]
                afit = (loc[2 * i + 1] - loc[2 * i]) / (nu64[iup - 1] - nu64[ilow - 1])
                j = np.arange(ilow, iup)
                out[c, j - 1] = 10.0 ** (loc[2 * i + 1] + afit * (nu64[j - 1] - nu64[iup - 1]))
        return out, ep

    gHI, epHI = gamma_series(T["lg_hi"], T["nu_gamma_hi"])
    gHeI, epHeI = gamma_series(T["lg_hei"], T["nu_gamma_hei"])
    gHeII, epHeII = gamma_series(T["lg_heii"], T["nu_gamma_heii"])

    # free-free coefficients (free_free / ffCoeff, :709-742)
    lnu = np.log10(nu).astype(np.float64)
    ff1 = np.zeros((n, nb))
    ff2 = np.zeros((n, nb))
    for c in range(n):
        e = np.exp(-nu64 * HCRYD_K / te[c])
        ff1[c] = FOURPI * 54.43 * gaunt(0.0, log10te[c], lnu, T["gaunt_dd"]) * e / sq[c]
        ff2[c] = FOURPI * 54.43 * 4.0 * gaunt(0.30103, log10te[c], lnu, T["gaunt_dd"]) * e / sq[c]

    # Milne relation above the series limits (:429-470)
    constant = 4.9874105e-6
    ix = {ion: k for k, ion in enumerate(ions)}
    xsH, xsHeI, xsHeII = xs[ix[(1, 1)]].astype(np.float64), xs[ix[(2, 1)]].astype(np.float64), \
        xs[ix[(2, 2)]].astype(np.float64)
    pH, pHeI, pHeII = locate(nu, HIONPOT), locate(nu, 1.80802), locate(nu, 4.0)
    heI_from, heII_from = epHeI[-1], epHeII[-1]
    stat = (2.0, 0.5, 2.0)
    for i in range(pH, nb + 1):
        fac = nu64[i - 1] ** 3 / (te * sq)
        k = i - 1
        gHI[:, k] = FOURPI * xsH[k] * stat[0] * HCRYD * constant * fac * \
            np.exp((-nu64[k] + nu64[pH - 1]) * HCRYD_K / te) * 1e40 + ff1[:, k]
        if i >= heI_from:
            gHeI[:, k] = FOURPI * xsHeI[k] * stat[1] * HCRYD * constant * fac * \
                np.exp((-nu64[k] + nu64[pHeI - 1]) * HCRYD_K / te) * 1e40 + ff1[:, k]
            if i >= heII_from:
                gHeII[:, k] = FOURPI * xsHeII[k] * stat[2] * HCRYD * constant * fac * \
                    np.exp((-nu64[k] + nu64[pHeII - 1]) * HCRYD_K / te) * 1e40 + ff2[:, k]

    # heavy-ion recombination continua (:473-527)
    gHeavy = np.zeros((n, nb))
    elem_index = {z: e for e, z in enumerate(balance.ELEMENTS)}
    for row, xso in zip(T["shells"], T["xs_outer"]):
        z, ion, _ne, _out, g0, g1, ip, hi = (int(v) for v in row)
        e = elem_index[z]
        w = (g0 / g1) * X[:, e, ion + 1] * abund[e]
        for i in range(ip, hi):
            k = i - 1
            gHeavy[:, k] += np.exp((-nu64[k] + nu64[ip - 1]) * HCRYD_K / te) * xso[k] * w
    gHeavy *= FOURPI * constant * HCRYD * (nu64[None, :] ** 3 / (te * sq)[:, None]) * 1e40

    # two-photon continua (twoPhoton / hydro2phot / HeI2photSub, :533-705)
    t4 = te * 1e-4

    ay_h = two_photon_ay

    tpHI = np.zeros((n, nb))
    tpHeII = np.zeros((n, nb))
    y = nu64 / 0.7496
    m = nu64 < 0.7496
    gnu = np.where(m, HPLANCK * y * ay_h(np.where(m, y, 0.5)) / 8.2249 * 1e27, 0.0)
    alpha = 0.8368 * t4 ** -0.723
    q = np.where(te <= 1e4, 5.31e-4, np.where(te >= 2e4, 4.71e-4,
                 10 ** (np.log10(5.31e-4) + np.log10(4.71e-4 / 5.31e-4) / np.log10(2.0) * np.log10(te / 1e4))))
    tpHI[:] = (alpha / (1.0 + ne * q / 8.23))[:, None] * gnu[None, :]
    y = nu64 / 3.0
    m = nu64 < 3.0
    gnu = np.where(m, HPLANCK * y * (64 * 0.9994667 * ay_h(np.where(m, y, 0.5))) / (8.226 * 64) * 1e27, 0.0)
    aHe = np.where(te <= 5000, 6.161, np.where(te >= 30000, 2.035, np.where(
        te <= 1e4, 10 ** (np.log10(6.161) + np.log10(4.091 / 6.161) / np.log10(2.0) * np.log10(te / 5000)),
        np.where(te <= 1.5e4, 10 ** (np.log10(4.091) + np.log10(3.189 / 4.091) / np.log10(1.5) * np.log10(te / 1e4)),
                 10 ** (np.log10(3.189) + np.log10(2.035 / 3.189) / np.log10(2.0) * np.log10(te / 1.5e4))))))
    tpHeII[:] = aHe[:, None] * gnu[None, :]
    ydat, aydat = T["y_ay"][:, 0].astype(np.float64), T["y_ay"][:, 1].astype(np.float64)
    tpHeI_bin = np.zeros(nb)
    j = 0
    for i in range(nb):
        yy = nu64[i] / 1.514
        if yy > ydat[j]:
            j += 1
        if j >= 40:
            break
        fit1 = (aydat[j + 1] - aydat[j]) / (ydat[j + 1] - ydat[j])
        fit2 = aydat[j] - ydat[j] * fit1
        ay = fit1 * yy + fit2
        if ay < 9.2163086e-03:
            ay = 0.0
        tpHeI_bin[i] = ay * 0.66262 * yy / 51.3
    tpHeI = (6.23 * t4 ** -0.827)[:, None] * tpHeI_bin[None, :]

    # total continuum emission (emissionDriver :116-128)
    eHI = (gHI + tpHI) * (abH * xH2 * ne)[:, None] + gHeavy * ne[:, None]
    eHeI = (gHeI + tpHeI) * (abHe * xHe2 * ne)[:, None]
    eHeII = (gHeII + tpHeII) * (abHe * xHe3 * ne)[:, None]
    for a in (eHI, eHeI, eHeII):
        a[a < 1e-15] = 0.0
    sHI = CRYD * wid[None, :] * eHI / 1e15
    sHeI = CRYD * wid[None, :] * eHeI / 1e15
    sHeII = CRYD * wid[None, :] * eHeII / 1e15

    # HeI 2^3S line (:996-1014) and HeII Lyman lines (:1016-1039)
    j2 = locate(nu, 1.45673)
    corr = 27.2 * t4 ** -0.678 * ne * abHe * xHe2 * 1.45673 * HCRYD * 1e11
    sHeI[:, j2 - 1] += corr
    lyd, lynu = T["heii_lyman"][:, 0].astype(np.float64), T["heii_lyman"][:, 1]
    lya = 10.0 ** (-0.792 * log10te + 6.01) * ne * xHe3 * abHe
    for i in range(4):
        val = lya if i == 3 else lyd[i] * lya
        sHeII[:, locate(nu, lynu[i]) - 1] += val
    sDust = np.zeros_like(sHI)
    if dust is not None:
        const = HPLANCK * 4.0 * PI * 1e25 * CRYD   # :1097-1100
        sDust = grain_emission(dust["tdust"], dust["xs_abs"], dust["gw"], dust["t_sub"], nu, False) * \
            (const * np.asarray(dust["ndust_over_hden"], dtype=np.float64))[:, None]
    normalize = sHI.sum(1) + sHeI.sum(1) + sHeII.sum(1) + sDust.sum(1)

    # recombination lines (RecLinesEmission :744-832) and normRec (:1122-1139)
    hbeta = 10 ** (-0.870 * log10te + 3.57) * ne * xH2 * abH
    lalpha = 10 ** (-0.897 * log10te + 5.05)
    norm_rec = hbeta * float(T["hi_rec"].astype(np.float64).sum()) + abH * xH2 * ne * lalpha
    h4686 = 10.0 ** (-0.997 * log10te + 5.16) * ne * abHe * xHe3
    norm_rec += h4686 * float(T["heii_rec"].astype(np.float64).sum())
    co = T["hei_rec"].astype(np.float64)
    ne_grid = np.asarray(ne)  # the density bracket reads the cell's Ne (>= 1e-5 makes no difference)
    hei = np.zeros(n)
    for c in range(n):
        nn = ne_grid[c]
        den = 0 if nn <= 100 else (1 if nn <= 1e4 else (2 if nn <= 1e6 else 3))
        t = t4[c]

        def fit(k):
            return co[:, k, 0] * t ** co[:, k, 1] * np.exp(co[:, k, 2] / t)
        if den in (1, 2):
            x1, x2 = fit(den - 1), fit(den)
            lines = x1 + (x2 - x1) * (nn - 100.0 ** den) / (100.0 ** (den + 1) - 100.0 ** den)
        elif den == 0:
            lines = fit(0)
        else:
            lines = fit(2)
        hei[c] = lines.sum() * nn * abHe * xHe2[c]
    norm_rec += hei
    norm_for = np.asarray(forb, dtype=np.float64).sum(1)
    total = norm_rec + norm_for

    # the CDF (:1177-1212) and the line fraction (:1302-1304)
    s = sHI + sHeI + sHeII + sDust
    cdf = np.cumsum(s, axis=1)
    last = cdf[:, -1].copy()
    ok = last > 0
    cdf[ok] = cdf[ok] / last[ok, None]
    cdf[~ok] = 1.0
    cdf[:, -1] = 1.0
    cdf[cdf > 0.999998] = 1.0
    tl = total / (normalize + total)
    return cdf, tl


def for_cells(te, ne, X, abund, tables_upd=None):
    """diffuse_pdf with the forbidden-line totals from the update oracle."""
    tu = balance.tables() if tables_upd is None else tables_upd
    forb = update_runner.forbidden_lines(tu, abund, te, ne, X)
    return diffuse_pdf(te, ne, X, abund, forb)
