"""Astrometric log-likelihood of a joint RV + astrometry fit (oracle; TEST
INFRASTRUCTURE ONLY).

FP64 numpy restatement of the functions the reference's generated script
defines for its astrometry blocks (written by ``ReddModel._write_model_AM``,
``src/astroemperor/emp_model.py:1232-1675``, with the constants and helpers
of ``support/astrometry/constants.scr``) and of ``support/likelihoods/a00.like``:

* ``calc_astro_new`` (emp_model.py:1309-1370): one Keplerian's sky-plane
  offsets at every IAD epoch from (P, K, phase, e, w, I, Omega) and the
  parallax (Thiele-Innes constants, emp_model.py:1256-1273);
* ``model_barycenter`` / ``obs_lin_prop_PA`` (emp_model.py:1473-1550): the
  barycentre's astrometry at each catalogue epoch from the DR3 solution
  minus the five offsets, propagated linearly in Cartesian space;
* ``compute_abs_signal_hipp`` / ``compute_abs_signal_gost`` with
  ``get_deltas_HIPP`` / ``get_deltas_GOST`` and ``obs_lin_prop_simple``
  (emp_model.py:1394-1470, 1553-1570): the along-scan abscissae;
* ``loglike_AM`` (emp_model.py:1622-1658): Hipparcos residuals with iid
  Gaussian errors and jitter, and for each Gaia release the five-parameter
  fit of the GOST abscissae against the catalogue solution with its
  covariance scaled by the jitter squared.

The reference converts mas to degrees in ``np.longdouble`` (``mas2deg``:
80-bit on x86) and does everything else in FP64; ``dtype=np.float64`` (the
default) follows it, and the fixture ``tests/golden/am_kat.npz`` holds the
reference's own functions executed on the same data, which the restatement
equals to ~1e-12.  The formulas handle absolute positions in degrees (~60
degrees for HIP 21850), so their FP64 rounding is 7e-15 degrees = 2.5e-8
mas per ulp, and one ulp of the Gaia DR3-epoch position moves the Gaia term
of HIP 21850 by up to 2.8e-9 of the total log-likelihood.
``dtype=np.longdouble`` evaluates the barycentre and the Gaia scan-epoch
propagation (the parts that handle absolute positions) in extended
precision: the value of the reference's formulas without that rounding
noise, against which both FP64 evaluations (the reference's and the
device's) are measured.
"""
from __future__ import annotations

import numpy as np

LOG_2PI = np.log(2 * np.pi)
MAS_PER_DEG = 3.6e6
PC_PER_KPC = 1e3
DAY_PER_YEAR = 365.25
PC2AU = 206265.0
AUYR2KMS = 4.74047


def kepler_E(M, e):
    """E - e sin E = M (FP64 Halley, as the RV oracle's solver)."""
    from .rv import kepler_solve
    return kepler_solve(M, np.repeat(e, len(M)))


def thiele_innes(omega, Omega, sinI, cosI):
    sO, cO = np.sin(Omega), np.cos(Omega)
    so, co = np.sin(omega), np.cos(omega)
    A = co * cO - so * sO * cosI
    B = co * sO + so * cO * cosI
    F = -so * cO - co * sO * cosI
    G = -so * sO + co * cO * cosI
    C = so * sinI
    H = co * sinI
    return A, B, F, G, C, H


def calc_astro(theta7, plx, t_iad, common_t):
    """rows rasP, decP, plxP (mas) of one planet at the IAD epochs."""
    per, K, pha, ecc, omega, I, Om = theta7
    sinI, cosI = np.sin(I), np.cos(I)
    sq = np.sqrt(1 - ecc ** 2)
    M = 2. * np.pi / per * (t_iad - common_t) + pha
    E = kepler_E(M, ecc)
    A, B, F, G, C, H = thiele_innes(omega, Om, sinI, cosI)
    X = np.cos(E) - ecc
    Y = sq * np.sin(E)
    beta0 = per / DAY_PER_YEAR * (K / PC_PER_KPC / AUYR2KMS) * sq / (2 * np.pi) / sinI
    beta = -beta0 * plx
    ras = beta * (B * X + G * Y)
    dec = beta * (A * X + F * Y)
    plxP = -beta * (C * X + H * Y) * plx / 206265e3
    return np.array([ras, dec, plxP])


def _xyz2bl(x, y, z):
    b = np.arctan2(z, np.sqrt(x ** 2 + y ** 2))
    b = np.where(b > np.pi / 2, b - np.pi, b)
    l = np.arctan2(y, x) % (2 * np.pi)
    return b, l


def barycenter(am, off5, dtype=np.float64):
    """[3 catalogues, 6]: ra, dec (deg), parallax, pmra, pmdec (mas, mas/yr),
    rv of the barycentre at each catalogue epoch (model_barycenter)."""
    cat = np.asarray(am['catalogs'], dtype=dtype)
    ref = cat[-1, 1:]                                    # DR3 solution (AM_iref_ = -1)
    t_refed = cat[:, 0] - cat[-1, 0]
    th = np.array(off5, dtype=dtype)
    th0 = np.empty(6, dtype=dtype)
    th0[0] = th[0] / MAS_PER_DEG / np.cos(np.deg2rad(ref[1]))
    th0[1] = th[1] / MAS_PER_DEG
    th0[2:5] = th[2:5]
    th0[5] = 0.0
    RA, DE, PLX, PMRA, PMDE, RV = ref - th0
    ra, de = np.deg2rad(RA), np.deg2rad(DE)
    cosde, sinde = np.cos(de), np.sin(de)
    cosra, sinra = np.cos(ra), np.sin(ra)
    d = 1 / PLX
    x, y, z = np.array([cosde * cosra, cosde * sinra, sinde]) * d * PC_PER_KPC
    vra, vde = PMRA * d, PMDE * d
    vr = RV / AUYR2KMS
    vx = vr * cosde * cosra - vde * sinde * cosra - vra * sinra
    vy = vr * cosde * sinra - vde * sinde * sinra + vra * cosra
    vz = vr * sinde + vde * cosde
    tf = t_refed / (DAY_PER_YEAR * PC2AU)
    x1, y1, z1 = x + vx * tf, y + vy * tf, z + vz * tf
    de1, ra1 = _xyz2bl(x1, y1, z1)
    d1 = np.sqrt(x1 ** 2 + y1 ** 2 + z1 ** 2) * 1e-3
    c1, s1 = np.cos(ra1), np.sin(ra1)
    cd1, sd1 = np.cos(de1), np.sin(de1)
    # rot = roty(de1) @ rotz(ra1) applied to (vx, vy, vz)
    u0 = c1 * vx + s1 * vy
    u1 = -s1 * vx + c1 * vy
    u2 = vz
    v0 = cd1 * u0 + sd1 * u2
    v1 = u1
    v2 = -sd1 * u0 + cd1 * u2
    return np.column_stack([np.rad2deg(ra1), np.rad2deg(de1), 1 / d1, v1 / d1, v2 / d1, v0 * AUYR2KMS])


def loglike_am(am, theta_planets, off5, jit2, dtype=np.float64):
    """loglike_AM(theta): planets [(P, K, phase, e, w, I, Omega)], the five
    offsets (RA, DE, PLX, pm RA, pm DE) and the jitters (Hipparcos, Gaia).
    ``dtype`` is the type of the barycentre and scan-epoch propagation (the
    planets' offsets, in mas, are FP64 either way)."""
    hp, gs = am['hipp'], am['gost']
    cat = np.asarray(am['catalogs'], dtype=dtype)
    nh, ng = len(hp['BJD']), len(gs['BJD'])
    t_iad = np.concatenate([hp['BJD'], gs['BJD']])
    plx0 = cat[-1, 3] - off5[2]
    coor = np.zeros((3, nh + ng))
    for th in theta_planets:
        coor += calc_astro(th, plx0, t_iad, am['common_t'])
    bary = barycenter(am, off5, dtype)
    J_H, J_G = jit2
    # Hipparcos: bary at the Hipparcos epoch against the Hipparcos solution
    ref_ra, ref_dec, ref_plx, ref_pmra, ref_pmde = cat[0, 1:6]
    b = bary[0]
    mean_dec = 0.5 * (ref_dec + b[1])
    dra = (b[0] - ref_ra) * np.cos(np.deg2rad(mean_dec)) * MAS_PER_DEG
    dde = (b[1] - ref_dec) * MAS_PER_DEG
    dplx, dpmra, dpmde = b[2] - ref_plx, b[3] - ref_pmra, b[4] - ref_pmde
    abs_h = (hp['CPSI'] * (coor[0, :nh] + dra + dpmra * hp['EPOCH']) +
             hp['SPSI'] * (coor[1, :nh] + dde + dpmde * hp['EPOCH']) +
             hp['PARF'] * dplx)
    res = hp['RES'] - abs_h
    var = hp['SRES'] ** 2 + J_H ** 2
    ll = -0.5 * (np.sum(res ** 2 / var + np.log(var)) + nh * LOG_2PI)
    # GOST: the DR3 barycentre propagated to each scan epoch
    b3 = bary[-1]
    t_g = np.asarray(gs['BJD'], dtype=dtype) - cat[-1, 0]
    decs = np.deg2rad(b3[1]) + b3[4] * t_g / DAY_PER_YEAR / 206265e3
    ras = np.deg2rad(b3[0]) + b3[3] * t_g / DAY_PER_YEAR / np.cos(decs) / 206265e3
    ref_ra3, ref_dec3 = cat[-1, 1], cat[-1, 2]
    # dec = deg(decs) + mas2deg(epoch dec); ddec = (dec - ref_dec) mas
    ddeg = (np.rad2deg(decs) - ref_dec3) + coor[1, nh:] / MAS_PER_DEG
    dec = ref_dec3 + ddeg
    dra_g = (np.rad2deg(ras) - ref_ra3) * np.cos(np.deg2rad(dec)) * MAS_PER_DEG + coor[0, nh:]
    ddec_g = ddeg * MAS_PER_DEG
    dplx_g = b3[2] + coor[2, nh:]
    abs_g = gs['SPSI'] * dra_g + gs['CPSI'] * ddec_g + gs['parf'] * dplx_g
    for row, (catn, ci) in enumerate((('GDR2', 1), ('GDR3', 2))):
        p = np.asarray(am['gsv'][catn], dtype=dtype) @ abs_g[am['masks'][catn]]
        r = np.asarray(am['astro_gost'][row], dtype=dtype) - p
        quad = r @ np.asarray(am['inv_cov'][ci], dtype=dtype) @ r / J_G ** 2
        ll += -0.5 * (quad + 5 * np.log(J_G ** 2) + am['log_det_cov'][ci] + 5 * LOG_2PI)
    return ll if dtype is not np.float64 else float(ll)
