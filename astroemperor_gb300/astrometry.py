"""Astrometric data of a joint RV + astrometry fit: Hipparcos intermediate
astrometric data (IAD), Gaia GOST scan epochs and the Hipparcos/Gaia DR2/DR3
catalogue solutions.

Mirrors ``DataWrapper``'s AM mode (``src/astroemperor/qol_utils.py:103-455``)
and the data prologue of the generated script
(``src/astroemperor/emp_model.py:609-706``) without pandas:

* ``datafiles/<target>/AM/*_hipgaia.hg123`` -- the catalogue rows (Hipparcos,
  Gaia DR2, Gaia DR3): reference epoch, position, parallax, proper motion,
  radial velocity, their errors and correlations; the 5x5 covariance of
  each row (``_construct_cov``), its inverse and log-determinant; the DR2
  and DR3 offsets relative to DR3 in mas (``astrometry_astro``);
* ``*_hip2.abs`` -- the Hipparcos abscissa residuals (BJD, EPOCH, PARF,
  CPSI, SPSI, RES, SRES);
* ``*_gost.csv`` -- the Gaia scan epochs (barycentric BJD, scan angle psi,
  along-scan parallax factor), kept before the DR3 baseline; each release's
  epochs outside its dead-time intervals (``astrometry_validate_epochs``;
  the intervals are given in on-board mission time and converted to BJD)
  and before its baseline, and the pseudo-inverse of its five-parameter
  design matrix (``astrometry_gost_coef``, ``astrometry_gost_gaia_sol_vec``).

The dead-time tables are Gaia's published astrometric gaps of DR2 and EDR3
(two columns, start and end, in OBMT revolutions); pass them as arrays.
"""
from __future__ import annotations

import csv
import os
from dataclasses import dataclass, field

import numpy as np

# epochs and baselines of the catalogues (qol_utils.py:200-220)
HIPP_EPOCH = 2448348.75
GDR2_REF_EP = 2457206.0
GDR2_BASELINE = 2457532.0
GDR3_REF_EP = 2457388.5
GDR3_BASELINE = 2457902.0
DAY_PER_YEAR = 365.25
# OBMT (revolutions) to BJD: 2457023.75 + (obmt - 1717.6256) * 365.25 / 1461
OBMT_ORIGIN_BJD = 2457023.75
OBMT_OFFSET = 1717.6256
CATS = ('GDR2', 'GDR3')
COV_KEYS = ('ra', 'dec', 'parallax', 'pmra', 'pmdec')


def _read_whitespace_table(path):
    """{column: values} of a whitespace table with a header line; numeric
    columns as float64, the others as strings."""
    with open(path) as f:
        rows = [l.split() for l in f if l.strip()]
    head, body = rows[0], rows[1:]
    out = {}
    for j, name in enumerate(head):
        col = [r[j] if j < len(r) else '' for r in body]
        try:
            out[name] = np.array([float(v) for v in col], dtype=np.float64)
        except ValueError:
            out[name] = np.array(col)
    return out


def _read_csv(path):
    with open(path, newline='') as f:
        rd = csv.reader(f)
        head = [h.strip() for h in next(rd)]
        body = [r for r in rd if r]
    out = {}
    for j, name in enumerate(head):
        col = [r[j].strip() for r in body]
        try:
            out[name] = np.array([float(v) for v in col], dtype=np.float64)
        except ValueError:
            out[name] = np.array(col)
    return out


def _construct_cov(hg):
    """5x5 covariance of every catalogue row (qol_utils.py:429-446)."""
    n = len(hg['ra'])
    cov = np.zeros((n, 5, 5))
    for r in range(n):
        for i, ki in enumerate(COV_KEYS):
            cov[r, i, i] = hg[f'{ki}_error'][r] ** 2
            for j in range(i + 1, 5):
                cov[r, i, j] = cov[r, j, i] = hg[f'{ki}_{COV_KEYS[j]}_cov'][r]
    return cov


@dataclass
class AMData:
    """Arrays of the astrometric likelihood (FP64)."""
    catalogs: np.ndarray           # [3, 7]: ref_epoch, ra, dec, parallax, pmra, pmdec, rv
    inv_cov: np.ndarray            # [3, 5, 5]
    log_det_cov: np.ndarray        # [3]
    astro_gost: np.ndarray         # [2, 5]: DR2, DR3 offsets from DR3 (mas) and plx, pm
    hipp: dict                     # BJD, EPOCH, PARF, CPSI, SPSI, RES, SRES [N_HIPP]
    gost: dict                     # BJD, CPSI, SPSI, parf [N_GOST]
    masks: dict                    # GDR2, GDR3 -> bool [N_GOST]
    gsv: dict                      # GDR2, GDR3 -> [5, n_cat] pseudo-inverse
    common_t: float = 0.0          # the RV time origin (min BJD of the RV data)
    labels: list = field(default_factory=list)

    @property
    def n_hipp(self):
        return len(self.hipp['BJD'])

    @property
    def n_gost(self):
        return len(self.gost['BJD'])

    def as_dict(self) -> dict:
        return {'catalogs': self.catalogs, 'inv_cov': self.inv_cov, 'log_det_cov': self.log_det_cov,
                'astro_gost': self.astro_gost, 'hipp': self.hipp, 'gost': self.gost,
                'masks': self.masks, 'gsv': self.gsv, 'common_t': self.common_t}


def gaia_masks(bjd, dead_dr2, dead_dr3):
    """Epochs of each Gaia release: before its baseline and outside its
    dead-time intervals (qol_utils.py:301-338)."""
    out = {}
    for cat, dead, base in (('GDR2', dead_dr2, GDR2_BASELINE), ('GDR3', dead_dr3, GDR3_BASELINE)):
        valid = np.ones(len(bjd), dtype=bool)
        d = np.asarray(dead, dtype=np.float64).reshape(-1, 2)
        scale = DAY_PER_YEAR / 1461.0
        start = OBMT_ORIGIN_BJD + (d[:, 0] - OBMT_OFFSET) * scale
        end = OBMT_ORIGIN_BJD + (d[:, 1] - OBMT_OFFSET) * scale
        for s, e in zip(start, end):
            valid[(bjd >= s) & (bjd <= e)] = False
        out[cat] = (bjd < base) & valid
    return out


def gost_solution_vectors(gost, masks):
    """Pseudo-inverse of each release's design matrix [sin psi, cos psi,
    parf, dt sin psi, dt cos psi] (qol_utils.py:383-420)."""
    out = {}
    for cat, ref in (('GDR2', GDR2_REF_EP), ('GDR3', GDR3_REF_EP)):
        m = masks[cat]
        tf = (gost['BJD'][m] - ref) / DAY_PER_YEAR
        s, c = gost['SPSI'][m], gost['CPSI'][m]
        X = np.column_stack([s, c, gost['parf'][m], tf * s, tf * c])
        out[cat] = np.linalg.pinv(X)
    return out


def load_am(folder: str, dead_dr2, dead_dr3, common_t: float) -> AMData:
    """``DataWrapper`` AM mode for ``folder`` (``datafiles/<target>/AM/``)."""
    files = sorted(fn for fn in os.listdir(folder) if fn != '.DS_Store')
    hg = hipp = gost_raw = None
    for fn in files:
        ident = fn.split('_')[-1]
        path = os.path.join(folder, fn)
        if ident == 'hipgaia.hg123':
            hg = _read_whitespace_table(path)
        elif ident == 'hip2.abs':
            hipp = _read_whitespace_table(path)
        elif ident == 'gost.csv':
            gost_raw = _read_csv(path)
    if hg is None or hipp is None or gost_raw is None:
        raise FileNotFoundError(f'{folder}: need *_hipgaia.hg123, *_hip2.abs and *_gost.csv')
    return build_am(hg, hipp, gost_raw, dead_dr2, dead_dr3, common_t, labels=files)


def build_am(hg, hipp, gost_raw, dead_dr2, dead_dr3, common_t, labels=()) -> AMData:
    """AMData from the three tables as {column: values} dictionaries."""
    cols = ['ref_epoch', 'ra', 'dec', 'parallax', 'pmra', 'pmdec', 'radial_velocity']
    catalogs = np.column_stack([np.asarray(hg[c], dtype=np.float64) for c in cols])
    cov = _construct_cov(hg)
    inv_cov = np.array([np.linalg.inv(c) for c in cov])
    log_det = []
    for c in cov:
        sign, ld = np.linalg.slogdet(c)
        if sign <= 0:
            raise ValueError('a catalogue covariance matrix is not positive definite')
        log_det.append(ld)
    # DR2 and DR3 relative to DR3 (qol_utils.py:236-245): ra offsets with the
    # DR2 declination's cosine, in mas
    ra, dec = np.asarray(hg['ra'])[-2:], np.asarray(hg['dec'])[-2:]
    astro = np.column_stack([(ra - ra[-1]) * np.cos(dec[-2] * np.pi / 180) * 3.6e6,
                             (dec - dec[-1]) * 3.6e6,
                             np.asarray(hg['parallax'])[-2:], np.asarray(hg['pmra'])[-2:],
                             np.asarray(hg['pmdec'])[-2:]])
    hp = {k: np.asarray(hipp[k], dtype=np.float64) for k in
          ('BJD', 'EPOCH', 'PARF', 'CPSI', 'SPSI', 'RES', 'SRES')}
    bjd = np.asarray(gost_raw['ObservationTimeAtBarycentre[BarycentricJulianDateInTCB]'], dtype=np.float64)
    psi = np.asarray(gost_raw['scanAngle[rad]'], dtype=np.float64)
    parf = np.asarray(gost_raw['parallaxFactorAlongScan'], dtype=np.float64)
    keep = bjd < GDR3_BASELINE
    gost = {'BJD': bjd[keep], 'CPSI': np.cos(psi[keep]), 'SPSI': np.sin(psi[keep]), 'parf': parf[keep]}
    masks = gaia_masks(gost['BJD'], dead_dr2, dead_dr3)
    gsv = gost_solution_vectors(gost, masks)
    return AMData(catalogs=catalogs, inv_cov=inv_cov, log_det_cov=np.array(log_det), astro_gost=astro,
                  hipp=hp, gost=gost, masks=masks, gsv=gsv, common_t=float(common_t), labels=list(labels))


def read_deadtime(path):
    """(start, end) rows of a Gaia astrometric-gaps table (comment lines '#')."""
    with open(path) as f:
        rows = [l for l in f if l.strip() and not l.lstrip().startswith('#')]
    rd = csv.reader(rows)
    head = [h.strip() for h in next(rd)]
    i0, i1 = head.index('start'), head.index('end')
    return np.array([[float(r[i0]), float(r[i1])] for r in rd if r], dtype=np.float64)
