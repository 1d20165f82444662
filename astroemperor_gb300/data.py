"""Radial-velocity data loading and preprocessing.

Mirrors EMPEROR's ``DataWrapper`` (``src/astroemperor/qol_utils.py:16-198``)
for the RV mode, without pandas:

* ``datafiles/<target>/RV/*.vels`` files are read in sorted file-name order,
  one instrument per file, columns BJD, RV, eRV (extra activity columns are
  ignored, as EMPEROR does when ``switch_SA`` is off, ``emp.py:2307-2309``);
* each instrument's RV mean is subtracted when |mean| > 1e-6
  (``qol_utils.py:84-85``) and rows get ``Flag`` = 1-based instrument index
  (``qol_utils.py:95``);
* rows are sorted by BJD and ``common_t`` = min(BJD) is subtracted
  (``qol_utils.py:192-198``).  The sort here is stable.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np


@dataclass
class RVData:
    """Preprocessed RV table; the columns of EMPEROR's ``my_data``."""
    BJD: np.ndarray            # days since common_t (float64)
    RV: np.ndarray             # m/s, per-instrument mean removed (float64)
    eRV: np.ndarray            # m/s (float64)
    Flag: np.ndarray           # 1..nins (int64)
    common_t: float
    labels: list = field(default_factory=list)

    @property
    def nins(self) -> int:
        return len(self.labels) if self.labels else int(self.Flag.max(initial=0))

    @property
    def ndata(self) -> int:
        return len(self.BJD)

    def as_dict(self) -> dict:
        return {'X': self.BJD, 'Y': self.RV, 'YERR': self.eRV, 'Flag': self.Flag,
                'common_t': self.common_t, 'nins': self.nins}


def preprocess_instruments(instruments, labels=None) -> RVData:
    """Build an :class:`RVData` from per-instrument ``(BJD, RV, eRV)`` arrays."""
    if len(instruments) == 0:
        raise ValueError('no RV instruments given')
    bjd, rv, erv, flag = [], [], [], []
    for k, d in enumerate(instruments):
        d = np.asarray(d, dtype=np.float64)
        if d.ndim != 2 or d.shape[1] < 3 or d.shape[0] == 0:
            raise ValueError(f'instrument {k + 1}: expected an (n>0, >=3) array, got {d.shape}')
        r = d[:, 1].astype(np.float64, copy=True)
        mean = float(np.mean(r))
        if abs(mean) > 1e-6:
            r -= mean
        bjd.append(d[:, 0])
        rv.append(r)
        erv.append(d[:, 2])
        flag.append(np.full(d.shape[0], k + 1, dtype=np.int64))
    bjd = np.concatenate(bjd)
    order = np.argsort(bjd, kind='mergesort')
    bjd = bjd[order]
    common_t = float(bjd[0])
    if labels is None:
        labels = [f'INS{k + 1}' for k in range(len(instruments))]
    return RVData(BJD=bjd - common_t, RV=np.concatenate(rv)[order],
                  eRV=np.concatenate(erv)[order], Flag=np.concatenate(flag)[order],
                  common_t=common_t, labels=list(labels))


def load_rv_folder(folder: str) -> RVData:
    """Read every ``*.vels``-style file in ``folder`` (one per instrument)."""
    names = [fn for fn in sorted(os.listdir(folder)) if fn != '.DS_Store']
    if not names:
        raise FileNotFoundError(f'no RV files in {folder}')
    arrays = [np.loadtxt(os.path.join(folder, fn), ndmin=2) for fn in names]
    return preprocess_instruments(arrays, labels=names)


def load_target(target: str, read_loc: str = '') -> RVData:
    """``DataWrapper(target, read_loc)`` RV mode: ``{read_loc}datafiles/{target}/RV/``."""
    return load_rv_folder(f'{read_loc}datafiles/{target}/RV/')
