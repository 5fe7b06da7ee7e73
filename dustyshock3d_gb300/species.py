"""Host-side particle arrays in the reference's SoA FP64 layout (data.h:19-20, 49-55).

One ``Species`` holds one particle species: the gas (x, y, z, Vx..Vz, Ax..Az,
rho, p, e, mas, Ind) or one dust species (x..Vz, rho, mas, t_stop, h, ind).
Fields a species does not use stay zero.  ``h`` is the per-particle smoothing
length (the reference keeps one for dust, data.h:49, and one global h for gas).
"""
from __future__ import annotations

from dataclasses import dataclass, fields
from typing import Optional

import numpy as np

FLOAT_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts")


@dataclass
class Species:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: Optional[np.ndarray] = None
    vy: Optional[np.ndarray] = None
    vz: Optional[np.ndarray] = None
    ax: Optional[np.ndarray] = None
    ay: Optional[np.ndarray] = None
    az: Optional[np.ndarray] = None
    rho: Optional[np.ndarray] = None
    p: Optional[np.ndarray] = None
    e: Optional[np.ndarray] = None
    m: Optional[np.ndarray] = None
    h: Optional[np.ndarray] = None
    ts: Optional[np.ndarray] = None
    ind: Optional[np.ndarray] = None

    @property
    def n(self) -> int:
        return int(len(self.x))

    def fill_missing(self) -> "Species":
        n = self.n
        for f in FLOAT_FIELDS:
            a = getattr(self, f)
            if a is None:
                a = np.zeros(n, dtype=np.float64)
            setattr(self, f, np.ascontiguousarray(a, dtype=np.float64))
        self.ind = np.ascontiguousarray(self.ind if self.ind is not None else np.zeros(n, np.int32),
                                        dtype=np.int32)
        return self

    def copy(self) -> "Species":
        kw = {}
        for f in fields(self):
            a = getattr(self, f.name)
            kw[f.name] = None if a is None else np.array(a, copy=True)
        return Species(**kw)

    def take(self, idx) -> "Species":
        kw = {}
        for f in fields(self):
            a = getattr(self, f.name)
            kw[f.name] = None if a is None else np.ascontiguousarray(a[idx])
        return Species(**kw)
