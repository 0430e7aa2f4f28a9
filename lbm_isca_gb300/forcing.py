"""Time-varying MJO temperature forcing (the reference's forcing.py:99-157).

`MJOForcing` keeps the reference's call sequence: the first ``spinup`` calls
of ``.step()`` return the day-1 field; from then on the field marches through
the daily records, linearly interpolated over ``nt`` sub-steps,
``work(L) = gtf(it) + (gtf(it+1) - gtf(it)) / nt * (L-1)``.  The records are
given in memory (``gtf[day][lat][lon][lev]``, K/s); reading the Fortran record
files of the reference stays on its side.

For the fused stepper, `SpectralInterpolation` analyses every daily record to
spectral space once and forms each step's forcing on the device as the same
linear combination of two analysed records (the analysis is linear, so this
equals analysing the interpolated grid field, to FP64 rounding).  It follows
the forcing object's own state, read before each ``.step()`` call.
"""

from __future__ import annotations

import numpy as np
import torch


class MJOForcing:
    """Daily MJO heating records, held during spin-up, then interpolated."""

    def __init__(self, gtf, nt=72, spinup=435):
        self.gtf = np.asarray(gtf, dtype=np.float64)          # (day, lat, lon, lev)
        self.ndays = self.gtf.shape[0]
        self.nt, self.spinup = int(nt), int(spinup)
        self.reset()

    def reset(self):
        self.counter = 0
        self.counter2 = 0
        self.it = 1                  # 1-based day index
        self.spinning = True
        self._work = None
        self._field = self.gtf[0].copy()

    def plan(self):
        """(day a, day b, weight of b) of the field the next ``.step()`` returns
        (0-based days); the object's state is not changed."""
        counter = self.counter + 1
        spinning, it, c2 = self.spinning, self.it, self.counter2
        if spinning:
            if counter < self.spinup:
                return 0, 0, 0.0
            c2, it = 0, 1
        a = min(it, self.ndays) - 1
        b = min(it + 1, self.ndays) - 1
        return a, b, c2 / self.nt

    def step(self):
        """Advance one dynamics call and return the current forcing field."""
        self.counter += 1
        if self.spinning:
            if self.counter < self.spinup:
                return self._field
            self.counter2 = 0
            self.it = 1
            self.spinning = False
        if self.counter2 == 0:
            it = min(self.it, self.ndays)
            nxt = min(self.it + 1, self.ndays)
            a = self.gtf[it - 1]
            ka = (self.gtf[nxt - 1] - a) / self.nt
            self._work = a[None, ...] + ka[None, ...] * np.arange(self.nt)[:, None, None, None]
        self._field = self._work[self.counter2]
        self.counter2 += 1
        if self.counter2 == self.nt:
            self.counter2 = 0
            self.it += 1
        return self._field

    @property
    def day(self):
        return self.it


class SpectralInterpolation:
    """Device-side spectral forcing of an `MJOForcing`-like object.

    ``analyse(grid)`` maps a (lat, lon, lev) field to the model's spectral
    forcing (1, M, M, K); every daily record is analysed once.  ``next()``
    advances the object by one call and returns the spectral forcing of the
    field that call returns, as spec[a] + w (spec[b] - spec[a])."""

    def __init__(self, forcing, analyse):
        self.src = forcing
        days = forcing.gtf
        self.spec = torch.cat([analyse(torch.as_tensor(days[d])) for d in range(days.shape[0])])
        self._key = None
        self._out = None

    @staticmethod
    def supports(forcing):
        return all(hasattr(forcing, a) for a in ("gtf", "nt", "spinup", "plan", "step"))

    def next(self):
        a, b, w = self.src.plan()
        self.src.step()
        key = (a, b, w)
        if key != self._key:
            sa = self.spec[a:a + 1]
            self._out = sa if (b == a or w == 0.0) else sa + (self.spec[b:b + 1] - sa) * w
            self._key = key
        return self._out
