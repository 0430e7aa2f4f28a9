#!/usr/bin/env python3
"""Golden states of the plain single-member FP64 configuration at T42L20,
produced by running the reference package itself.

Usage (where the reference checkout is available):

    python tests/golden/make_golden_t42l20_run.py <path of the reference checkout>

The workload: T42 (128 x 64 Gaussian grid), 20 equally spaced sigma levels,
the solid-body basic state of ``lbm_isca_gb300.configs`` (u = 15 cos(lat),
T from a 6.5 K/km lapse rate, ps in gradient-wind balance, q = 0), the
elliptic heating centred at (0N, 120E) peaking at 2 K/day at sigma = 0.45,
the plain damping (1-day drag at the bottom and top levels, 30 days between,
del^4 hyperdiffusion with a 6-h e-folding, no sponge, no vertical diffusion),
dt = 1200 s, the reference's default dynamics (kinetic-energy term kept).
One call of ``LBM.run`` for 30 days (2160 advancing steps after the two
start-up calls, model.py:213-247); the state is recorded after 722 calls
(day 10) by the forcing object, which the reference's loop calls once at
the top of every call (model.py:224), and after the last call (day 30).

Stored per day: the current level ``ga`` as packed spectral coefficients
(vor, div, t, pi, q; the reference's own ``State.to_spectral``) and its grid
ps'.  About 2 MB in total.
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lbm_isca_gb300 import configs  # noqa: E402

DAY10_CALLS = 720 + 2


def pack(x, M):
    """[..., M, M, (K)] rectangle -> [..., NS, (K)] over n >= m."""
    x = np.asarray(x)
    mm, nn = np.nonzero(np.triu(np.ones((M, M), dtype=bool)))
    if x.shape[-2:] == (M, M):
        return x[..., mm, nn]
    return x[..., mm, nn, :]


def main(refdir):
    sys.path.insert(0, refdir)
    import pylbm_isca as ref

    nlon, nlat, nmax, K = 128, 64, 42, 20
    M = nmax + 1
    sigm = configs.equal_sigma_half_levels(K)
    bs = configs.solid_body_basic_state(nlon, nlat, sigm)
    heat = configs.elliptic_heating(nlon, nlat, sigm)
    sp = ref.Spectral(nlon=nlon, nlat=nlat, nmax=nmax, device="cpu")
    vg = ref.VerticalGrid(sigm=sigm, device="cpu")
    model = ref.LBM(bs, sp, vg, ref.Config(ndays=30.0, **configs.plain_damping(K)))
    out = {}

    def record(tag):
        spec = model.ga.to_spectral(sp)
        for name in ("vor", "div", "t", "pi", "q"):
            out[f"{tag}_{name}"] = pack(spec[name], M)
        out[f"{tag}_ps"] = np.asarray(model.ga.ps).copy()

    class Heating:
        """Constant heating; records the state at the top of call 723."""
        calls = 0

        def step(self):
            Heating.calls += 1
            if Heating.calls == DAY10_CALLS + 1:
                record("day10")
            return heat

    t0 = time.time()
    model.run(mjo_forcing=Heating(), verbose=False)
    record("day30")
    out["calls"] = np.array(Heating.calls)
    np.savez_compressed(os.path.join(HERE, "t42l20_reference_run.npz"), **out)
    print(f"t42l20_reference_run.npz written ({Heating.calls} calls, {time.time() - t0:.0f} s)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
