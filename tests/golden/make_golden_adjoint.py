#!/usr/bin/env python3
"""Golden fixture for the adjoint: the reference's own tangent-linear model
of the tendencies (``Dynamics(strictly_linear=True).tendencies``, the
operator its tests/test_tangent_linear.py verifies), applied to its own
band-limited test direction (analysis/tl_verification.py: ``load_basic``
synthetic jet, ``make_direction``, ``state_at`` with amplitude 1) on the
T21 grid with 5 sigma layers.

Stores (``adjoint_tl.npz``): the zonally uniform basic state as (nlat, K)
profiles plus its constant ps, the direction (u0 v0 t0 q0 pi0), and the five
spectral tendencies L(direction).

Also the derivative of the reference's own nonlinear tendency (default
dynamics, kinetic energy kept, exact pi' <-> ps') about a non-zero state:
x0 = state_at(direction, 0.5), perturbed along a second direction d
(``make_direction`` seed 1) in the reference's coordinates (u, v, T, q, pi'),
by central differences with eps = 1e-4: D = (F(x0 + eps d) - F(x0 - eps d))
/ (2 eps), stored as ``D_*`` with d as ``d_*``.

Usage (where the reference checkout is available):

    python tests/golden/make_golden_adjoint.py <path of the reference checkout>
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import bs_inputs  # noqa: E402


def main(refdir):
    sys.path.insert(0, refdir)
    sys.path.insert(0, os.path.join(refdir, "analysis"))
    from pylbm_isca import Spectral, VerticalGrid
    from pylbm_isca.dynamics import BasicStateTerms, Dynamics
    import tl_verification as tl

    sp = Spectral(nlon=64, nlat=32, nmax=21, device="cpu")
    vg = VerticalGrid(sigm=bs_inputs.SIGM5, device="cpu")
    bs, _ = tl.load_basic(sp, vg, path=None)
    bst = BasicStateTerms(sp, vg, bs)
    dyn = Dynamics(sp, vg, bst, strictly_linear=True)
    direction = tl.make_direction(sp, vg)
    out = dyn.tendencies(tl.state_at(sp, vg, bs, direction, 1.0))
    for a in (bs.u, bs.t, bs.q):
        assert np.all(a == a[:, :1, :])          # zonally uniform
    assert np.all(bs.v == 0) and np.all(bs.ps == bs.ps.flat[0])
    names = ("vor", "div", "t", "pi", "q")
    full = Dynamics(sp, vg, bst, strictly_linear=False)
    d = tl.make_direction(sp, vg, seed=1)
    eps = 1e-4

    def at(s):
        x = [a0 + s * b for a0, b in zip((0.5 * c for c in direction), d)]
        return tl.state_at(sp, vg, bs, x, 1.0)
    fp, fm = full.tendencies(at(eps)), full.tendencies(at(-eps))
    np.savez_compressed(
        os.path.join(HERE, "adjoint_tl.npz"),
        bs_u=bs.u[:, 0, :], bs_t=bs.t[:, 0, :], bs_q=bs.q[:, 0, :], bs_ps=bs.ps.flat[0],
        sigm=bs_inputs.SIGM5, u0=direction[0], v0=direction[1], t0=direction[2],
        q0=direction[3], pi0=direction[4],
        d_u=d[0], d_v=d[1], d_t=d[2], d_q=d[3], d_pi=d[4],
        **{f"L_{k}": np.asarray(x) for k, x in zip(names, out)},
        **{f"D_{k}": (np.asarray(a) - np.asarray(b)) / (2 * eps)
           for k, a, b in zip(names, fp, fm)})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
