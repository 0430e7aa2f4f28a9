"""Spherical-harmonic transforms on the Gaussian grid, on the GPU.

Drop-in for ``pylbm_isca.spectral.Spectral`` (spectral.py:43-289): same
constructor, attributes, method names, shapes and index order (grid
``(nlat, nlon[, nk])`` north first, spectral ``(nmax+1, nmax+1[, nk])``
indexed ``[m, n]``, zero for ``n < m``).  Arrays are torch tensors on the
CUDA device; methods accept host (numpy) or device input, as the
reference's accept host or device input.

Everything numeric runs in the lbm_gb300 kernels: Gauss nodes and the
Legendre recurrences are generated in FP64 on the device
(``lbm_gauss_legendre``, ``lbm_legendre_tables``), the longitude transforms
are the library's real FFTs (``lbm_fourier_forward/inverse``) and the
Legendre contractions its analysis/synthesis kernels.  Only the Laplacian
scalings (a multiply by a per-n vector) are plain tensor arithmetic.
"""

from __future__ import annotations

import numpy as np
import torch

from . import ops as _ops  # noqa: F401  (registers torch.ops.lbm_gb300.*)
from ._lib import LBM_F32, LBM_F64, lib
from .backend import resolve, to_device
from .constants import ER, IMAX, JMAX, NMAX

_PREC = {"fp64": (torch.float64, torch.complex128, LBM_F64),
         "fp32": (torch.float32, torch.complex64, LBM_F32)}


class Spectral:
    """Gaussian grid + spherical-harmonic transform operators (GPU)."""

    #: True for the ensemble (member-axis) subclass, as in the reference.
    batched = False

    def __init__(self, nlon=IMAX, nlat=JMAX, nmax=NMAX, radius=ER, device="auto",
                 precision="fp64"):
        self.device = resolve(device)
        self.xp = torch
        self.nlon, self.nlat, self.nmax = int(nlon), int(nlat), int(nmax)
        self.a = float(radius)
        if self.nlon not in (64, 128, 256):
            raise ValueError("nlon must be 64, 128 or 256 for the GB300 FFT kernels")
        if 2 * (self.nmax + 1) > self.nlon:
            raise ValueError("nmax too large for nlon (need 2*(nmax+1) <= nlon)")
        if precision not in _PREC:
            raise ValueError(f"precision must be one of {list(_PREC)}")
        self.precision = precision
        self.rdtype, self.cdtype, self.prec_id = _PREC[precision]
        lib()                                      # fails loudly without the library
        dev = self.device
        M, J = self.nmax + 1, self.nlat
        f64 = dict(device=dev, dtype=torch.float64)
        LO = torch.ops.lbm_gb300
        # --- Gaussian grid (FP64 on the device; spectral.py:58-61) ----------
        mu, gw = LO.gauss_legendre(torch.empty(0, **f64), J)
        self.mu = mu.cpu().numpy()                 # host, like the reference
        self.gw = gw.cpu().numpy()
        self.lat = np.arcsin(self.mu)
        self.lon = np.arange(self.nlon) * (2.0 * np.pi / self.nlon)
        coslat_h = np.sqrt(1.0 - self.mu ** 2)
        self.gwdel = self.gw / self.a / (1.0 - self.mu ** 2)
        # --- Legendre tables (FP64 on the device; spectral.py:93-154) -------
        P, H = LO.legendre_tables(mu, self.nmax)
        self.pnm, self.hnm = P, H
        gw_d = gw
        gwdel_d = torch.as_tensor(self.gwdel, **f64)
        self.pnm_gw = P * gw_d
        self.pnm_gwdel = P * gwdel_d
        self.hnm_gwdel = H * gwdel_d
        self.pnm_T = P.transpose(1, 2).contiguous()
        self.hnm_T = H.transpose(1, 2).contiguous()
        n = np.arange(M, dtype=np.float64)
        eps = np.zeros((M, M + 1))
        for m in range(M):
            nn = np.arange(m + 1, M + 1, dtype=np.float64)
            eps[m, m + 1:] = np.sqrt((nn ** 2 - m ** 2) / (4.0 * nn ** 2 - 1.0))
        self.eps = eps
        nn1 = n * (n + 1.0)
        self.nn1 = nn1
        inv = np.zeros(M)
        inv[1:] = -self.a ** 2 / nn1[1:]
        self.coslat = torch.as_tensor(coslat_h, **f64)
        self.laplace = torch.as_tensor(-nn1 / self.a ** 2, **f64)
        self.inv_laplace = torch.as_tensor(inv, **f64)
        self.im = torch.as_tensor(1j * n, device=dev, dtype=torch.complex128)
        mm, nn_ = np.meshgrid(np.arange(M), np.arange(M), indexing="ij")
        self.mask = nn_ >= mm
        tw = torch.view_as_real(LO.fft_twiddles(torch.empty(0, **f64), self.nlon)).reshape(-1)
        self._tw64 = tw
        # working-precision copies used by the transform kernels
        rd = self.rdtype
        self._t = {
            "P": P.to(rd).contiguous(), "H": H.to(rd).contiguous(),
            "Pgw": self.pnm_gw.to(rd).contiguous(),
            "Pgwdel": self.pnm_gwdel.to(rd).contiguous(),
            "Hgwdel": self.hnm_gwdel.to(rd).contiguous(),
            "tw": tw.to(rd).contiguous(),
            "cos": self.coslat.to(rd).contiguous(),
            "rcos": (1.0 / (self.a * self.coslat)).to(rd).contiguous(),
            "invlap": self.inv_laplace.to(rd).contiguous(),
        }

    # ------------------------------------------------------------------
    # layout helpers: reference layouts are already [batch][A][B][cols]
    # ------------------------------------------------------------------
    def _has_k(self, x):
        return x.dim() == (4 if self.batched else 3)

    def _grid(self, f):
        t = to_device(f, self.device, self.rdtype)
        k = self._has_k(t)
        shape = t.shape
        if self.batched:
            B = shape[0]
            t4 = t if k else t.unsqueeze(-1)
        else:
            B = 1
            t4 = (t if k else t.unsqueeze(-1)).unsqueeze(0)
        return t4.contiguous(), (shape, k, B)

    def _spec(self, x):
        if isinstance(x, torch.Tensor):
            t = x.to(device=self.device)
        else:
            t = torch.as_tensor(np.asarray(x), device=self.device)
        if not torch.is_complex(t):
            t = t.to(self.rdtype)
        t = t.to(self.cdtype)
        k = self._has_k(t)
        shape = t.shape
        if self.batched:
            B = shape[0]
            t4 = t if k else t.unsqueeze(-1)
        else:
            B = 1
            t4 = (t if k else t.unsqueeze(-1)).unsqueeze(0)
        return t4.contiguous(), (shape, k, B)

    def _out_shape(self, meta, a, b):
        shape, k, B = meta
        lead = (shape[0],) if self.batched else ()
        tail = (shape[-1],) if k else ()
        return lead + (a, b) + tail

    # ------------------------------------------------------------------
    # kernel wrappers
    # ------------------------------------------------------------------
    def _fwd(self, g4, jscale=None):
        return torch.ops.lbm_gb300.fourier_forward(g4.to(self.rdtype), jscale,
                                                   self._t["tw"], self.nmax)

    def _inv(self, four, jscale=None):
        return torch.ops.lbm_gb300.fourier_inverse(four.to(self.cdtype), jscale,
                                                   self._t["tw"], self.nlon)

    def _anal(self, fa, ta, ima, fb=None, tb=None, imb=0, sb=1.0, nfac=None):
        return torch.ops.lbm_gb300.legendre_analysis(fa.to(self.cdtype), ta, int(ima), fb, tb,
                                                     int(imb), float(sb), nfac)

    def _synth(self, sa, ta, ima, na=None, sbp=None, tb=None, imb=0, nb=None, sb=1.0):
        return torch.ops.lbm_gb300.legendre_synthesis(sa.to(self.cdtype), ta, int(ima), na,
                                                      sbp, tb, int(imb), nb, float(sb))

    def _ret_grid(self, g4, meta):
        return g4.reshape(self._out_shape(meta, self.nlat, self.nlon))

    def _ret_spec(self, s4, meta):
        M = self.nmax + 1
        return s4.reshape(self._out_shape(meta, M, M))

    # ------------------------------------------------------------------
    # scalar transforms (spectral.py:186-197)
    # ------------------------------------------------------------------
    def grid_to_wave(self, f):
        g4, meta = self._grid(f)
        four = self._fwd(g4)
        return self._ret_spec(self._anal(four, self._t["Pgw"], 0), meta)

    def wave_to_grid(self, xi):
        s4, meta = self._spec(xi)
        return self._ret_grid(self._inv(self._synth(s4, self._t["P"], 0)), meta)

    # ------------------------------------------------------------------
    # differential operators (spectral.py:202-276)
    # ------------------------------------------------------------------
    def _nfac(self, xi, v):
        t = xi if isinstance(xi, torch.Tensor) else torch.as_tensor(np.asarray(xi),
                                                                     device=self.device)
        t = t.to(self.device)
        v = v.to(t.real.dtype if torch.is_complex(t) else t.dtype)
        return t * (v[:, None] if self._has_k(t) else v)

    def laplacian(self, xi):
        return self._nfac(xi, self.laplace)

    def inverse_laplacian(self, xi):
        return self._nfac(xi, self.inv_laplace)

    def hgrad(self, xi):
        s4, meta = self._spec(xi)
        rc = self._t["rcos"]
        gx = self._inv(self._synth(s4, self._t["P"], 1), rc)
        gy = self._inv(self._synth(s4, self._t["H"], 0), rc)
        return self._ret_grid(gx, meta), self._ret_grid(gy, meta)

    def uv_to_vordiv(self, u, v):
        gu, meta = self._grid(u)
        gv, _ = self._grid(v)
        c = self._t["cos"]
        Fu = self._fwd(gu, c)
        Fv = self._fwd(gv, c)
        pg, hg = self._t["Pgwdel"], self._t["Hgwdel"]
        vor = self._anal(Fv, pg, 1, Fu, hg, 0, 1.0)
        div = self._anal(Fu, pg, 1, Fv, hg, 0, -1.0)
        return self._ret_spec(vor, meta), self._ret_spec(div, meta)

    def neg_divergence(self, fx, fy):
        return -self.uv_to_vordiv(fx, fy)[1]

    def curl(self, fx, fy):
        return self.uv_to_vordiv(fx, fy)[0]

    def vordiv_to_uv(self, vor, div):
        """Spectral vorticity/divergence -> (u, v), the inverse Laplacian
        folded into the synthesis."""
        sv, meta = self._spec(vor)
        sd, _ = self._spec(div)
        P, H, il, rc = self._t["P"], self._t["H"], self._t["invlap"], self._t["rcos"]
        Um = self._synth(sd, P, 1, il, sv, H, 0, il, -1.0)
        Vm = self._synth(sv, P, 1, il, sd, H, 0, il, 1.0)
        return self._ret_grid(self._inv(Um, rc), meta), self._ret_grid(self._inv(Vm, rc), meta)

    def psichi_to_uv(self, psi, chi):
        sp_, meta = self._spec(psi)
        sc, _ = self._spec(chi)
        P, H, rc = self._t["P"], self._t["H"], self._t["rcos"]
        Um = self._synth(sc, P, 1, None, sp_, H, 0, None, -1.0)
        Vm = self._synth(sp_, P, 1, None, sc, H, 0, None, 1.0)
        return self._ret_grid(self._inv(Um, rc), meta), self._ret_grid(self._inv(Vm, rc), meta)

    def truncate(self, f):
        return self.wave_to_grid(self.grid_to_wave(f))

    @property
    def lat_deg(self):
        return np.degrees(self.lat)

    @property
    def lon_deg(self):
        return np.degrees(self.lon)
