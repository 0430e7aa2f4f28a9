"""History output (drop-in for pylbm_isca/output.py).

``GradsWriter`` writes the reference's GrADS flat binary (output.py:1-16,
39-107): per output day one Fortran sequential record per level of psi,
chi, u, v, w, t, z and one of ps -- big-endian int32 byte count, big-endian
real*4 values on the model's north-first grid, byte count again -- with
z += ps * 100 / (rho0 g), and a ``.ctl`` descriptor (``OPTIONS SEQUENTIAL
YREV BIG_ENDIAN``, sigma levels, one day per time step).  The records of a
day are assembled on the device by ``lbm_grads_records`` (z term, rounding
to FP32, byte order, markers) and reach the host in one copy; ``LBM.run``
hands it the day's fields without bringing them to the host first.

``MultiWriter`` fans a history stream out to several writers.  The
reference's netCDF writer (output.py:109-150) needs xarray, which neither
this package nor its test machines have; it is not provided.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from .backend import asnumpy, stream_handle
from .constants import GRAV_GT2GR, RHO00

VARS = ["psi", "chi", "u", "v", "w", "t", "z", "p"]
VAR_INFO = {
    "psi": ("stream function", "m**2/s"),
    "chi": ("velocity potential", "m**2/s"),
    "u": ("zonal wind", "m/s"),
    "v": ("meridional wind", "m/s"),
    "w": ("p-vertical velocity", "hPa/s"),
    "t": ("temperature", "K"),
    "z": ("geopotential height", "m"),
    "p": ("surface pressure", "hPa"),
}


def _device_f64(a, device):
    t = a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a))
    return t.to(device=device, dtype=torch.float64).contiguous()


def grads_records(fields, apply_z=True, device="cuda"):
    """The day's GrADS records as bytes (big-endian), packed on the device.

    ``fields`` maps psi, chi, u, v, w, t, z to (nlat, nlon, K) and p to
    (nlat, nlon) arrays (host or device)."""
    from ._lib import check, lib
    dev = torch.device(device)
    if dev.type != "cuda":
        raise RuntimeError("grads_records packs on a CUDA device (there is no CPU path)")
    ts = [_device_f64(fields[n], dev) for n in VARS]
    nlat, nlon = ts[7].shape[-2:]
    kmax = ts[0].shape[-1]
    npts = nlat * nlon
    for n, t in zip(VARS[:7], ts[:7]):
        if tuple(t.shape) != (nlat, nlon, kmax):
            raise ValueError(f"history field {n} has shape {tuple(t.shape)}, "
                             f"expected {(nlat, nlon, kmax)}")
    out = torch.empty((7 * kmax + 1) * (npts + 2), dtype=torch.int32, device=dev)
    ptrs = (C.c_void_p * 8)(*[t.data_ptr() for t in ts])
    check(lib().lbm_grads_records(npts, kmax, ptrs, 1 if apply_z else 0, 1.0e2,
                                  RHO00 * GRAV_GT2GR,
                                  C.c_void_p(out.data_ptr()),
                                  C.c_void_p(stream_handle(torch.cuda.current_stream(dev)))),
          "lbm_grads_records")
    return out.cpu().numpy().tobytes()


class GradsWriter:
    """Writes ``out.grd`` + ``out.ctl`` GrADS flat binary."""

    accepts_device = True      # LBM.run may pass device tensors to add()

    def __init__(self, path, spectral, vertical, ctl_path=None,
                 apply_gt2gr_z=True, title="PyLBM-Isca T42L20"):
        self.path = path
        self.ctl_path = ctl_path or (os.path.splitext(path)[0] + ".ctl")
        self.sp, self.vg = spectral, vertical
        self.apply_gt2gr_z = apply_gt2gr_z
        self.title = title
        self.ntime = 0
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        self.fh = open(path, "wb")

    def add(self, day, fields):
        dev = next((v.device for v in fields.values()
                    if isinstance(v, torch.Tensor) and v.is_cuda), None)
        self.fh.write(grads_records(fields, self.apply_gt2gr_z,
                                    device=dev if dev is not None else "cuda"))
        self.ntime += 1

    def close(self):
        if not self.fh.closed:
            self.fh.close()
        self.write_ctl()

    def ctl_text(self):
        """The descriptor: lists latitudes south to north (YREV), sigma
        levels and one day per record set."""
        sp, vg = self.sp, self.vg
        lat = np.asarray(asnumpy(sp.lat_deg))[::-1]
        sig = np.asarray(asnumpy(vg.sig))
        kmax = int(vg.kmax)
        out = [f"DSET ^{os.path.basename(self.path)}",
               "OPTIONS SEQUENTIAL YREV BIG_ENDIAN",
               f"TITLE {self.title}",
               "UNDEF -999.",
               f"XDEF {sp.nlon} LINEAR 0. {360.0 / sp.nlon:.6g}",
               f"YDEF {sp.nlat} LEVELS"]
        out += [" " + " ".join(f"{x:9.4f}" for x in lat[i:i + 6]) for i in range(0, len(lat), 6)]
        out.append(f"ZDEF {kmax} LEVELS")
        out += [" " + " ".join(f"{x:.6g}" for x in sig[i:i + 6]) for i in range(0, kmax, 6)]
        out.append(f"TDEF {max(self.ntime, 1)} LINEAR 01jan0001 1dy")
        out.append(f"VARS {len(VARS)}")
        for name in VARS:
            desc, unit = VAR_INFO[name]
            out.append(f"{name:4s} {0 if name == 'p' else kmax:3d} 99 {desc} [{unit}]")
        out.append("ENDVARS")
        return "\n".join(out) + "\n"

    def write_ctl(self):
        with open(self.ctl_path, "w") as fh:
            fh.write(self.ctl_text())


class MultiWriter:
    """Fan a history stream out to several writers (output.py:153-165)."""

    def __init__(self, *writers):
        self.writers = [w for w in writers if w is not None]
        self.accepts_device = all(getattr(w, "accepts_device", False) for w in self.writers)

    def add(self, day, fields):
        for w in self.writers:
            w.add(day, fields)

    def close(self):
        for w in self.writers:
            w.close()
