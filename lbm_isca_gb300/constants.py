"""Physical constants and default resolution.

Values are the GFDL/Isca Earth defaults the reference uses
(pylbm_isca/constants.py:38-97); names follow the reference so callers can
switch packages without edits.
"""

import numpy as np

ER = 6.371e6               # earth radius [m]           (constants.py:38)
GRAV = 9.80                # gravity [m s-2]            (constants.py:39)
RDGAS = 287.04             # dry-air gas constant       (constants.py:40)
RVGAS = 461.50             # water-vapour gas constant  (constants.py:41)
KAPPA = 2.0 / 7.0          # R/Cp                       (constants.py:42)
CP = RDGAS / KAPPA
OMEGA = 7.2921150e-5       # rotation rate [rad s-1]    (constants.py:49)
RAIR = RDGAS
EPSV = RDGAS / RVGAS
EPSVT = RVGAS / RDGAS - 1.0  # virtual-temperature factor (constants.py:56)
DAYLEN_SEC = 86400.0
S2D = 86400.0
RHO00 = 1.225
GRAV_GT2GR = 9.80

IMAX = 128                 # longitudes                 (constants.py:69)
JMAX = 64                  # Gaussian latitudes
KMAX = 20                  # sigma levels
NMAX = 42                  # triangular truncation
MMAX = NMAX
LMAX = NMAX
MINT = 1
IDIM = IMAX + 1
IJDIM = IDIM * JMAX
NSPEC = (NMAX + 1) * (NMAX + 2) // 2

# the 17 ERA5 pressure levels of the basic-state input files [hPa]
# (constants.py:100-103)
PLEV17 = np.array([1000., 925., 850., 700., 600., 500., 400., 300., 250.,
                   200., 150., 100., 70., 50., 30., 20., 10.], dtype=np.float64)

# L20 sigma half levels, index 0 = surface (constants.py:92-97)
SIGM = np.array([
    1.000, 0.990, 0.970, 0.930, 0.870,
    0.790, 0.700, 0.600, 0.500, 0.410,
    0.330, 0.260, 0.200, 0.150, 0.100,
    0.070, 0.050, 0.040, 0.030, 0.020, 0.000,
], dtype=np.float64)
