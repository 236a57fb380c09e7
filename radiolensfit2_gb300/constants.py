"""Numeric constants of the shape-measurement path.

Values are those of the reference's default_params.h:28-79 and datatype.h:27-40, kept
bit-identical so that facet sizes, priors and fit tolerances agree with the reference.
"""
import math

PI = 3.14159265358979323846
C0 = 299792458.0
ARCS2RAD = PI / 648000.0
DEG2RAD = PI / 180.0

EFFICIENCY = 0.9
SEFD_SKA = 400e6          # micro-Jy
REF_FREQ = 1.4e9
PSF_NAT = 38
RMIN = 0.3
RMAX = 3.5
NUM_R = 29
ADD = -0.93
ESP = 0.33
R_STD = 0.3136
E_MAX = 0.804
E_0 = 0.0732
DISP = 0.2298
TOL = 1.0e-3
NP_MAX = 30
E_RES = 3.0e-3
VAR = 1e-4
NUM_ORIENT = 5


def ro_grid():
    """Scalelength nodes (arcsec), RadioLensfit2.cpp:371-389: Ro[0]=0 (unused), Ro[1]=RMIN,
    then quadratic spacing until a node reaches RMAX.  Returns the list including Ro[0]."""
    ro = [0.0, RMIN]
    while len(ro) < NUM_R and ro[-1] < RMAX:
        interval = 0.08 + 0.4 * math.pow((ro[-1] - RMIN) / (RMAX - RMIN), 2)
        ro.append(ro[-1] + interval)
    return ro


def scale_mean(flux):
    """distributions.c:59-62: mean of ln(scalelength[arcsec]) at a flux in micro-Jy."""
    return ADD + ESP * math.log(flux)


def rfunc(mu, sigma, r):
    """distributions.c:72-87: ln of the lognormal scalelength prior."""
    x = (math.log(r) - mu) / sigma
    return -(x * x) * 0.5 - math.log(r * sigma)


def facet_size(theta_med, length):
    """evaluate_uv_grid.c:50-55, with the unparenthesised ARCS2RAD macro expanded in the
    reference's left-to-right order."""
    return int(2 * math.ceil(length * PSF_NAT * theta_med * PI / 648000.0))
