"""Restatement of ``meepmeep.backends.numba.newton.eclipse_light_travel_time``
used only by tests/golden/make_golden.py (meepmeep is not installed): the
extra light travel time of the eclipse relative to the transit, the
line-of-sight distance between the planet's positions at the two conjunctions,
(r_transit + r_eclipse) sin i, in stellar radii of rstar solar radii (IAU
nominal R_sun), over c, in days."""
from math import cos, pi, sin

R_SUN = 6.957e8          # m
C_LIGHT = 299792458.0    # m / s


def eclipse_light_travel_time(p, a, i, e, w, rstar):
    r_tr = a * (1.0 - e * e) / (1.0 + e * cos(0.5 * pi - w))
    r_ec = a * (1.0 - e * e) / (1.0 + e * cos(1.5 * pi - w))
    return (r_tr + r_ec) * sin(i) * rstar * R_SUN / C_LIGHT / 86400.0
