"""Restatement of ``meepmeep.backends.numba.point2d`` (solve2d, sep_c, pos_c,
bounding_box) in plain Python, used only by tests/golden/make_golden.py to run
the reference's RoadRunner code.

The call sites in the reference fix the interface:
``solve2d(phase, p, a, i, e, w) -> c[2, 5]`` with ``x(t) = sum_j c[0, j] t^j``,
``y(t) = sum_j c[1, j] t^j`` (pytransit/models/numba/gdmodel.py:441-442), t in
days from conjunction; ``sep_c(t, c)`` the sky separation; and
``bounding_box(k, c) -> (t1, t4)``, the first and last contact times
(pytransit/models/roadrunner/model_full.py:60,65,95).

The Taylor coefficients are the exact time derivatives of the Keplerian sky
position (a Taylor jet of r'' = -mu r / |r|^3), the contact times follow the
bisection of pytransit/orbits/taylor_z.py:299-328 on the Taylor polynomial
(bracketed with the sky speed |dx/dt|, so it also serves an expansion about
mid-eclipse, where dx/dt < 0).
The oracle (oracle/rr_oracle.c) and the CUDA orbit kernel implement the same
statement; agreement with meepmeep's own numbers is not pinned.
"""
from math import atan2, cos, pi, sin, sqrt

import numpy as np


def _ea_newton(M, e):
    E, err, k = M, 0.05, 0
    while abs(err) > 1e-8 and k < 1000:
        err = E - e * sin(E) - M
        E = E - err / (1.0 - e * cos(E))
        k += 1
    return E


def solve2d(phase, p, a, i, e, w):
    n = 2.0 * pi / p
    se = sqrt(1.0 - e * e)
    if phase == 0.0:
        cth, sth = 0.0, 1.0
        sf, cf = cos(w), sin(w)
        r = a * (1.0 - e * e) / (1.0 + e * cf)
    else:
        f0 = 0.5 * pi - w
        E0 = atan2(se * sin(f0), e + cos(f0))
        M = E0 - e * sin(E0) + n * phase
        E = _ea_newton(M, e)
        f = atan2(se * sin(E) / (1.0 - e * cos(E)), (cos(E) - e) / (1.0 - e * cos(E)))
        sf, cf = sin(f), cos(f)
        cth, sth = cos(w + f), sin(w + f)
        r = a * (1.0 - e * e) / (1.0 + e * cf)
    vr = n * a * e * sf / se
    vt = n * a * (1.0 + e * cf) / se
    P = [[r * cth, r * sth], [vr * cth - vt * sth, vr * sth + vt * cth], [0, 0], [0, 0], [0, 0]]
    mu = n * n * a * a * a
    alpha = -1.5
    q0 = P[0][0] * P[0][0] + P[0][1] * P[0][1]
    q1 = 2.0 * (P[0][0] * P[1][0] + P[0][1] * P[1][1])
    s0 = 1.0 / (q0 * sqrt(q0))
    P[2] = [-mu * s0 * P[0][d] / 2.0 for d in range(2)]
    s1 = alpha * q1 * s0 / q0
    P[3] = [-mu * (s0 * P[1][d] + s1 * P[0][d]) / 6.0 for d in range(2)]
    q2 = 2.0 * (P[0][0] * P[2][0] + P[0][1] * P[2][1]) + (P[1][0] * P[1][0] + P[1][1] * P[1][1])
    s2 = ((alpha - 1.0) * q1 * s1 + 2.0 * alpha * q2 * s0) / (2.0 * q0)
    P[4] = [-mu * (s0 * P[2][d] + s1 * P[1][d] + s2 * P[0][d]) / 12.0 for d in range(2)]
    ci = cos(i)
    c = np.zeros((2, 5))
    for j in range(5):
        c[0, j] = -P[j][0]
        c[1, j] = -ci * P[j][1]
    return c


def pos_c(t, c):
    x = c[0, 0] + t * (c[0, 1] + t * (c[0, 2] + t * (c[0, 3] + t * c[0, 4])))
    y = c[1, 0] + t * (c[1, 1] + t * (c[1, 2] + t * (c[1, 3] + t * c[1, 4])))
    return x, y


def sep_c(t, c):
    x, y = pos_c(t, c)
    return sqrt(x * x + y * y)


def find_contact_point(k, point, c):
    s = -1.0 if point in (1, 2) else 1.0
    zt = 1.0 + k if point in (1, 4) else 1.0 - k
    t0 = 0.0
    t2 = s * 2.0 / abs(c[0, 1])     # the sky speed: x velocity is negative about an eclipse
    t1 = 0.5 * t2
    z0 = sep_c(t0, c) - zt
    z1 = sep_c(t1, c) - zt
    i = 0
    while abs(t2 - t0) > 1e-6 and i < 100:
        if z0 * z1 < 0.0:
            t1, t2 = 0.5 * (t0 + t1), t1
            z1 = sep_c(t1, c) - zt
        else:
            t0, t1 = t1, 0.5 * (t1 + t2)
            z0, z1 = z1, sep_c(t1, c) - zt
        i += 1
    return t1


def bounding_box(k, c):
    return find_contact_point(k, 1, c), find_contact_point(k, 4, c)
