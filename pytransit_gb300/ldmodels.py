"""Limb-darkening laws on the host (numpy), for user code and host callables.

Same names, arguments and formulas as pytransit/models/numba/ldmodels.py
(the RoadRunner copies, including ldi_linear's normalisation 2*pi/6*(3-2u)).
The GPU evaluates the named laws itself (rr_ld_tables_* in the C ABI); these
functions serve users who pass them as callables, and the law table maps each
of them back to its device law id so such calls still run on the GPU.
"""
from math import pi

import numpy as np

__all__ = ['ld_uniform', 'ldi_uniform', 'ld_linear', 'ldi_linear', 'ld_quadratic', 'ldi_quadratic',
           'ld_quadratic_tri', 'ldi_quadratic_tri', 'ld_nonlinear', 'ld_general', 'ld_square_root',
           'ld_logarithmic', 'ld_exponential', 'ld_power_2', 'ldi_power_2', 'ld_power_2_pm',
           'ldd_linear', 'ldd_quadratic', 'ldd_power_2', 'evaluate_ld', 'evaluate_ldi', 'LAW_IDS',
           'NAMED_LAWS']


def ld_uniform(mu, pv):
    return np.ones(np.size(mu))


def ldi_uniform(pv):
    return pi


def ld_linear(mu, pv):
    return 1. - pv[0] * (1. - mu)


def ldi_linear(pv):
    return 2 * pi * 1 / 6 * (3 - 2 * pv[0])


def ldd_linear(mu, pv):
    ldd = np.zeros((2, np.size(mu)))
    ldd[0] = pv[0]
    ldd[1] = mu - 1.0
    return ldd


def ld_quadratic(mu, pv):
    return 1. - pv[0] * (1. - mu) - pv[1] * (1. - mu) ** 2


def ldi_quadratic(pv):
    return 2 * pi * 1 / 12 * (-2 * pv[0] - pv[1] + 6)


def ldd_quadratic(mu, pv):
    ldd = np.zeros((3, np.size(mu)))
    ldd[0] = pv[0] + 2 * pv[1] - 2 * pv[1] * mu
    ldd[1] = mu - 1.0
    ldd[2] = -(1.0 - mu) ** 2
    return ldd


def ld_quadratic_tri(mu, pv):
    a, b = np.sqrt(pv[0]), 2 * pv[1]
    u, v = a * b, a * (1. - b)
    return 1. - u * (1. - mu) - v * (1. - mu) ** 2


def ldi_quadratic_tri(pv):
    a, b = np.sqrt(pv[0]), 2 * pv[1]
    u, v = a * b, a * (1. - b)
    return 2 * pi * 1 / 12 * (-2 * u - v + 6)


def ld_nonlinear(mu, pv):
    return (1. - pv[0] * (1. - np.sqrt(mu)) - pv[1] * (1. - mu) - pv[2] * (1. - np.power(mu, 1.5))
            - pv[3] * (1. - mu ** 2))


def ld_general(mu, pv):
    ldp = np.zeros(np.size(mu))
    for i in range(np.size(pv)):
        ldp += pv[i] * (1.0 - mu ** (i + 1))
    return ldp


def ld_square_root(mu, pv):
    return 1. - pv[0] * (1. - mu) - pv[1] * (1. - np.sqrt(mu))


def ld_logarithmic(mu, pv):
    return 1. - pv[0] * (1. - mu) - pv[1] * mu * np.log(mu)


def ld_exponential(mu, pv):
    return 1. - pv[0] * (1. - mu) - pv[1] / (1. - np.exp(mu))


def ld_power_2(mu, pv):
    return 1. - pv[0] * (1. - mu ** pv[1])


def ldi_power_2(pv):
    return 2 * pi * (-pv[0] * pv[1] + pv[1] + 2) / (2 * pv[1] + 4)


def ldd_power_2(mu, pv):
    ldd = np.zeros((3, np.size(mu)))
    ldd[0] = pv[0] * pv[1] * mu ** (pv[1] - 1.0)
    ldd[1] = mu ** pv[1] - 1.0
    ldd[2] = pv[0] * mu ** pv[1] * np.log(mu)
    return ldd


def ld_power_2_pm(mu, pv):
    c = 1 - pv[0] + pv[1]
    a = np.log2(c / pv[1])
    return 1. - c * (1. - mu ** a)


def _as3d(pvo):
    pvo = np.asarray(pvo, np.float64)
    if pvo.ndim == 1:
        return pvo.reshape((1, 1, -1))
    if pvo.ndim == 2:
        return pvo.reshape((1, pvo.shape[0], -1))
    return pvo


def evaluate_ld(ldm, mu, pvo):
    """ldp[npv, npb, nmu] of a host LD callable (ldmodels.py:143-158).  A 2D
    coefficient array is read as [npb, ncoef]."""
    pv = _as3d(pvo)
    ldp = np.zeros((pv.shape[0], pv.shape[1], np.size(mu)))
    for ipv in range(pv.shape[0]):
        for ipb in range(pv.shape[1]):
            ldp[ipv, ipb, :] = ldm(mu, pv[ipv, ipb])
    return ldp


def evaluate_ldi(ldi, pvo):
    """istar[npv, npb] of a host disk-integral callable (ldmodels.py:161-174)."""
    pv = _as3d(pvo)
    istar = np.zeros((pv.shape[0], pv.shape[1]))
    for ipv in range(pv.shape[0]):
        for ipb in range(pv.shape[1]):
            istar[ipv, ipb] = ldi(pv[ipv, ipb])
    return istar


# Device law ids (include/pytransit_gb300.h RR_LD_*), the names of
# RoadRunnerModel.ldmodels (rrmodel.py:48-58) and their host functions.
LAW_IDS = {'uniform': 0, 'linear': 1, 'quadratic': 2, 'quadratic-tri': 3, 'nonlinear': 4, 'general': 5,
           'square_root': 6, 'logarithmic': 7, 'exponential': 8, 'power-2': 9, 'power-2-pm': 10}

NAMED_LAWS = {'uniform': (ld_uniform, ldi_uniform),
              'linear': (ld_linear, ldi_linear),
              'quadratic': (ld_quadratic, ldi_quadratic),
              'quadratic-tri': (ld_quadratic_tri, ldi_quadratic_tri),
              'nonlinear': ld_nonlinear,
              'general': ld_general,
              'square_root': ld_square_root,
              'logarithmic': ld_logarithmic,
              'exponential': ld_exponential,
              'power-2': (ld_power_2, ldi_power_2),
              'power-2-pm': ld_power_2_pm}

# Number of coefficients per law (None: any).
LAW_NPAR = {'uniform': None, 'linear': 1, 'quadratic': 2, 'quadratic-tri': 2, 'nonlinear': 4,
            'general': None, 'square_root': 2, 'logarithmic': 2, 'exponential': 2, 'power-2': 2,
            'power-2-pm': 2}
