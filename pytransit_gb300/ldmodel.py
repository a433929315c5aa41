"""User limb-darkening model protocol, as pytransit/models/ldmodel.py:21-38.

An LDModel is called on the host with the radial mu grid and the coefficient
array and returns ``(ldp[npv, npb, nmu], istar[npv, npb])``; the RoadRunner
model uploads both and runs the rest of the path on the GPU.
"""
from typing import Tuple

from numpy import linspace, ndarray, pi, sqrt, trapezoid, zeros

__all__ = ['LDModel']


class LDModel:
    def __init__(self, niz: int = 200):
        self._int_z = linspace(0, 1, niz)
        self._int_mu = sqrt(1 - self._int_z ** 2)

    def __call__(self, mu: ndarray, x: ndarray) -> Tuple[ndarray, ndarray]:
        return self._evaluate(mu, x), self._integrate(x)

    def _evaluate(self, mu: ndarray, x: ndarray) -> ndarray:
        raise NotImplementedError

    def _integrate(self, x: ndarray) -> ndarray:
        """Disk integral 2 pi int z I(mu(z)) dz by the trapezoid rule on a
        uniform z grid, per (pv, pb)."""
        npv, npb = x.shape[0], x.shape[1]
        ldi = zeros((npv, npb))
        for ipv in range(npv):
            for ipb in range(npb):
                prof = self._evaluate(self._int_mu, x[ipv:ipv + 1, ipb:ipb + 1])
                ldi[ipv, ipb] = 2. * pi * trapezoid(self._int_z * prof.reshape(-1), self._int_z)
        return ldi
