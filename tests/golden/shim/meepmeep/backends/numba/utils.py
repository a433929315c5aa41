"""Restatement of ``meepmeep.backends.numba.utils.eclipse_time_offset`` used
only by tests/golden/make_golden.py: the time from mid-transit to mid-eclipse,
from the mean anomalies at the two conjunctions, as the reference's own
pytransit/orbits/orbits_py.py:544-555 (eclipse_phase) computes it."""
from math import atan2, cos, pi, sin, sqrt


def eclipse_time_offset(p, i, e, w):
    se = sqrt(1.0 - e * e)
    etr = atan2(se * sin(0.5 * pi - w), e + cos(0.5 * pi - w))
    eec = atan2(se * sin(0.5 * pi + pi - w), e + cos(0.5 * pi + pi - w))
    mtr = etr - e * sin(etr)
    mec = eec - e * sin(eec)
    phase = (mec - mtr) * p / (2.0 * pi)
    return phase if phase > 0.0 else p + phase
