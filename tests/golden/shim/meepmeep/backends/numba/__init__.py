"""Restated stand-in for the third-party ``meepmeep`` package (>= 1.0.0), which
the reference imports but does not vendor.  Used only to run the reference's
RoadRunner code when generating golden fixtures."""
