"""pytransit_gb300: PyTransit's RoadRunner transit-model evaluation path,
GB300-native (hand-written sm_103a CUDA kernels behind a C ABI).

Drop-in names: RoadRunnerModel / RRModel, TransmissionSpectroscopyModel /
TSModel, EclipseSpectroscopyModel / ESModel, LDModel, TransitModel
(hpparvi/PyTransit 2.8.1, pytransit/models/__init__.py:17-26) and EclipseModel
(pytransit/models/new_eclipse_model.py).
"""
from .transitmodel import TransitModel
from .ldmodel import LDModel
from .rrmodel import RoadRunnerModel, create_z_grid
from .tsmodel import TransmissionSpectroscopyModel, TSModel
from .eclipse import EclipseModel, EclipseSpectroscopyModel, ESModel

RRModel = RoadRunnerModel

__all__ = ['TransitModel', 'LDModel', 'RoadRunnerModel', 'RRModel', 'TransmissionSpectroscopyModel', 'TSModel',
           'EclipseModel', 'EclipseSpectroscopyModel', 'ESModel', 'create_z_grid']
__version__ = '0.1.0'
