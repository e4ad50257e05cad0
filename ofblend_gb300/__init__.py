"""flof-gb300: the FlOF hot path of thunil/ofblend (4D optical-flow
deformation between space-time SDF data sets, and its semi-Lagrangian
application) as hand-written CUDA for GB300 (sm_103a), behind a C ABI
(include/flof_gb300.h) and the reference's Python call surface.

Importing the package does not touch the GPU; the first grid or plugin call
loads libflof_gb300.so and fails loudly if it has not been built.
"""
from .api import *  # noqa: F401,F403
from .api import __all__  # noqa: F401
