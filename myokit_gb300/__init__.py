"""
myokit_gb300 -- a GB300-native (sm_103a) backend for myokit's multicellular
tissue simulations.

``SimulationCUDA`` has the API of ``myokit.SimulationOpenCL`` and
``FiberTissueSimulationCUDA`` that of ``myokit.FiberTissueSimulation``; their
kernels are generated per model by ``myokit_gb300.exporter`` and run through
the C ABI declared in ``include/mkg_tissue.h``. ``myokit_gb300.adjoint``
holds the discrete adjoint, ``myokit_gb300.batch`` batched tissues.
"""
from ._deps import myokit  # noqa: F401
from .simulation import SimulationCUDA, compile_kernel  # noqa: F401
from .exporter import TissueKernel, CudaExpressionWriter  # noqa: F401
from .fiber_tissue import FiberTissueSimulationCUDA  # noqa: F401
from .batch import CableBatch, SheetBatch  # noqa: F401

__version__ = '0.1.0'
