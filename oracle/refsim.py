"""
The reference ``myokit.SimulationOpenCL``, unmodified, on a CPU backend.

TEST INFRASTRUCTURE (the oracle). Only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py`` use it.

``SimulationOpenCL.__init__`` builds its compiled module with
``CModule._compile`` (``myokit/_sim/openclsim.py:320``), which needs OpenCL
headers and a platform. :class:`ReferenceCpuSimulation` overrides only that
call and returns :class:`oracle.cpu_backend.CpuBackend`, which executes the
kernel text the reference renders for every run. Everything else -- model
preparation, Rush-Larsen conversion, kernel rendering, log handling and
NaN diagnosis -- is the reference's own Python code.
"""
import os
import sys

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _ROOT not in sys.path:   # pragma: no cover
    sys.path.insert(0, _ROOT)

from myokit_gb300._deps import myokit  # noqa: E402
from oracle.cpu_backend import CpuBackend  # noqa: E402


class ReferenceCpuSimulation(myokit.SimulationOpenCL):
    """``myokit.SimulationOpenCL`` with its OpenCL module replaced by a CPU
    executor of the same rendered kernel."""

    def _compile(self, name, template, variables, libs, libd=None, incd=None,
                 larg=None, carg=None, store_build=False,
                 continue_in_debug_mode=False):
        return CpuBackend(
            variables['model'], variables['precision'], variables['dims'])

    def set_threads(self, n):
        """Host threads used for the cell and diffusion kernels."""
        self._sim.threads = max(1, int(n))
