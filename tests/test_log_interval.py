"""
Log entry timing, checked with the reference's own test logic
(``myokit/tests/test_simulation_log_interval.py``, ``PeriodicTest.periodic``)
run on the oracle and on SimulationCUDA, and the fiber-tissue periodic
logging checks (``test_simulation_opencl_log_interval.py``) restated for
both fiber-tissue classes.
"""
import numpy as np
import pytest

from conftest import myokit
import myokit_gb300 as mg
from oracle.refsim import ReferenceCpuSimulation
from oracle.ft_backend import ReferenceFiberTissueCpu

RUN = ['oracle', pytest.param('cuda', marks=pytest.mark.gpu)]


def _lr91():
    import os
    path = os.path.join(os.path.dirname(myokit.__file__), 'tests', 'data',
                        'lr-1991.mmt')
    return myokit.load(path)


@pytest.mark.parametrize('impl', RUN)
def test_periodic_logging(impl):
    from myokit.tests.test_simulation_log_interval import PeriodicTest
    m, p, _ = _lr91()
    cls = ReferenceCpuSimulation if impl == 'oracle' else mg.SimulationCUDA
    s = cls(m, p, ncells=1)
    t = PeriodicTest('periodic')
    t.periodic(s)


@pytest.mark.parametrize('impl', RUN)
def test_periodic_logging_fiber_tissue(impl):
    m, p, _ = _lr91()
    cls = (ReferenceFiberTissueCpu if impl == 'oracle'
           else mg.FiberTissueSimulationCUDA)
    s = cls(m, m, p, ncells_fiber=(1, 1), ncells_tissue=(1, 1))
    emax = 1e-2
    for dur, interval in ((5, 0.5), (1, 0.5)):
        s.reset()
        d, e = s.run(dur, logf=['engine.time'], logt=myokit.LOG_NONE,
                     log_interval=interval)
        t = d.npview()['engine.time']
        q = np.arange(0, dur, interval)
        assert len(t) == len(q)
        assert np.max(np.abs(t - q)) < emax
    # Stop and start: the logs continue on the same grid
    s.reset()
    d, e = s.run(1, logf=['engine.time'], logt=myokit.LOG_NONE,
                 log_interval=0.5)
    d, e = s.run(2, logf=d, logt=myokit.LOG_NONE, log_interval=0.5)
    d, e = s.run(2, logf=d, logt=myokit.LOG_NONE, log_interval=0.5)
    t = d.npview()['engine.time']
    q = np.arange(0, 5, 0.5)
    assert len(t) == len(q)
    assert np.max(np.abs(t - q)) < emax
