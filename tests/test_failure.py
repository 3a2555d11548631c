"""
Failure detection without a GPU fault: every device wait between steps is
bounded. A host-side hook (mkg_set_wait) raises the target of every step
wait so that nothing ever satisfies it; the kernel must give up within the
bound, report MKG_DEV_TIMEOUT, and leave the context usable, so that the
next run gives the same results as an undisturbed one.
"""
import time

import numpy as np
import pytest

from conftest import myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib

pytestmark = pytest.mark.gpu


def _sim(decker, sync, stage):
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=0.2)
    s = mg.SimulationCUDA(decker, p, ncells=(64, 32), rl=True,
                          stage_tiles=stage, block=128, min_blocks=1)
    s._sync = sync
    s.set_paced_cells(3, 32)
    return s


@pytest.mark.parametrize('sync', ['barrier', 'neighbors'])
@pytest.mark.parametrize('stage', [False, True])
def test_step_wait_times_out_and_context_survives(decker, sync, stage):
    s = _sim(decker, sync, stage)
    ref = s.run(1.0, log=['engine.time', 'membrane.V'], log_interval=0.1)
    ref_state = s.state_array()
    s.reset()
    be = s._backend[1]
    assert be.lib.mkg_set_wait(be.h, 20000000, 1000) == 0   # 20 ms
    t0 = time.perf_counter()
    with pytest.raises(_lib.MkgError) as e:
        s.run(1.0, log=['engine.time', 'membrane.V'], log_interval=0.1)
    assert time.perf_counter() - t0 < 10
    assert e.value.code == _lib.MKG_ERR_TIMEOUT
    assert 'timed out' in str(e.value)
    # Same backend, normal waits again: the undisturbed results
    assert s._backend[1] is be
    assert be.lib.mkg_set_wait(be.h, 2000000000, 0) == 0
    s.reset()
    d = s.run(1.0, log=['engine.time', 'membrane.V'], log_interval=0.1)
    assert np.array_equal(s.state_array(), ref_state)
    for k in ref.keys():
        assert np.array_equal(np.asarray(ref[k]), np.asarray(d[k]))


def test_wait_bound_is_checked(decker):
    s = _sim(decker, 'barrier', False)
    s.run(0.1)
    be = s._backend[1]
    for bad in ((0, 0), (10 ** 12, 0), (2000000000, -1),
                (2000000000, 65537)):
        assert be.lib.mkg_set_wait(be.h, *bad) == _lib.MKG_ERR_ARG
