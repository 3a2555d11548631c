"""
The allocation-free state upload, ``mkg_set_state_static``.

Callers that cannot call cudaMalloc where they upload a state (inside a
CUDA-graph stream capture, or in a real-time loop that cannot afford
cudaMalloc's device-wide synchronisation) use this entry point instead of
``mkg_set_state``. It stages through a fixed 16 MiB device array, so it
must give exactly what ``mkg_set_state`` gives, call after call, and must
refuse states larger than that array.

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from conftest import load, myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib

pytestmark = pytest.mark.gpu


def _handle(model, ncells, precision):
    """A simulation whose backend (C handle) exists, after a short run."""
    s = mg.SimulationCUDA(model, ncells=ncells, precision=precision)
    s.run(0.01)
    be = s._backend[1]
    return s, be


def _download(be, n):
    out = np.empty(n)
    be.check(be.lib.mkg_get_state(be.h, _lib.dptr(out), n))
    return out


@pytest.mark.parametrize('precision', [myokit.SINGLE_PRECISION,
                                       myokit.DOUBLE_PRECISION])
def test_static_upload_matches_allocating_upload(precision):
    m = load('beeler-1977-model.mmt')
    s, be = _handle(m, (37, 23), precision)
    n = s._nstate * s._ntotal
    rng = np.random.default_rng(11)
    tol = 0.0   # both paths convert the same doubles with the same rounding
    for call in range(2):
        state = np.ascontiguousarray(rng.normal(size=n) * 50)
        be.check(be.lib.mkg_set_state(be.h, _lib.dptr(state), n))
        expected = _download(be, n)
        # Scramble the device state, then upload through the static path
        junk = np.ascontiguousarray(rng.normal(size=n))
        be.check(be.lib.mkg_set_state(be.h, _lib.dptr(junk), n))
        be.check(be.lib.mkg_set_state_static(be.h, _lib.dptr(state), n))
        got = _download(be, n)
        assert np.max(np.abs(got - expected)) <= tol, call


def test_static_upload_then_run_matches(br77):
    # A run after a static upload equals a run after a normal upload
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    out = []
    for static in (False, True):
        s = mg.SimulationCUDA(br77, p, ncells=30,
                              precision=myokit.DOUBLE_PRECISION)
        s.run(0.01)
        be = s._backend[1]
        state = np.ascontiguousarray(s.state_array())
        n = state.size
        if static:
            be.check(be.lib.mkg_set_state_static(be.h, _lib.dptr(state), n))
        else:
            be.check(be.lib.mkg_set_state(be.h, _lib.dptr(state), n))
        be.check(be.lib.mkg_run_begin(be.h, 0.0, 2.0, 0.005, 1.0))
        t = ctypes.c_double()
        rows = ctypes.c_int64()
        code = _lib.MKG_OK
        while code == _lib.MKG_OK:
            code = be.check(be.lib.mkg_run_chunk(
                be.h, 10000, ctypes.byref(t), ctypes.byref(rows)))
        out.append(_download(be, n))
    assert np.array_equal(out[0], out[1])


def test_static_upload_rejects_oversized_state():
    m = load('decker-2009.mmt')   # 48 states
    s, be = _handle(m, 50000, myokit.SINGLE_PRECISION)
    n = s._nstate * s._ntotal     # 2.4e6 values > 2,097,152
    state = np.ascontiguousarray(np.zeros(n))
    with pytest.raises(_lib.MkgError, match='static staging area'):
        be.check(be.lib.mkg_set_state_static(be.h, _lib.dptr(state), n))
    with pytest.raises(_lib.MkgError, match='must have size'):
        be.check(be.lib.mkg_set_state_static(be.h, _lib.dptr(state), n - 1))
