"""
The allocation-free state upload, ``mkg_set_state_static``.

Callers that must not call cudaMalloc where they upload a state (a
real-time pacing loop that cannot afford cudaMalloc's device-wide
synchronisation, or a host that keeps device memory in its own pool or
under a fixed budget) use this entry point instead of ``mkg_set_state``.
It stages through a fixed 16 MiB device array, so it must give exactly
what ``mkg_set_state`` gives, call after call, and must refuse states
larger than that array.

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


def test_static_upload_allocates_nothing(br77):
    # On a handle that never staged a state through mkg_set_state (so the
    # handle's own staging buffer does not exist), the static upload takes
    # no device memory: free device memory is unchanged, while the
    # allocating upload of the same 16 MB state then takes some.
    import torch
    s0, be0 = _handle(br77, 40, myokit.DOUBLE_PRECISION)
    st0 = np.ascontiguousarray(s0.state_array())
    # Loads the library's device image and looks up the array's address
    be0.check(be0.lib.mkg_set_state_static(be0.h, _lib.dptr(st0), st0.size))
    s = mg.SimulationCUDA(br77, ncells=250000,
                          precision=myokit.DOUBLE_PRECISION)
    be = s._get_backend(s._kernel([]))   # a new handle, no state uploaded
    state = np.ascontiguousarray(s.state_array())
    n = state.size                       # 2,000,000 values, 16 MB
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    be.check(be.lib.mkg_set_state_static(be.h, _lib.dptr(state), n))
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0
    got = _download(be, n)
    assert np.array_equal(got, state)
    be.check(be.lib.mkg_set_state(be.h, _lib.dptr(state), n))
    free2 = torch.cuda.mem_get_info()[0]
    assert free2 < free1


def test_static_upload_refuses_accumulated_states(br77):
    # FP32 kernels with FP64 or compensated V and concentrations keep extra
    # planes that only mkg_set_state fills
    s = mg.SimulationCUDA(br77, ncells=30, accumulate='kahan')
    s.run(0.01)
    be = s._backend[1]
    state = np.ascontiguousarray(s.state_array())
    with pytest.raises(_lib.MkgError, match='use mkg_set_state'):
        be.check(be.lib.mkg_set_state_static(be.h, _lib.dptr(state),
                                             state.size))
