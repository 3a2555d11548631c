"""
CPU tests of the host library: it loads without a GPU, exports every symbol
declared in ``include/mkg_tissue.h``, reports errors through
``mkg_last_error``, and follows the reference's step schedule and event
pacing exactly (``openclsim.c:1051-1162``, ``pacing.h``).
"""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load, myokit
from myokit_gb300 import _lib
from oracle.refsim import ReferenceCpuSimulation


def declared_functions():
    with open(os.path.join(ROOT, 'include', 'mkg_tissue.h')) as f:
        text = f.read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    names = re.findall(r'\b(mkg_[a-z_]+)\s*\(', text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name


def test_errors_without_handle():
    lib = _lib.load()
    h = ctypes.c_void_p()
    cfg = _lib.MkgConfig()
    cfg.nx = 0
    cfg.ny = 1
    cfg.real_bytes = 8
    cfg.n_state = 1
    cfg.block_x = cfg.block_y = 1
    code = lib.mkg_create(ctypes.byref(cfg), b'x', 1, ctypes.byref(h))
    assert code == _lib.MKG_ERR_ARG
    assert b'at least 1' in lib.mkg_last_error(None)
    cfg.nx = 4
    cfg.real_bytes = 2
    code = lib.mkg_create(ctypes.byref(cfg), b'x', 1, ctypes.byref(h))
    assert code == _lib.MKG_ERR_ARG
    assert b'single and double' in lib.mkg_last_error(None)
    assert lib.mkg_set_state(None, None, 0) == _lib.MKG_ERR_ARG
    assert lib.mkg_run_chunk(None, 1, None, None) == _lib.MKG_ERR_ARG
    lib.mkg_destroy(None)   # must be a no-op


def test_compile_error_reports_log():
    with pytest.raises(_lib.MkgError) as e:
        _lib.compile_source('this is not cuda', ['--gpu-architecture=sm_103a'])
    assert e.value.code == _lib.MKG_ERR_COMPILE
    assert 'error' in str(e.value)


def _events(protocol):
    return [[e.level(), e.start(), e.duration(), e.period(), e.multiplier()]
            for e in protocol.events()]


@pytest.mark.parametrize('tmin,dur,dt,logi', [
    (0, 15, 0.005, 0.5),
    (0, 7.3, 0.01, 0.37),
    (-10, 12.5, 0.02, 1.0),
    (3.0, 4.0, 0.1, 1e-9),
])
def test_schedule_matches_reference(tmin, dur, dt, logi):
    # The reference (on the CPU oracle) logs time and pace at every log
    # point; the host library's schedule must log at the same times.
    m = load('beeler-1977-model.mmt')
    p = myokit.pacing.blocktrain(period=2.5, duration=0.75, offset=0.3,
                                 level=2.0)
    s = ReferenceCpuSimulation(m, p, ncells=2,
                               precision=myokit.DOUBLE_PRECISION)
    s.set_step_size(dt)
    s.set_time(tmin)
    d = s.run(dur, log=['engine.time', 'engine.pace'], log_interval=logi)
    t, h, pace, lg = _lib.schedule_preview(
        _events(p), tmin, tmin + dur, dt, logi, 10 ** 6)
    assert abs(t[-1] + h[-1] - (tmin + dur)) < 1e-9
    np.testing.assert_array_equal(np.asarray(d['engine.time']), t[lg])
    np.testing.assert_array_equal(np.asarray(d['engine.pace']), pace[lg])


def test_schedule_every_step_matches_reference():
    # log_interval 0 logs every step: the full schedule must agree
    m = load('beeler-1977-model.mmt')
    p = myokit.Protocol()
    p.schedule(level=1, start=0.0123, duration=0.5, period=1.1,
               multiplier=3)
    p.schedule(level=3, start=0.9, duration=0.05)
    s = ReferenceCpuSimulation(m, p, ncells=1,
                               precision=myokit.DOUBLE_PRECISION)
    s.set_step_size(0.03)
    d = s.run(5, log=['engine.time', 'engine.pace'], log_interval=0)
    t, h, pace, lg = _lib.schedule_preview(_events(p), 0, 5, 0.03, 1e-9,
                                           10 ** 6)
    assert lg.all()
    np.testing.assert_array_equal(np.asarray(d['engine.time']), t)
    np.testing.assert_array_equal(np.asarray(d['engine.pace']), pace)


def test_schedule_pacing_errors():
    with pytest.raises(_lib.MkgError):
        _lib.schedule_preview([[1, 0, 1, 0, 2]], 0, 1, 0.1, 1, 100)
    with pytest.raises(_lib.MkgError):
        _lib.schedule_preview([[1, 0, 1, -1, 0]], 0, 1, 0.1, 1, 100)
    with pytest.raises(_lib.MkgError):
        # Two events starting at the same time
        _lib.schedule_preview([[1, 0, 1, 0, 0], [1, 0, 2, 0, 0]], 0, 1, 0.1,
                              1, 100)
