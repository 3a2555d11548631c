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


@pytest.mark.parametrize('split,block,ok', [
    (3, 128, False), (32, 128, False), (-1, 128, False),
    (8, 96, False),      # 3 warps: neither whole teams nor whole CTAs
    (16, 32, False),     # a cluster of 16 CTAs (at most 8)
    (4, 128, True), (8, 128, True), (16, 128, True), (8, 32, True)])
def test_create_validates_split(split, block, ok):
    # Checked before any device call: a refused shape names the rule, an
    # accepted one fails later for want of a GPU (or a valid kernel image)
    lib = _lib.load()
    h = ctypes.c_void_p()
    cfg = _lib.MkgConfig()
    cfg.nx = 200
    cfg.ny = 1
    cfg.real_bytes = 8
    cfg.n_state = 8
    cfg.block_x = block
    cfg.block_y = 1
    cfg.split = split
    code = lib.mkg_create(ctypes.byref(cfg), b'x', 1, ctypes.byref(h))
    assert code != _lib.MKG_OK
    msg = lib.mkg_last_error(None)
    if ok:
        assert b'split' not in msg
    else:
        assert code == _lib.MKG_ERR_ARG
        assert b'split' in msg
    if h:
        lib.mkg_destroy(h)


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


def _decays(n_state):
    # A model of n_state independent decays, V among them (for diffusion)
    m = myokit.Model('decays')
    c = m.add_component('c')
    t = c.add_variable('t')
    t.set_binding('time')
    t.set_rhs(0)
    for i in range(n_state):
        x = c.add_variable('x%d' % i)
        x.promote(float(i + 1))
        x.set_rhs('-%g * x%d' % (0.01 * (i + 1), i))
    c.get('x0').set_label('membrane_potential')
    idiff = c.add_variable('idiff')
    idiff.set_rhs(0)
    idiff.set_binding('diffusion_current')
    m.validate()
    return m


@pytest.mark.gpu
@pytest.mark.parametrize('n_state', [5, 96, 97, 130])
@pytest.mark.parametrize('precision', ['single', 'double'])
def test_state_round_trip_through_device_layout(n_state, precision):
    # The state goes to the device's plane layout and back: exact in
    # double precision, float rounding in single precision, for models
    # within the tiled conversion's limit (96 states) and beyond it, on a
    # cell count that is not a multiple of the 32-cell tile
    import myokit_gb300 as mg
    prec = myokit.DOUBLE_PRECISION if precision == 'double' else \
        myokit.SINGLE_PRECISION
    s = mg.SimulationCUDA(_decays(n_state), ncells=(37, 23), precision=prec)
    s.run(0.01)
    be = s._backend[1]
    n = s._nstate * s._ntotal
    rng = np.random.default_rng(n_state)
    for _ in range(2):
        x = np.ascontiguousarray(rng.normal(size=n) * 30)
        be.check(be.lib.mkg_set_state(be.h, _lib.dptr(x), n))
        y = np.empty(n)
        be.check(be.lib.mkg_get_state(be.h, _lib.dptr(y), n))
        want = x if precision == 'double' else \
            x.astype(np.float32).astype(float)
        assert np.array_equal(y, want)
