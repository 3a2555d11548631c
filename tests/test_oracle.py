"""
Pins the CPU oracle (the reference SimulationOpenCL running its own rendered
kernel on the CPU) against the reference's known answers:

- Simulation1d, the reference's independent C cable code, through the
  committed golden fixtures (``tests/golden``) and live, to the 1e-13 bound
  of ``myokit/tests/test_simulation_opencl_vs_sim1d.py:123-136``;
- connections equal set_conductance (``test_simulation_opencl.py:394-528``);
- find_nan's pinned answers (``test_simulation_opencl.py:1536-1576``).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load, myokit
from oracle.refsim import ReferenceCpuSimulation

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION


def _small(cls, precision=DP):
    m = load('beeler-1977-model.mmt')
    m.get('membrane.i_stim.amplitude').set_rhs(-80)
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=3)
    s = cls(m, p, ncells=10, precision=precision)
    s.set_step_size(0.005)
    s.set_paced_cells(2)
    return s


LOG = ['engine.time', 'membrane.V', 'engine.pace', 'isi.Isi',
       'membrane.i_diff']


def test_oracle_vs_golden_sim1d():
    g = np.load(os.path.join(GOLDEN, 'br77_sim1d.npz'))
    d = _small(ReferenceCpuSimulation).run(
        15, log=LOG, log_interval=0.5).npview()
    assert np.max(np.abs(d['engine.time'] - g['engine_time'])) < 1e-17
    assert np.max(np.abs(d['engine.pace'] - g['engine_pace'])) < 1e-17
    for c in range(10):
        for v in ('membrane.V', 'membrane.i_diff', 'isi.Isi'):
            ref = g[str(c) + '_' + v.replace('.', '_')]
            assert np.max(np.abs(d[v, c] - ref)) < 1e-13, (v, c)


def test_oracle_vs_live_sim1d():
    m = load('beeler-1977-model.mmt')
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    sa = myokit.Simulation1d(m, p, ncells=12)
    sb = ReferenceCpuSimulation(m, p, ncells=12, precision=DP)
    for s in (sa, sb):
        s.set_step_size(0.01)
        s.set_conductance(9)
        s.set_paced_cells(3)
    da = sa.run(12, log=['engine.time', 'membrane.V'],
                log_interval=0.25).npview()
    db = sb.run(12, log=['engine.time', 'membrane.V'],
                log_interval=0.25).npview()
    for c in range(12):
        assert np.max(np.abs(da['membrane.V', c] - db['membrane.V', c])) \
            < 1e-13


def test_oracle_cable200_golden():
    g = np.load(os.path.join(GOLDEN, 'br77_cable200_sim1d.npz'))
    m = load('beeler-1977-model.mmt')
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = ReferenceCpuSimulation(m, p, ncells=200, precision=DP)
    s.set_step_size(0.005)
    s.set_conductance(9)
    s.set_paced_cells(5)
    d = s.run(20, log=['engine.time', 'membrane.V'], log_interval=1).npview()
    assert np.max(np.abs(d['engine.time'] - g['engine_time'])) == 0
    worst = max(np.max(np.abs(d['membrane.V', c] - g[
        '%d_membrane_V' % c])) for c in range(200))
    assert worst < 1e-12


@pytest.mark.parametrize('precision,tol', [(SP, 1e-4), (DP, 1e-9)])
def test_oracle_connections_equal_conductance(precision, tol):
    m = load('beeler-1977-model.mmt')
    p = myokit.pacing.blocktrain(1000, 10, level=1)
    s = ReferenceCpuSimulation(m, p, ncells=10, precision=precision)
    s.set_paced_cells(3)
    log = ['engine.time', 'membrane.V', 'membrane.i_diff']
    s.set_conductance(5, 0)
    d1 = s.run(10, log=log, log_interval=0.1).npview()
    s.reset()
    s.set_connections([(i, i + 1, 5) for i in range(9)])
    d2 = s.run(10, log=log, log_interval=0.1).npview()
    for c in (0, 9):
        assert np.max(np.abs(d1['membrane.V', c] - d2['membrane.V', c])) < tol


def _nan_model():
    # Voltage-clamped LR1991 (test_simulation_opencl.py:1459-1470)
    m = myokit.load_model('example')
    m.binding('pace').set_binding(None)
    v = m.get('membrane.V')
    v.set_rhs(-80)
    v.demote()
    v.set_label(None)
    v.set_binding('pace')
    m.get('ica.Ca_i').set_label('membrane_potential')
    m.get('membrane').move_variable(v, m.get('engine'))
    return m


def nan_sim(cls):
    p = myokit.Protocol()
    p.schedule(start=0, level=-80, duration=1.234)
    p.schedule(start=1.234, level=-47.13, duration=1000)
    s = cls(_nan_model(), p, ncells=(3, 3))
    s.set_paced_cell_list([[1, 1]])
    return s


def check_find_nan(cls):
    s = nan_sim(cls)
    p = myokit.Protocol()
    p.schedule(start=0, level=-90, duration=4)
    p.schedule(start=4, level=-47.13, duration=1000)
    s.set_protocol(p)
    x = s.state(0, 0)
    x[2] = 0.9
    s.set_state(x, 2, 2)
    d = s.run(10, report_nan=False)
    time, icell, var, value, states, bounds = s.find_nan(d)
    assert abs(time - 4.005) < 1e-5
    assert icell == [1, 1]
    assert var == 'ina.m'
    time, icell, var, value, states, bounds = s.find_nan(
        d, 'ina.j', [0.5, 1])
    assert 2 < time < 3
    assert icell == [2, 2]
    time, icell, var, value, states, bounds = s.find_nan(
        d, 'ina.j', [0.2, 1])
    assert 5 < time < 6
    assert icell == [2, 2]


def check_one_over_zero(cls):
    s = nan_sim(cls)
    with pytest.raises(myokit.SimulationError, match='Time:  1.23'):
        s.run(5)


def test_oracle_find_nan():
    check_find_nan(ReferenceCpuSimulation)


def test_oracle_one_over_zero():
    check_one_over_zero(ReferenceCpuSimulation)
