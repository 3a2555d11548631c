"""
Parity at the benchmark sizes: the timed sheets against the FP64 oracle
(the reference SimulationOpenCL running its own rendered kernel on all host
cores), over truncated windows that cover the paced upstroke.

- The 512 x 512 sheet exactly as the benchmark builds it (Decker 2009,
  Rush-Larsen, GKr/GNa lognormal(0, 0.2) fields from seed 0, the 4 left
  columns paced, V at 256 seeded probe cells), over 3 ms.
- The 2048 x 2048 S1 sheet (no fields, the 4 left columns paced), over
  1.2 ms.

Every probe trace and the whole final state are compared. Double precision
must agree to 1e-9 (mV for V, relative for the state; the reference's own
bar against Simulation1d is 1e-13 for a 10-cell cable, and CUDA and libm
transcendental functions differ in their last bits). Single precision, with
and without FP64 or Kahan-compensated V and concentrations, is compared
with the largest |dV| it is allowed, written beside each mode below.
"""
import os

import numpy as np
import pytest

from conftest import myokit
import myokit_gb300 as mg
from oracle.refsim import ReferenceCpuSimulation
import bench

pytestmark = pytest.mark.gpu

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION

# Largest |dV| (mV) against the FP64 oracle, per single-precision mode
FP32_DV = {
    'fp32': 1.0,
    'fp32+kahan': 0.5,
    'fp32+double': 0.5,
}
MODES = [
    ('fp64', DP, {}),
    ('fp32', SP, {}),
    ('fp32+kahan', SP, {'accumulate': 'kahan'}),
    ('fp32+double', SP, {'accumulate': 'double'}),
]


def _traces(d, keys):
    return np.stack([np.asarray(d[k], dtype=float) for k in keys])


def _compare(name, got, ref, keys, n_state, i_vm, report):
    """Probe traces and final states of one mode against the oracle."""
    (dg, sg), (dr, sr) = got, ref
    # Single precision logs hold the float32 rounding of the times
    tg = np.asarray(dg['engine.time'])
    tr = np.asarray(dr['engine.time']).astype(tg.dtype)
    assert np.array_equal(tg, tr)
    tv = np.max(np.abs(_traces(dg, keys) - _traces(dr, keys)))
    sg = sg.reshape(-1, n_state)
    sr = sr.reshape(-1, n_state)
    assert np.all(np.isfinite(sg))
    fv = np.max(np.abs(sg[:, i_vm] - sr[:, i_vm]))
    rel = np.max(np.abs(sg - sr) / (np.abs(sr) + 1e-12))
    report[name] = (tv, fv, rel)
    print('%s: max|dV| probes %.3g mV, final V %.3g mV, state rel %.3g'
          % (name, tv, fv, rel))
    if name == 'fp64':
        assert tv <= 1e-9
        assert fv <= 1e-9
        assert rel <= 1e-9
    else:
        assert tv <= FP32_DV[name]
        assert fv <= FP32_DV[name]


def _oracle(so, duration, log, log_interval):
    so.set_threads(os.cpu_count() or 1)
    d = so.run(duration, log=log, log_interval=log_interval)
    return d, np.asarray(so.state(), dtype=float)


def test_bench_sheet512_vs_oracle():
    # 600 steps of the 512 x 512 benchmark sheet: 1.6e8 cell-steps for the
    # oracle, the paced columns' upstroke included
    so, log = bench.make_sheet(ReferenceCpuSimulation, DP, 512)
    keys = log[1:]
    ref = _oracle(so, 3, log, 0.05)
    del so
    report = {}
    for name, prec, kw in MODES:
        s, log_ = bench.make_sheet(mg.SimulationCUDA, prec, 512, **kw)
        assert log_ == log
        d = s.run(3, log=log, log_interval=0.05)
        _compare(name, (d, s.state_array()), ref, keys, s._nstate,
                 s._model.label('membrane_potential').index(), report)
    # The upstroke happened inside the window
    assert _traces(ref[0], keys).max() > 0


def test_sheet2048_vs_oracle():
    # 240 steps of the 2048 x 2048 S1 sheet: 1.0e9 cell-steps for the
    # oracle; the paced columns' upstroke peaks inside the window
    n = 2048
    m = bench.load_model()

    def make(cls, precision=DP, **kw):
        p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
        s = cls(m, p, ncells=(n, n), precision=precision, rl=True, **kw)
        s.set_step_size(0.005)
        s.set_paced_cells(nx=4, ny=n, x=0, y=0)
        return s
    rng = np.random.default_rng(4)
    cells = sorted(rng.choice(n * n, 64, replace=False))
    keys = ['%d.%d.membrane.V' % (c % n, c // n) for c in cells] + [
        '%d.%d.membrane.V' % (x, y) for x in (0, 3, 4, 5) for y in (0, 2047)]
    log = ['engine.time'] + keys
    ref = _oracle(make(ReferenceCpuSimulation), 1.2, log, 0.05)
    report = {}
    i_vm = m.label('membrane_potential').index()
    for name, prec, kw in (MODES[0], MODES[2]):
        s = make(mg.SimulationCUDA, prec, **kw)
        d = s.run(1.2, log=log, log_interval=0.05)
        _compare(name, (d, s.state_array()), ref, keys, s._nstate, i_vm,
                 report)
        del s, d
    assert np.asarray(ref[0]['0.0.membrane.V']).max() > 0
