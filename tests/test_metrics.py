"""
Accuracy metrics (CPU): the frame-set versions (every cell at once, on the
frames' device) give exactly the per-trace activation times, APD90s and
comparisons.
"""
import numpy as np
import pytest
import torch

from myokit_gb300 import metrics


def _traces(n_cells=60, seed=0):
    # Action-potential-like traces: upstroke at a random time, plateau,
    # repolarisation; some cells never activate, some never repolarise
    rng = np.random.default_rng(seed)
    t = np.linspace(0, 400, 401)
    out = np.empty((len(t), n_cells))
    for c in range(n_cells):
        ta = rng.uniform(5, 80)
        dur = rng.uniform(150, 300)
        up = 1 / (1 + np.exp(-(t - ta) / 0.7))
        down = 1 / (1 + np.exp((t - ta - dur) / 12.0))
        v = -85 + 120 * up * down + rng.normal(0, 0.05, len(t))
        if c % 7 == 3:
            v = -85 + rng.normal(0, 0.05, len(t))       # no activation
        if c % 11 == 5:
            v = -85 + 120 * up                          # no repolarisation
        out[:, c] = v
    return t, out


def test_activation_and_apd_maps_equal_per_trace():
    t, v = _traces()
    frames = torch.tensor(v.reshape(len(t), 6, 10))
    ta = metrics.activation_map(t, frames).numpy().reshape(-1)
    apd = metrics.apd90_map(t, frames).numpy().reshape(-1)
    ref_ta = np.array([metrics.activation_time(t, v[:, c])
                       for c in range(v.shape[1])])
    ref_apd = np.array([metrics.apd90(t, v[:, c]) for c in range(v.shape[1])])
    np.testing.assert_array_equal(ta, ref_ta)
    np.testing.assert_array_equal(apd, ref_apd)
    assert np.isnan(ta).sum() > 0 and np.isnan(apd).sum() > np.isnan(ta).sum()
    assert np.isfinite(apd).sum() > 30


def test_compare_frames_equals_compare():
    t, v = _traces(seed=1)
    _, w = _traces(seed=1)
    w = w + np.random.default_rng(2).normal(0, 0.2, w.shape)
    frames = torch.tensor(v.reshape(len(t), 5, 12), dtype=torch.float32)
    ref = v.reshape(len(t), 5, 12) * 0 + w.reshape(len(t), 5, 12)
    got = metrics.compare_frames(t, frames, ref)
    v32 = frames.double().numpy().reshape(len(t), -1)
    exp = metrics.compare(
        t, {c: v32[:, c] for c in range(60)},
        {c: w[:, c] for c in range(60)})
    assert got['max_abs_dV_mV'] == exp['max_abs_dV_mV']
    assert got['max_activation_error_ms'] == exp['max_activation_error_ms']
    assert got['max_apd90_error_ms'] == exp['max_apd90_error_ms']
    assert got['cells_with_apd90'] == exp['traces_with_apd90']


def test_frame_metric_argument_checks():
    with pytest.raises(ValueError, match='One time per frame'):
        metrics.activation_map(np.arange(3.0), np.zeros((4, 2)))
    with pytest.raises(ValueError, match='same shape'):
        metrics.compare_frames(np.arange(3.0), np.zeros((3, 2)),
                               np.zeros((3, 3)))


@pytest.fixture(scope='module')
def cable_block():
    # A paced 80-cell Beeler-Reuter cable run by the oracle (the reference
    # SimulationOpenCL on its CPU backend), as a reference DataBlock1d
    from conftest import load, myokit
    from oracle.refsim import ReferenceCpuSimulation
    m = load('beeler-1977-model.mmt')
    m.get('membrane.i_stim.amplitude').set_rhs(-80)
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1)
    s = ReferenceCpuSimulation(m, p, ncells=80,
                               precision=myokit.DOUBLE_PRECISION)
    s.set_paced_cells(3)
    d = s.run(30, log=['engine.time', 'membrane.V'], log_interval=0.25)
    return myokit.DataBlock1d.from_log(d)


@pytest.mark.parametrize('kw', [{}, {'threshold': -20, 'border': 5},
                                {'length': 0.02, 'border': 0}])
def test_cable_cv_equals_reference(cable_block, kw):
    t = cable_block.time()
    v = cable_block.get1d('membrane.V')
    ref = cable_block.cv('membrane.V', **kw)
    got = metrics.cable_cv(t, torch.tensor(v, dtype=torch.float64), **kw)
    assert ref > 0 and got == ref


def test_cable_cv_edge_cases():
    t = np.arange(10.0)
    flat = np.full((10, 12), -85.0)
    assert metrics.cable_cv(t, flat) == 0
    with pytest.raises(ValueError, match='negative'):
        metrics.cable_cv(t, flat, border=-1)
    with pytest.raises(ValueError, match='less than half'):
        metrics.cable_cv(t, flat, border=6)
    with pytest.raises(ValueError, match='shaped'):
        metrics.cable_cv(t, np.zeros((10, 2, 2)))
