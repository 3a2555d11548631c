"""
GPU parity: SimulationCUDA (fused sm_103a kernel, through the C ABI) against
the golden fixtures of the reference's Simulation1d and against the CPU
oracle (the reference SimulationOpenCL running its own rendered kernel).

Tolerances: the bar is |dV| <= 1e-3 mV in double precision; observed
differences are ~1e-13..1e-10 (CUDA and libm transcendental functions
differ in the last bits). Single precision is compared with a looser bound
that reflects float rounding, not a different algorithm.

At sizes where the oracle is too slow, size-independent properties are
checked instead: symmetry of a sheet paced along a full edge, equality of a
sheet row with the 1D cable, equality of batched and separate cables, and
run-to-run determinism.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load, myokit
import myokit_gb300 as mg
from oracle.refsim import ReferenceCpuSimulation

pytestmark = pytest.mark.gpu

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION
FP64_TOL = 1e-9     # mV; the bar is 1e-3 mV


def maxdiff(a, b, skip=()):
    worst = 0.0
    assert set(a.keys()) == set(b.keys())
    for k in a.keys():
        if k in skip:
            continue
        x = np.asarray(a[k], dtype=float)
        y = np.asarray(b[k], dtype=float)
        assert x.shape == y.shape, k
        if len(x):
            worst = max(worst, float(np.max(np.abs(x - y))))
    return worst


def both(make, **run):
    out = []
    for cls in (ReferenceCpuSimulation, mg.SimulationCUDA):
        s = make(cls)
        out.append((s.run(**run), s))
    return out


def test_golden_sim1d_br77():
    g = np.load(os.path.join(GOLDEN, 'br77_sim1d.npz'))
    m = load('beeler-1977-model.mmt')
    m.get('membrane.i_stim.amplitude').set_rhs(-80)
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=3)
    s = mg.SimulationCUDA(m, p, ncells=10, precision=DP)
    s.set_step_size(0.005)
    s.set_paced_cells(2)
    d = s.run(15, log=['engine.time', 'membrane.V', 'engine.pace', 'isi.Isi',
                       'membrane.i_diff'], log_interval=0.5).npview()
    assert np.max(np.abs(d['engine.time'] - g['engine_time'])) < 1e-17
    assert np.max(np.abs(d['engine.pace'] - g['engine_pace'])) < 1e-17
    for c in range(10):
        for v in ('membrane.V', 'membrane.i_diff', 'isi.Isi'):
            ref = g[str(c) + '_' + v.replace('.', '_')]
            assert np.max(np.abs(d[v, c] - ref)) < 1e-10, (v, c)


def test_golden_cable200():
    g = np.load(os.path.join(GOLDEN, 'br77_cable200_sim1d.npz'))
    m = load('beeler-1977-model.mmt')
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = mg.SimulationCUDA(m, p, ncells=200, precision=DP)
    s.set_step_size(0.005)
    s.set_conductance(9)
    s.set_paced_cells(5)
    d = s.run(20, log=['engine.time', 'membrane.V'], log_interval=1).npview()
    assert np.max(np.abs(d['engine.time'] - g['engine_time'])) == 0
    worst = max(np.max(np.abs(d['membrane.V', c] - g['%d_membrane_V' % c]))
                for c in range(200))
    assert worst < FP64_TOL


@pytest.mark.parametrize('precision,tol', [(DP, FP64_TOL), (SP, 2e-3)])
def test_2d_grid(br77, precision, tol):
    p = myokit.pacing.blocktrain(duration=2, offset=1, period=1000)

    def make(cls):
        s = cls(br77, p, ncells=(37, 11), precision=precision)
        s.set_paced_cells(3, 4, 1, 2)
        s.set_conductance(8, 5)
        return s
    (a, sa), (b, sb) = both(make, duration=10, log_interval=0.25,
                            log=['engine.time', 'engine.pace', 'membrane.V',
                                 'membrane.i_diff', 'isi.Isi'])
    assert maxdiff(a, b) < tol
    assert np.max(np.abs(np.array(sa.state()) - np.array(sb.state()))) < tol


def test_heterogeneous_2d(br77):
    p = myokit.pacing.blocktrain(duration=2, offset=1, period=1000)
    rng = np.random.default_rng(3)
    gx = rng.uniform(0, 12, (9, 19))
    gy = rng.uniform(0, 6, (8, 20))

    def make(cls):
        s = cls(br77, p, ncells=(20, 9), precision=DP)
        s.set_paced_cells(2, 9)
        s.set_conductance_field(gx, gy)
        return s
    (a, _), (b, _) = both(make, duration=12, log_interval=0.5,
                          log=['engine.time', 'membrane.V',
                               'membrane.i_diff'])
    assert maxdiff(a, b) < FP64_TOL


def test_connections_graph(br77):
    p = myokit.pacing.blocktrain(1000, 3, level=1)
    rng = np.random.default_rng(5)
    n = 40
    conns = []
    seen = set()
    for _ in range(90):
        i, j = sorted(rng.choice(n, 2, replace=False))
        if (i, j) not in seen:
            seen.add((i, j))
            conns.append((int(j), int(i), float(rng.uniform(0.5, 8))))

    def make(cls):
        s = cls(br77, p, ncells=n, precision=DP)
        s.set_paced_cell_list([0, 7, 13])
        s.set_connections(conns)
        return s
    (a, _), (b, _) = both(make, duration=8, log_interval=0.2,
                          log=['engine.time', 'membrane.V',
                               'membrane.i_diff'])
    # The reference sums currents with float atomics in arbitrary order;
    # here both sides sum in connection order.
    assert maxdiff(a, b) < FP64_TOL


def test_rl_fields_decker(decker):
    rng = np.random.default_rng(1)
    fkr = 0.0138542 * rng.lognormal(0, 0.2, (12, 17))
    fna = 9.075 * rng.lognormal(0, 0.2, (12, 17))
    p = myokit.pacing.blocktrain(1000, 2, level=1)

    def make(cls):
        s = cls(decker, p, ncells=(17, 12), precision=DP, rl=True)
        s.set_paced_cells(4, 12)
        s.set_field('ikr.Gbar', fkr)
        s.set_field('ina.Gbar', fna)
        return s
    (a, sa), (b, sb) = both(make, duration=6, log_interval=0.5,
                            log=myokit.LOG_STATE + myokit.LOG_BOUND)
    assert maxdiff(a, b) < FP64_TOL * 100
    va = np.array(sa.state())
    vb = np.array(sb.state())
    assert np.max(np.abs(va - vb)) < 1e-6


def test_log_all_inter(br77):
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=0.5)

    def make(cls):
        s = cls(br77, p, ncells=(3, 2), precision=DP, rl=True)
        s.set_paced_cells(1, 1)
        return s
    (a, _), (b, _) = both(make, duration=4, log_interval=0.1,
                          log=myokit.LOG_ALL)
    assert len(a) > 100
    assert maxdiff(a, b) < FP64_TOL * 100


def test_no_diffusion_fields(br77):
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1)
    vals = np.linspace(0.05, 0.15, 13)

    def make(cls):
        s = cls(br77, p, ncells=13, diffusion=False, precision=DP)
        s.set_field('isi.gsBar', vals)
        return s
    (a, _), (b, _) = both(make, duration=20, log_interval=1,
                          log=['engine.time', 'membrane.V', 'isi.Isi'])
    assert maxdiff(a, b) < FP64_TOL


def test_native_maths_single(br77):
    p = myokit.pacing.blocktrain(duration=2, offset=1, period=1000)

    def make(cls):
        s = cls(br77, p, ncells=(6, 5), native_maths=True)
        s.set_paced_cells(2, 5)
        return s
    (a, _), (b, _) = both(make, duration=8, log_interval=0.5,
                          log=['engine.time', 'membrane.V'])
    assert maxdiff(a, b, skip=('engine.time',)) < 0.5


@pytest.mark.parametrize('shape', [(1, 1), (1, 7), (7, 1), 1])
def test_degenerate_grids(br77, shape):
    p = myokit.pacing.blocktrain(duration=2, offset=1, period=1000)

    def make(cls):
        s = cls(br77, p, ncells=shape, precision=DP)
        s.set_paced_cells(1, 1)
        return s
    (a, _), (b, _) = both(make, duration=5, log_interval=0.5,
                          log=['engine.time', 'membrane.V',
                               'membrane.i_diff'])
    assert maxdiff(a, b) < FP64_TOL


def test_empty_run_and_zero_duration(br77):
    s = mg.SimulationCUDA(br77, ncells=4)
    d = s.run(0, log=['engine.time', 'membrane.V'])
    assert len(d['engine.time']) == 0
    x = s.state()
    s.run(0)
    assert s.state() == x


# ---------------------------------------------------------------------------
# Full-size properties
# ---------------------------------------------------------------------------

def _sheet(model, n, precision, ny=None, rl=True):
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    ny = n if ny is None else ny
    s = mg.SimulationCUDA(model, p, ncells=(n, ny), precision=precision,
                          rl=rl)
    s.set_paced_cells(nx=4, ny=ny, x=0, y=0)
    return s


@pytest.mark.parametrize('precision', [SP, DP])
def test_sheet512_rows_equal_cable(decker, precision):
    # A sheet paced along its full left edge has identical rows, and every
    # row equals the 1D cable of the same length, bit for bit.
    n = 512
    s = _sheet(decker, n, precision)
    keys = ['%d.%d.membrane.V' % (x, y) for x in (0, 5, 100, 511)
            for y in (0, 1, 255, 511)]
    d = s.run(3, log=keys, log_interval=0.5)
    st = s.state_array().reshape(n, n, -1)
    assert np.all(np.isfinite(st))
    assert np.array_equal(st, np.broadcast_to(st[:1], st.shape))
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    c = mg.SimulationCUDA(decker, p, ncells=n, precision=precision, rl=True)
    c.set_conductance(10)
    c.set_paced_cells(4)
    c.run(3)
    assert np.array_equal(c.state_array().reshape(n, -1), st[0])
    for x in (0, 5, 100, 511):
        ref = np.asarray(d['%d.0.membrane.V' % x])
        for y in (1, 255, 511):
            assert np.array_equal(np.asarray(d['%d.%d.membrane.V' % (x, y)]),
                                  ref)


def test_sheet512_deterministic(decker):
    rng = np.random.default_rng(0)
    f = 0.0138542 * rng.lognormal(0, 0.2, (512, 512))
    out = []
    for _ in range(2):
        s = _sheet(decker, 512, SP)
        s.set_field('ikr.Gbar', f)
        s.run(2)
        out.append(s.state_array())
    assert np.array_equal(out[0], out[1])


def test_batched_cables_equal_separate(br77):
    # Cables of uneven length in one launch (zero conductance between them)
    # give exactly the results of separate runs.
    rng = np.random.default_rng(7)
    lengths = rng.integers(5, 60, 9)
    scale = rng.lognormal(0, 0.3, 9)
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    n = int(lengths.sum())
    g = np.full(n - 1, 9.0)
    starts = np.concatenate([[0], np.cumsum(lengths)[:-1]])
    g[starts[1:] - 1] = 0
    field = np.repeat(0.09 * scale, lengths)
    paced = [int(s + k) for s in starts for k in range(3)]
    b = mg.SimulationCUDA(br77, p, ncells=n, precision=DP)
    b.set_conductance_field(g)
    b.set_field('isi.gsBar', field)
    b.set_paced_cell_list(paced)
    b.run(6)
    big = np.array(b.state()).reshape(n, -1)
    for k, (s0, ln) in enumerate(zip(starts, lengths)):
        c = mg.SimulationCUDA(br77, p, ncells=int(ln), precision=DP)
        c.set_conductance_field(np.full(ln - 1, 9.0))
        c.set_field('isi.gsBar', np.full(ln, 0.09 * scale[k]))
        c.set_paced_cell_list([0, 1, 2])
        c.run(6)
        assert np.array_equal(np.array(c.state()).reshape(ln, -1),
                              big[s0:s0 + ln]), k


def test_sheet2048_runs(decker):
    # The largest benchmark sheet: 4.2e6 cells, a few steps
    s = _sheet(decker, 2048, SP)
    d = s.run(0.1, log=['engine.time', '0.0.membrane.V',
                        '2047.2047.membrane.V'], log_interval=0.05)
    assert len(d['engine.time']) == 2
    st = s.state_array().reshape(2048, 2048, -1)
    assert np.all(np.isfinite(st))
    assert np.array_equal(st[0], st[2047])


# ---------------------------------------------------------------------------
# Launch grouping and tuning change nothing in the results
# ---------------------------------------------------------------------------

@pytest.mark.parametrize('spl,block', [(1, None), (7, None), (0, (32, 2)),
                                       (5, (64, 8))])
def test_launch_grouping_is_exact(decker, spl, block):
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    out = []
    for kw in ({}, {'steps_per_launch': spl, 'block': block}):
        s = mg.SimulationCUDA(decker, p, ncells=(70, 33), rl=True, **kw)
        s.set_paced_cells(3, 33)
        d = s.run(3, log=['engine.time', '5.5.membrane.V',
                          '69.32.membrane.V'], log_interval=0.1)
        out.append((s.state_array(), d))
    assert np.array_equal(out[0][0], out[1][0])
    for k in out[0][1].keys():
        assert np.array_equal(np.asarray(out[0][1][k]),
                              np.asarray(out[1][1][k]))


def test_nan_halt_across_launches():
    import test_oracle as to
    s = to.nan_sim(mg.SimulationCUDA)
    s._steps_per_launch = 7
    with pytest.raises(myokit.SimulationError, match='Time:  1.23'):
        s.run(5)


def test_autotune_keeps_results(br77, tmp_path, monkeypatch):
    monkeypatch.setenv('MYOKIT_GB300_CACHE', str(tmp_path))
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = mg.SimulationCUDA(br77, p, ncells=(40, 40))
    x0 = s.state_array()
    best = s.autotune(duration=0.2)
    assert best is not None
    assert np.array_equal(s.state_array(), x0) and s.time() == 0
    s.run(2)
    a = s.state_array()
    c = mg.SimulationCUDA(br77, p, ncells=(40, 40))   # picks the cache
    assert c._tuned_choice() is not None
    c.run(2)
    assert np.array_equal(a, c.state_array())


def test_run_frames_equal_logged_values(decker):
    # Frames kept on the device equal the values a normal log records
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    out = []
    for frames in (True, False):
        s = mg.SimulationCUDA(decker, p, ncells=(40, 24), rl=True)
        s.set_paced_cells(3, 24)
        if frames:
            t, f = s.run_frames(6, 1.5)
            out.append((np.asarray(t), f.cpu().numpy(), s.state_array()))
        else:
            keys = ['%d.%d.membrane.V' % (x, y) for y in range(24)
                    for x in range(40)]
            d = s.run(6, log=['engine.time'] + keys, log_interval=1.5)
            v = np.stack([np.asarray(d[k]) for k in keys], axis=1)
            out.append((np.asarray(d['engine.time']),
                        v.reshape(-1, 24, 40), s.state_array()))
    assert len(out[0][0]) == 4
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])


def test_run_frames_after_probe_runs(decker):
    # Frame runs keep their log columns between calls; a probe-logged run
    # in between replaces them, and the next frame run sets them again
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    out = []
    for mixed in (False, True):
        s = mg.SimulationCUDA(decker, p, ncells=(40, 24), rl=True)
        s.set_paced_cells(3, 24)
        frames = []
        for i in range(3):
            if mixed and i == 1:
                st, t0 = s.state_array(), s.time()
                s.run(1.5, log=['engine.time', '3.3.membrane.V'],
                      log_interval=0.5)
                s.set_state(st)
                s.set_time(t0)
            t, f = s.run_frames(1.5, 0.5)
            frames.append(f.cpu().numpy())
        out.append(np.concatenate(frames))
    assert np.array_equal(out[0], out[1])
