"""
Batched tissues (myokit_gb300.batch): construction of the packed
conductances, paced cells and fields on the CPU, and on the GPU equality of
every batched cable and sheet with the same tissue simulated alone.
"""
import numpy as np
import pytest

from conftest import myokit
import myokit_gb300 as mg
from myokit_gb300.batch import CableBatch, SheetBatch, frames_to_block

SP = myokit.SINGLE_PRECISION
DP = myokit.DOUBLE_PRECISION


def _p():
    return myokit.pacing.blocktrain(period=1000, duration=2, offset=0.5)


def test_cable_batch_layout(br77):
    b = CableBatch(br77, [4, 1, 3], _p(), conductance=[2.0, 3.0, 5.0],
                   paced_cells=2, fields={'isi.gsBar': [1.0, 2.0, 3.0]})
    assert list(b.starts) == [0, 4, 5] and b.ncells == 8
    g = b.edge_conductances([2.0, 3.0, 5.0])
    assert list(g) == [2, 2, 2, 0, 0, 5, 5]
    assert b.paced_cells(2) == [0, 1, 4, 5, 6]
    assert list(b.per_cell([1.0, 2.0, 3.0])) == [1, 1, 1, 1, 2, 3, 3, 3]
    assert b.cable_log_keys(2) == ['5.membrane.V', '6.membrane.V',
                                   '7.membrane.V']
    with pytest.raises(ValueError):
        CableBatch(br77, [3, 0])
    with pytest.raises(ValueError):
        b.per_cell([1.0, 2.0])


def test_sheet_batch_layout(br77):
    b = SheetBatch(br77, [(3, 2), (2, 3)], _p(), conductance=(4.0, 7.0),
                   paced_columns=1, fields={'isi.gsBar': [1.0, 2.0]})
    assert (b.nx, b.ny) == (5, 3) and list(b.x0) == [0, 3]
    gx, gy = b.edge_conductances((4.0, 7.0))
    assert gx.tolist() == [[4, 4, 0, 4], [4, 4, 0, 4], [0, 0, 0, 4]]
    assert gy.tolist() == [[7, 7, 7, 7, 7], [0, 0, 0, 7, 7]]
    assert b.paced_cells(1) == [(0, 0), (0, 1), (3, 0), (3, 1), (3, 2)]
    base = br77.get('isi.gsBar').eval()
    f = b.per_cell([1.0, 2.0], base)
    assert f[2, 0] == base and f[0, 0] == 1.0 and f[2, 4] == 2.0


def _cable(model, n, g, field, precision):
    s = mg.SimulationCUDA(model, _p(), ncells=n, precision=precision)
    if n > 1:
        s.set_conductance_field(np.full(n - 1, g))
    s.set_paced_cells(min(n, 3))
    s.set_field('isi.gsBar', np.full(n, field))
    return s


@pytest.mark.gpu
@pytest.mark.parametrize('precision', [SP, DP])
def test_batched_cables_equal_separate_runs(br77, precision):
    lengths = [40, 73, 5, 1, 190]
    gs = [9.0, 5.0, 7.0, 3.0, 11.0]
    fs = [0.07, 0.09, 0.05, 0.1, 0.08]
    b = CableBatch(br77, lengths, _p(), conductance=gs, paced_cells=3,
                   fields={'isi.gsBar': fs}, precision=precision)
    b.sim.run(12)
    for c, n in enumerate(lengths):
        s = _cable(br77, n, gs[c], fs[c], precision)
        s.run(12)
        one = np.asarray(s.state()).reshape(n, -1)
        assert np.array_equal(one, b.cable_state(c)), c


@pytest.mark.gpu
def test_batched_sheets_equal_separate_runs(br77):
    shapes = [(12, 9), (7, 14), (20, 3)]
    b = SheetBatch(br77, shapes, _p(), conductance=(9.0, 6.0),
                   paced_columns=2, fields={'isi.gsBar': [0.07, 0.09, 0.05]},
                   precision=DP)
    b.sim.run(10)
    for i, (w, h) in enumerate(shapes):
        s = mg.SimulationCUDA(br77, _p(), ncells=(w, h), precision=DP)
        s.set_conductance_field(np.full((h, w - 1), 9.0),
                                np.full((h - 1, w), 6.0))
        s.set_paced_cells(2, h)
        s.set_field('isi.gsBar', np.full((h, w), [0.07, 0.09, 0.05][i]))
        s.run(10)
        one = np.asarray(s.state()).reshape(h, w, -1)
        assert np.array_equal(one, b.sheet_state(i)), i


@pytest.mark.gpu
def test_frames_to_block(br77):
    s = mg.SimulationCUDA(br77, _p(), ncells=(16, 8))
    s.set_paced_cells(2, 8)
    t, f = s.run_frames(3, 1)
    block = frames_to_block(t, f)
    assert block.len2d() == 1 and block.shape() == (len(t), 8, 16)
    assert np.array_equal(block.get2d('membrane.V'),
                          f.cpu().double().numpy())


# ---------------------------------------------------------------------------
# Batches against what the reference computes for the same tissues
# ---------------------------------------------------------------------------
#
# The reference expresses a batch of cables as one 1D SimulationOpenCL whose
# set_connections chains stop at cable ends, with set_paced_cell_list for
# the first cells of every cable and per-cell set_field values equal to the
# cable's value (openclsim.py:1387-1449, 1595-1629, 1495-1532). Sheets are
# expressed the same way: one 1D simulation whose connections form the grid
# of each sheet. The oracle runs exactly that through the reference's
# Python layer and its own rendered kernel.

BATCH_FIELDS = ['ina.Gbar', 'ikr.Gbar', 'ik1.Gbar']


def _oracle_1d(model, ncell, conns, paced, fields, dt, duration, log,
               protocol=None):
    from oracle.refsim import ReferenceCpuSimulation
    import os
    s = ReferenceCpuSimulation(model, protocol or _p(), ncells=ncell,
                               precision=DP, rl=True)
    s.set_threads(os.cpu_count() or 1)
    s.set_step_size(dt)
    s.set_connections(conns)
    s.set_paced_cell_list(paced)
    for name, values in fields.items():
        s.set_field(name, values)
    d = s.run(duration, log=log, log_interval=0.5)
    return d, np.asarray(s.state(), dtype=float).reshape(ncell, -1)


def _cable_case(model):
    rng = np.random.default_rng(13)
    lengths = rng.integers(20, 61, 8)
    fields = {name: model.get(name).eval() * rng.lognormal(0, 0.3, 8)
              for name in BATCH_FIELDS}
    starts = np.concatenate([[0], np.cumsum(lengths)[:-1]])
    conns = [(int(a + k), int(a + k + 1), 10.0)
             for a, ln in zip(starts, lengths) for k in range(int(ln) - 1)]
    paced = [int(a + k) for a in starts for k in range(5)]
    per_cell = {name: np.repeat(v, lengths) for name, v in fields.items()}
    return lengths, fields, conns, paced, per_cell


@pytest.mark.gpu
@pytest.mark.parametrize('mode', ['fp64', 'fp64-graphs', 'fp32+kahan'])
def test_cable_batch_matches_reference_connections(decker, mode):
    # 8 cables of 20-60 cells, three conductances per cable, the first 5
    # cells of each paced, dt 0.01 ms over 6 ms (the paced upstroke)
    lengths, fields, conns, paced, per_cell = _cable_case(decker)
    n = int(lengths.sum())
    log = ['engine.time'] + ['%d.membrane.V' % c for c in range(n)]
    ref, st_ref = _oracle_1d(decker, n, conns, paced, per_cell, 0.01, 6, log)
    kw = {'precision': DP, 'rl': True}
    if mode == 'fp64-graphs':
        kw['steps_per_launch'] = 100     # CUDA-graph chunks, as batched
    elif mode == 'fp32+kahan':
        kw = {'precision': SP, 'rl': True, 'accumulate': 'kahan'}
    b = CableBatch(decker, lengths, _p(), conductance=10.0, paced_cells=5,
                   fields=fields, **kw)
    b.sim.set_step_size(0.01)
    d = b.sim.run(6, log=log, log_interval=0.5)
    assert np.array_equal(np.asarray(d['engine.time']),
                          np.asarray(ref['engine.time']))
    dv = max(float(np.max(np.abs(np.asarray(d[k]) - np.asarray(ref[k]))))
             for k in log[1:])
    st = b.sim.state_array().reshape(n, -1)
    assert max(np.asarray(ref[k]).max() for k in log[1:]) > 0
    if mode == 'fp32+kahan':
        assert dv <= 0.5          # mV: the compensated single-precision bar
    else:
        assert dv <= 1e-9
        rel = np.max(np.abs(st - st_ref) / (np.abs(st_ref) + 1e-12))
        assert rel <= 1e-9


@pytest.mark.gpu
def test_sheet_batch_matches_reference_connections(decker):
    # Three sheets of uneven size packed in one 2D grid against one 1D
    # reference simulation whose connections form each sheet's grid
    shapes = [(40, 12), (33, 20), (17, 7)]
    g = (9.0, 6.0)
    vals = {'ina.Gbar': [1.1, 0.8, 1.3], 'ikr.Gbar': [0.7, 1.2, 1.0]}
    vals = {k: [x * decker.get(k).eval() for x in v] for k, v in vals.items()}
    offs = np.concatenate([[0], np.cumsum([w * h for w, h in shapes])[:-1]])
    conns, paced = [], []
    per_cell = {k: [] for k in vals}
    for i, ((w, h), o) in enumerate(zip(shapes, offs)):
        for y in range(h):
            for x in range(w):
                c = int(o + x + y * w)
                if x + 1 < w:
                    conns.append((c, c + 1, g[0]))
                if y + 1 < h:
                    conns.append((c, c + w, g[1]))
                if x < 3:
                    paced.append(c)
        for k in vals:
            per_cell[k].extend([vals[k][i]] * (w * h))
    ncell = int(sum(w * h for w, h in shapes))
    probe = [(0, 0, 0), (0, 39, 11), (1, 16, 10), (1, 32, 19), (2, 8, 6)]
    okeys = ['%d.membrane.V' % int(offs[i] + x + y * shapes[i][0])
             for i, x, y in probe]
    ref, st_ref = _oracle_1d(decker, ncell, conns, paced, per_cell, 0.005,
                             5, ['engine.time'] + okeys)
    b = SheetBatch(decker, shapes, _p(), conductance=g, paced_columns=3,
                   fields=vals, precision=DP, rl=True)
    bkeys = ['%d.%d.membrane.V' % (b.x0[i] + x, y) for i, x, y in probe]
    d = b.sim.run(5, log=['engine.time'] + bkeys, log_interval=0.5)
    for ok, bk in zip(okeys, bkeys):
        assert np.max(np.abs(np.asarray(d[bk]) - np.asarray(ref[ok]))) \
            <= 1e-9
    for i, ((w, h), o) in enumerate(zip(shapes, offs)):
        one = st_ref[o:o + w * h].reshape(h, w, -1)
        got = b.sheet_state(i)
        rel = np.max(np.abs(got - one) / (np.abs(one) + 1e-12))
        assert rel <= 1e-9, i


def test_reference_cable_chains_equal_conductance_field(decker):
    # In the oracle, the connection chains that express a batch of cables
    # and the heterogeneous conductances with zeros between cables (the
    # form CableBatch uses) give the same tissue, bit for bit
    from oracle.refsim import ReferenceCpuSimulation
    lengths, fields, conns, paced, per_cell = _cable_case(decker)
    n = int(lengths.sum())
    log = ['engine.time'] + ['%d.membrane.V' % c for c in range(0, n, 7)]
    ref, st_ref = _oracle_1d(decker, n, conns, paced, per_cell, 0.01, 3, log)
    s = ReferenceCpuSimulation(decker, _p(), ncells=n, precision=DP, rl=True)
    s.set_step_size(0.01)
    starts = np.concatenate([[0], np.cumsum(lengths)[:-1]])
    g = np.full(n - 1, 10.0)
    g[starts[1:] - 1] = 0
    s.set_conductance_field(g)
    s.set_paced_cell_list(paced)
    for k, v in per_cell.items():
        s.set_field(k, v)
    d = s.run(3, log=log, log_interval=0.5)
    for k in log:
        assert np.array_equal(np.asarray(d[k]), np.asarray(ref[k])), k
    assert np.array_equal(np.asarray(s.state()).reshape(n, -1), st_ref)


_CONFIG_REF = {}


@pytest.mark.gpu
@pytest.mark.parametrize('mode', ['fp64', 'fp32+kahan'])
def test_batched_cables_configuration_vs_reference(decker, mode):
    # The benchmark's batch at its own size: 512 cables of 50-2000 cells
    # (5.2e5 cells, seed 3), six conductances per cable, the first 5 cells
    # of each paced, dt 0.01 ms, over 2 ms (200 steps, the paced upstroke
    # included), against one 1D oracle simulation with connection chains
    # (computed once for both modes)
    import bench
    rng = np.random.default_rng(3)
    lengths = rng.integers(50, 2001, 512)
    fields = {name: decker.get(name).eval() * rng.lognormal(0, 0.3, 512)
              for name in bench.CABLE_FIELDS}
    starts = np.concatenate([[0], np.cumsum(lengths)[:-1]])
    n = int(lengths.sum())
    conns = [(int(a + k), int(a + k + 1), 10.0)
             for a, ln in zip(starts, lengths) for k in range(int(ln) - 1)]
    paced = [int(a + k) for a in starts for k in range(5)]
    per_cell = {name: np.repeat(v, lengths) for name, v in fields.items()}
    cells = sorted(set([0, n - 1] + [int(a + k) for a in starts[::37]
                                      for k in (0, 4, 5, 40)]))
    log = ['engine.time'] + ['%d.membrane.V' % c for c in cells]
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    if 'ref' not in _CONFIG_REF:
        _CONFIG_REF['ref'] = _oracle_1d(decker, n, conns, paced, per_cell,
                                        0.01, 2, log, p)
    ref, st_ref = _CONFIG_REF['ref']
    kw = {'precision': DP} if mode == 'fp64' else {
        'precision': SP, 'accumulate': 'kahan'}
    b = CableBatch(decker, lengths, p, conductance=10.0, paced_cells=5,
                   fields=fields, rl=True, steps_per_launch=100, **kw)
    b.sim.set_step_size(0.01)
    d = b.sim.run(2, log=log, log_interval=0.5)
    dv = max(float(np.max(np.abs(np.asarray(d[k], dtype=float) -
                                 np.asarray(ref[k])))) for k in log[1:])
    st = b.sim.state_array().reshape(n, -1)
    i_vm = decker.label('membrane_potential').index()
    fv = float(np.max(np.abs(st[:, i_vm] - st_ref[:, i_vm])))
    assert max(np.asarray(ref[k]).max() for k in log[1:]) > 0
    if mode == 'fp64':
        assert dv <= 1e-9 and fv <= 1e-9
        scale = np.max(np.abs(st_ref), axis=0) + 1e-300
        assert np.max(np.abs(st - st_ref) / scale) <= 1e-9
    else:
        assert dv <= 0.5 and fv <= 0.5
