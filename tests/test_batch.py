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
