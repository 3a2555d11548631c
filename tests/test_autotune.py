"""
Host logic of the launch-shape autotuner (CPU): configuration signatures,
the lookup order (user cache, then the shipped table), how a simulation
created without a launch shape takes the table's choice, and the validity
of the shipped table and of the candidate lists. Timing the candidates
needs a GPU (``tests/test_parity_gpu.py`` checks that tuning changes no
result).
"""
import json
import os

import numpy as np
import pytest

from conftest import myokit
import myokit_gb300 as mg
from myokit_gb300 import autotune as at

SP = myokit.SINGLE_PRECISION
DP = myokit.DOUBLE_PRECISION


@pytest.fixture
def empty_cache(tmp_path, monkeypatch):
    monkeypatch.setenv('MYOKIT_GB300_CACHE', str(tmp_path))
    return tmp_path


def _bench_sheet(decker, **kw):
    # The 512 x 512 bench sheet: Rush-Larsen, dt 0.005, GKr/GNa fields
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = mg.SimulationCUDA(decker, p, ncells=(512, 512), rl=True, **kw)
    s.set_step_size(0.005)
    s.set_paced_cells(nx=4, ny=512, x=0, y=0)
    ones = np.ones((512, 512))
    s.set_field('ikr.Gbar', decker.get('ikr.Gbar').eval() * ones)
    s.set_field('ina.Gbar', decker.get('ina.Gbar').eval() * ones)
    return s


def test_signature_separates_configurations(decker):
    base = at.signature(_bench_sheet(decker))
    assert base.startswith('Decker2009|')
    assert '|512|512|' in base
    others = [
        _bench_sheet(decker, accumulate='kahan'),
        _bench_sheet(decker, fp32_math='ieee'),
        _bench_sheet(decker, stage_tiles=False),
        _bench_sheet(decker, precision=DP),
        mg.SimulationCUDA(decker, None, ncells=(512, 256), rl=True),
    ]
    sigs = [at.signature(s) for s in others]
    assert base not in sigs and len(set(sigs)) == len(sigs)


def test_shipped_table_is_used_without_a_launch_shape(decker, empty_cache):
    s = _bench_sheet(decker)
    hit = at.lookup(s)
    assert hit is not None
    with open(at._shipped_path()) as f:
        assert json.load(f)[at.signature(s)] == hit
    k = s._kernel([])
    assert k.block == tuple(hit['block'])
    assert k.min_blocks == hit['min_blocks']
    assert k.stage_lazy == int(hit['stage_lazy'])
    assert k.sync == hit['sync']
    # An explicit launch shape wins over the table
    s2 = _bench_sheet(decker, block=128, min_blocks=1)
    k2 = s2._kernel([])
    assert k2.block == (128, 1) and k2.min_blocks == 1


def test_user_cache_wins_over_shipped_table(decker, empty_cache):
    s = _bench_sheet(decker)
    entry = {'block': [384, 1], 'min_blocks': 1, 'steps_per_launch': 0,
             'stage_lazy': 0, 'sync': 'neighbors', 'rate': 1.0,
             'when': 'test'}
    with open(os.path.join(str(empty_cache), 'tune.json'), 'w') as f:
        json.dump({at.signature(s): entry}, f)
    s = _bench_sheet(decker)
    assert at.lookup(s) == entry
    k = s._kernel([])
    assert k.block == (384, 1) and k.stage_lazy == 0
    assert k.sync == 'neighbors'


def test_apply_sets_every_field(decker):
    s = _bench_sheet(decker)
    at._apply(s, (640, 1), 1, 0, 2, 'neighbors')
    assert s._block == (640, 1) and s._min_blocks == 1
    assert s._steps_per_launch == 0 and s._stage_lazy == 2
    assert s._sync == 'neighbors'
    k = s._kernel([])
    # Two buffers of 20 warps would exceed the staging cap: one buffer
    assert k.block == (640, 1) and k.stage_buffers == 1


def test_shipped_table_and_candidates_are_valid():
    with open(at._shipped_path()) as f:
        table = json.load(f)
    assert len(table) >= 8
    for sig, e in table.items():
        assert e['block'][0] % 32 == 0 and e['block'][1] == 1, sig
        assert 32 <= e['block'][0] <= 1024
        assert e['block'][0] * e['min_blocks'] <= 2048, sig
        assert int(e['stage_lazy']) in (0, 1, 2)
        assert e['sync'] in ('barrier', 'neighbors')
        assert e['steps_per_launch'] >= 0 and e['rate'] > 0
    for cands in (at._CANDIDATES, at._CANDIDATES_FP64):
        assert len(set(cands)) == len(cands)
        for (bx, by), mb, spl, lazy, sync in cands:
            assert bx % 32 == 0 and by == 1 and bx * mb <= 2048
            assert int(lazy) in (0, 1, 2) and spl >= 0
            assert sync in ('barrier', 'neighbors')


def test_split_candidates_by_precision(br77):
    # Small grids try split tiles; cluster teams (8 and 16 warps of
    # 128-thread CTAs) only in double precision
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    dp = mg.SimulationCUDA(br77, p, ncells=200,
                           precision=myokit.DOUBLE_PRECISION)
    sp = mg.SimulationCUDA(br77, p, ncells=200)
    kahan = mg.SimulationCUDA(br77, p, ncells=200, accumulate='kahan')
    big = mg.SimulationCUDA(br77, p, ncells=(512, 512),
                            precision=myokit.DOUBLE_PRECISION)

    def splits(s):
        return sorted(c[5] for c in at._candidates(s) if len(c) > 5)
    assert splits(dp) == [2, 2, 4, 4, 8, 16]
    assert splits(sp) == [2, 2, 4, 4]
    assert splits(kahan) == []
    assert splits(big) == []
    for c in at._CANDIDATES_SPLIT:
        (bx, by), mb, spl, lazy, sync, split = c
        nwarp = bx // 32
        assert (split <= nwarp and nwarp % split == 0) or (
            split % nwarp == 0 and split // nwarp <= 8)
