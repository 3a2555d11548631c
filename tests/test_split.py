"""
Split warp tiles: on grids with fewer warp tiles than SMs, a team of 2 to
16 warps shares each tile's work (every warp updates its own share of the
states and computes additive terms of other warps' derivatives, with the
equations those need). Teams of 2 or 4 warps are part of one CTA; teams of
8 or 16 are clusters of 2 or 4 CTAs exchanging partial sums through
distributed shared memory. The results are those of the unsplit kernel (to
rounding: the derivatives are summed in another order, and the compiler
may contract a different set of multiply-adds in a part's smaller body)
and of the reference.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load, myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION


def _cable(model, precision, split, block, rl=False, n=200):
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = mg.SimulationCUDA(model, p, ncells=n, precision=precision, rl=rl,
                          block=block)
    s._split = split
    s.set_step_size(0.005)
    s.set_conductance(9)
    s.set_paced_cells(5)
    return s


@pytest.mark.parametrize('name,rl', [('beeler-1977-model.mmt', False),
                                     ('decker-2009.mmt', True),
                                     ('lr-1991.mmt', False)])
@pytest.mark.parametrize('split,block', [(2, 64), (4, 128), (4, 256),
                                         (8, 128), (16, 128), (8, 64)])
def test_split_partition_and_compile(name, rl, split, block):
    # Every state is updated by exactly one warp of the team, the shares
    # are balanced, and the kernel compiles for sm_103a
    m = load(name)
    s = _cable(m, DP, split, block, rl=rl)
    k = s._kernel([])
    assert k.split == split
    assert k.split_cl == max(1, split * 32 // block)
    src = k.source()
    assert k.split_body in src
    for i, st in enumerate(k.states):
        target = 'vout[cid] =' if i == k.i_vm else \
            'state[(long long)%d * pitch + cid] =' % i
        assert k.split_body.count(target) == 1, st.qname()
    assert k.split_body.count('mkg_team_sync();') == split
    assert max(k.split_costs) <= 0.7 * sum(k.split_costs)
    # dV/dt is divided into its currents (no equation refers to it)
    assert k.split_terms['membrane.V'] >= 4
    # Remote stores only across the CTAs of a cluster
    assert ('MKG_PP_PUT(' in k.split_body) == (k.split_cl > 1)
    cubin, _ = _lib.compile_source(src, k.options())
    assert cubin[:4] == b'\x7fELF'


def test_split_shares_of_the_br77_cable(br77):
    # Beeler-Reuter 1977: dV/dt alone is 27% of a cell's work, so teams
    # larger than 4 warps only pay with its currents divided among them
    largest = {}
    for split in (2, 4, 8, 16):
        s = _cable(br77, DP, split, 128)
        k = s._kernel([])
        largest[split] = max(k.split_costs) / sum(k.split_costs)
    assert largest[4] < 0.26
    assert largest[8] < 0.15
    assert largest[16] < 0.11


def test_split_falls_back_where_unsupported(br77):
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    # Accumulation planes
    s = mg.SimulationCUDA(br77, p, ncells=100, accumulate='kahan', block=128)
    s._split = 4
    assert s._kernel([]).split == 1
    # A CTA that does not hold whole teams, a team that is not whole CTAs
    s = mg.SimulationCUDA(br77, p, ncells=100, block=96)
    s._split = 4
    assert s._kernel([]).split == 1
    s._split = 8
    assert s._kernel([]).split == 1
    # Clusters of more than 8 CTAs
    s = mg.SimulationCUDA(br77, p, ncells=100, block=32)
    s._split = 16
    assert s._kernel([]).split == 1
    s._split = 8
    assert s._kernel([]).split_cl == 8
    s._split = 3
    with pytest.raises(ValueError, match='split must be'):
        s._kernel([])


@pytest.mark.gpu
@pytest.mark.parametrize('split,block', [(2, 64), (4, 128), (4, 256),
                                         (8, 128), (16, 128), (8, 64)])
def test_split_cable200_matches_golden(br77, split, block):
    # The 200-cell FP64 cable against the reference's Simulation1d
    g = np.load(os.path.join(GOLDEN, 'br77_cable200_sim1d.npz'))
    s = _cable(br77, DP, split, block)
    d = s.run(20, log=['engine.time', 'membrane.V'], log_interval=1).npview()
    assert s._last_kernel.split == split
    assert np.max(np.abs(d['engine.time'] - g['engine_time'])) == 0
    worst = max(np.max(np.abs(d['membrane.V', c] - g['%d_membrane_V' % c]))
                for c in range(200))
    assert worst < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize('split', [4, 16])
def test_split_graph_chunks_match_golden(br77, split):
    # Launches of 100 steps replayed from CUDA graphs (cooperative cluster
    # launches captured in a graph for 16 warps per tile)
    g = np.load(os.path.join(GOLDEN, 'br77_cable200_sim1d.npz'))
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = mg.SimulationCUDA(br77, p, ncells=200, precision=DP, block=128,
                          steps_per_launch=100)
    s._split = split
    s.set_step_size(0.005)
    s.set_conductance(9)
    s.set_paced_cells(5)
    d = s.run(20, log=['engine.time', 'membrane.V'], log_interval=1).npview()
    assert s._last_kernel.split == split
    assert s.last_run_stats()['launches'] >= 40
    worst = max(np.max(np.abs(d['membrane.V', c] - g['%d_membrane_V' % c]))
                for c in range(200))
    assert worst < 1e-9


def _same(a, b, n_state, rtol, vtol):
    # States: relative to each state's largest magnitude over the cells
    # (gates and concentrations span many decades); logs: absolute (mV)
    (sa, da), (sb, db) = a, b
    sa = sa.reshape(-1, n_state)
    sb = sb.reshape(-1, n_state)
    scale = np.max(np.abs(sb), axis=0) + 1e-300
    assert np.max(np.abs(sa - sb) / scale) <= rtol
    for k in da.keys():
        assert np.max(np.abs(np.asarray(da[k], dtype=float) -
                             np.asarray(db[k], dtype=float))) <= vtol, k


@pytest.mark.gpu
@pytest.mark.parametrize('precision', [DP, SP])
@pytest.mark.parametrize('case', ['cable', 'sheet', 'hetero', 'connections',
                                  'logged-inter'])
def test_split_equals_unsplit(decker, precision, case):
    out = []
    splits = (1, 2, 4, 8, 16)
    for split in splits:
        p = myokit.pacing.blocktrain(period=1000, duration=2, offset=0.5)
        shape = (70, 6) if case == 'sheet' else 150
        s = mg.SimulationCUDA(decker, p, ncells=shape, precision=precision,
                              rl=True, block=128)
        s._split = split
        if case == 'sheet':
            s.set_paced_cells(3, 6)
        else:
            s.set_paced_cells(5)
        if case == 'hetero':
            s.set_conductance_field(np.linspace(5, 12, 149))
        elif case == 'connections':
            s.set_connections([(i, i + 1, 9.0) for i in range(149)] +
                              [(3, 90, 2.0)])
        s.set_step_size(0.01)
        log = ['engine.time', 'membrane.V']
        if case == 'logged-inter':
            log += ['ina.INa', 'ical.ICaL']
        d = s.run(4, log=log, log_interval=0.5)
        assert s._last_kernel.split == split
        out.append((s.state_array(), d))
    # FP64: rounding only (the derivatives' terms are summed in another
    # order; 2e-11 after the upstroke), within the bar the oracle parity
    # tests hold double precision to; FP32: the compiler contracts
    # different multiply-adds in a part's body, and single precision
    # rounding grows over 400 steps
    rtol, vtol = (1e-9, 1e-9) if precision == DP else (2e-3, 1e-2)
    n = decker.count_states()
    for o in out[1:]:
        _same(out[0], o, n, rtol, vtol)


@pytest.mark.gpu
@pytest.mark.parametrize('split', [4, 8])
def test_split_nan_halt(split):
    import test_oracle as to
    s = to.nan_sim(mg.SimulationCUDA)
    s._block = 128
    s._split = split
    with pytest.raises(myokit.SimulationError, match='Time:  1.23'):
        s.run(5)
    assert s._last_kernel.split == split


@pytest.mark.gpu
def test_adjoint_of_a_split_simulation(br77):
    # The adjoint's trajectory kernel is never split; on a handle made for
    # a split kernel it gets the same gradients as on an unsplit one
    from myokit_gb300 import adjoint
    out = []
    for split in (1, 4, 8):
        p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1)
        s = mg.SimulationCUDA(br77, p, ncells=100, precision=DP, block=128)
        s._split = split
        s.set_paced_cells(3)
        s.set_field('isi.gsBar', np.linspace(0.07, 0.11, 100))
        s.run(0.5)
        assert s._last_kernel.split == split
        adj = adjoint.TissueAdjoint(s, [0, 40, 99], segment_steps=50)
        target = np.zeros((24, 3)) - 80
        out.append(adj.loss_and_gradient(12, target, 0.5))
    L1, g1 = out[0]
    for L4, g4 in out[1:]:
        assert abs(L4 - L1) <= 1e-12 * abs(L1)
        np.testing.assert_allclose(g4['isi.gsBar'], g1['isi.gsBar'],
                                   rtol=1e-9, atol=1e-12 * abs(L1))
        assert abs(g4['gx'] - g1['gx']) <= 1e-9 * abs(g1['gx'])


@pytest.mark.parametrize('name,rl', [('beeler-1977-model.mmt', False),
                                     ('decker-2009.mmt', True),
                                     ('lr-1991.mmt', False)])
def test_divided_derivatives_add_up(name, rl):
    # The terms a split kernel spreads over its warps add up to the
    # derivative they come from: evaluated in double precision at the
    # model's initial state, sum(c_k * T_k) equals dx/dt to rounding
    s = _cable(load(name), DP, 8, 128, rl=rl)
    k = s._kernel([])
    assert k.split_term_exprs
    m = k.model     # the simulation's own copy, whose variables terms use
    # Values of every variable at the initial state, with pacing on and
    # no diffusion current, in solvable order
    sub = {}
    for v, x in zip(m.states(), m.initial_values(as_floats=True)):
        sub[myokit.Name(v)] = myokit.Number(x)
    for label, value in (('pace', 1.0), ('diffusion_current', 0.0),
                         ('time', 0.0)):
        v = m.binding(label)
        if v is not None:
            sub[myokit.Name(v)] = myokit.Number(value)
    for group in m.solvable_order().values():
        for eq in group.equations(const=None):
            if eq.lhs.var() in [x.var() for x in sub] and \
                    not isinstance(eq.lhs, myokit.Derivative):
                continue
            val = eq.rhs.eval(subst=sub)
            sub[eq.lhs] = myokit.Number(val)
    checked = 0
    for qname, terms in k.split_term_exprs.items():
        v = m.get(qname)
        d = sub[myokit.Derivative(myokit.Name(v))].eval()
        total = sum(c * e.eval(subst=sub) for c, e in terms)
        assert total == pytest.approx(d, rel=1e-12, abs=1e-12 * (
            1 + sum(abs(c * e.eval(subst=sub)) for c, e in terms))), qname
        checked += 1
    assert checked >= 1


def _slot_check(k):
    """Static checks of a split body's partial-sum hand-over: every slot is
    written by one warp other than its reader, with a remote store exactly
    when the two are in different CTAs of the cluster, and read by one
    owner; indices and ranks are in range."""
    import re
    nwarp = k.block[0] // 32
    parts = re.split(r'\n\s*(?:else )?if \(part_ == (\d+)\) \{', '\n' +
                     k.split_body)
    assert [int(p) for p in parts[1::2]] == list(range(k.split))
    writes, reads = {}, {}
    for p, body in zip(parts[1::2], parts[2::2]):
        p = int(p)
        for slot in re.findall(r'MKG_PP_LOCAL\((\d+),', body):
            writes.setdefault(int(slot), []).append((p, None))
        for slot, rank in re.findall(r'MKG_PP_PUT\((\d+), (\d+),', body):
            writes.setdefault(int(slot), []).append((p, int(rank)))
        for slot in re.findall(r'MKG_PP_GET\((\d+)\)', body):
            reads.setdefault(int(slot), []).append(p)
        # the team barrier comes after every hand-over and before every read
        sync = body.index('mkg_team_sync();')
        assert 'MKG_PP_GET' not in body[:sync]
        assert 'MKG_PP_PUT' not in body[sync:]
        assert 'MKG_PP_LOCAL' not in body[sync:]
    assert sorted(writes) == sorted(reads) == list(range(k.split_nslot))
    for slot in writes:
        (w, rank), = writes[slot]
        (r,) = reads[slot]
        assert w != r
        if rank is None:
            assert k.split_cl == 1 or w // nwarp == r // nwarp
        else:
            assert k.split_cl > 1 and rank == r // nwarp != w // nwarp
            assert 0 <= rank < k.split_cl


@pytest.mark.parametrize('split,block', [(4, 128), (8, 128), (16, 64)])
def test_split_hand_over_of_every_model(split, block):
    # Every model of myokit's test data that the simulation accepts:
    # the partial-sum slots are consistent and the kernel compiles
    import test_models as tm
    for name in tm.ACCEPTED:
        m = tm._model(name)
        p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
        s = mg.SimulationCUDA(m, p, ncells=100, precision=DP, block=block)
        s._split = split
        k = s._kernel([])
        assert k.split == split, name
        _slot_check(k)
        cubin, _ = _lib.compile_source(k.source(), k.options())
        assert cubin[:4] == b'\x7fELF', name
