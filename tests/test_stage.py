"""
Warp-tile staging with TMA tensor copies: the host library and the exporter
lay out a staged tile the same way (CPU), and on the GPU a staged kernel
gives bit-identical results to the kernel that loads from global memory,
and matches the oracle in double precision.
"""
import ctypes

import numpy as np
import pytest

from conftest import load, myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib, exporter

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION
FP64_TOL = 1e-9


# (real, n_state, i_vm, n_field, n_hi, hi_mode, v_double, diffusion, two_d,
#  nx, ny)
LAYOUTS = [
    (4, 48, 0, 0, 0, 0, 0, exporter.DIFF_GRID, 1, 512, 512),
    (4, 48, 0, 2, 8, 2, 0, exporter.DIFF_GRID, 1, 510, 300),
    (4, 48, 0, 2, 8, 1, 1, exporter.DIFF_GRID, 1, 64, 64),
    (4, 48, 0, 2, 7, 1, 0, exporter.DIFF_HETERO, 1, 33, 40),
    (8, 8, 0, 1, 0, 0, 0, exporter.DIFF_GRID, 0, 5000, 1),
    (4, 19, 3, 6, 4, 2, 0, exporter.DIFF_HETERO, 0, 520262, 1),
    (8, 41, 40, 0, 0, 0, 0, exporter.DIFF_CONN, 0, 900, 1),
    (4, 1, 0, 0, 0, 0, 0, exporter.DIFF_GRID, 1, 30, 30),
    (4, 12, -1, 3, 0, 0, 0, exporter.DIFF_NONE, 0, 4096, 1),
]


@pytest.mark.parametrize('case', LAYOUTS)
def test_host_and_exporter_layouts_agree(case):
    (real, ns, ivm, nf, nhi, hmode, vdbl, diff, two_d, nx, ny) = case
    cfg = _lib.MkgConfig()
    cfg.nx, cfg.ny = nx, ny
    cfg.real_bytes, cfg.n_state, cfg.n_field, cfg.i_vm = real, ns, nf, ivm
    cfg.diffusion, cfg.two_d = diff, two_d
    cfg.hi_mode, cfg.n_hi, cfg.v_double, cfg.stage = hmode, nhi, vdbl, 1
    out = (ctypes.c_int64 * 7)()
    lib = _lib.load()
    assert lib.mkg_stage_layout(ctypes.byref(cfg), out) == 0
    grid = diff in (exporter.DIFF_GRID, exporter.DIFF_HETERO)
    t2 = bool(two_d) and grid
    lay = exporter.stage_layout(
        real, ns, ivm if diff != exporter.DIFF_NONE else -1, nf, nhi,
        8 if hmode == 1 else real, 8 if vdbl else real,
        (3 if t2 else 1) if grid else 0,
        diff == exporter.DIFF_HETERO and not t2, t2 and nx % 4 != 0)
    assert list(out) == [lay['sw'], lay['lo'], lay['np'], lay['v_rows'],
                         lay['gx'], lay['bytes'], lay['tx']]
    # Every copy starts 16-byte aligned and is a whole number of 16 bytes
    assert (lay['sw'] * real) % 16 == 0 and (lay['vw'] * real) % 16 == 0
    for k in ('state_off', 'hi_off', 'field_off', 'v_off', 'gx_off'):
        assert lay[k] % 128 == 0


def test_layout_zero_without_staging():
    cfg = _lib.MkgConfig()
    cfg.nx, cfg.ny, cfg.real_bytes, cfg.n_state = 100, 1, 4, 8
    out = (ctypes.c_int64 * 7)(*([1] * 7))
    assert _lib.load().mkg_stage_layout(ctypes.byref(cfg), out) == 0
    assert list(out) == [0] * 7


def test_kernels_stage_only_large_grids(br77):
    for n, staged in ((200, False), (300, True)):
        s = mg.SimulationCUDA(br77, None, ncells=n)
        assert bool(s._kernel([]).layout) == staged
    s = mg.SimulationCUDA(br77, None, ncells=1000, stage_tiles=False)
    assert s._kernel([]).layout is None


def test_two_buffer_staging_compiles_and_falls_back(decker):
    # Two buffers per warp where they fit (the CTA's staging memory under
    # the cap), one otherwise; the host sizes shared memory from the
    # simulation's configuration (mkg_config.stage = buffers)
    for block, bufs in ((256, 2), (640, 1)):
        s = mg.SimulationCUDA(decker, None, ncells=(64, 32), rl=True,
                              block=block, min_blocks=1)
        s._stage_lazy = 2
        k = s._kernel([])
        assert k.layout is not None and k.stage_buffers == bufs
        assert ('#define STAGE_BUFS %d' % bufs) in k.source()
        assert k.stage_lazy == bufs
        cubin, _ = _lib.compile_source(k.source(), k.options())
        assert cubin[:4] == b'\x7fELF'
    with pytest.raises(ValueError):
        exporter.TissueKernel(
            decker, myokit.SINGLE_PRECISION, False, {}, [], 0, False, [], {},
            (256, 1), stage=True, stage_lazy=3)


@pytest.mark.parametrize('mode', [
    (SP, None), (SP, 'kahan'), (SP, 'double'), (myokit.DOUBLE_PRECISION,
                                                 None)],
    ids=['fp32', 'kahan', 'double', 'fp64'])
def test_every_staging_and_sync_mode_compiles(br77, mode):
    # Direct loads, prefetch, lazy with one or two buffers, each with the
    # grid barrier and with neighbour waits, 2D and 1D heterogeneous
    precision, acc = mode
    for ncells, hetero in (((48, 12), False), (600, True)):
        for lazy in (None, 0, 1, 2):
            for sync in ('barrier', 'neighbors'):
                s = mg.SimulationCUDA(br77, None, ncells=ncells, rl=True,
                                      precision=precision, accumulate=acc,
                                      stage_tiles=lazy is not None,
                                      block=128, min_blocks=1)
                s._stage_lazy = lazy or 0
                s._sync = sync
                if hetero:
                    s.set_conductance_field(np.full(599, 2.0), None)
                k = s._kernel([])
                assert (k.layout is not None) == (lazy is not None)
                assert k.sync == sync
                cubin, _ = _lib.compile_source(k.source(), k.options())
                assert cubin[:4] == b'\x7fELF'


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def _run(model, stage, ncells, precision=SP, rl=False, fields=None,
         gfield=None, conn=None, diffusion=True, dur=4.0, **kw):
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=0.5)
    lazy = {'lazy': 1, 'lazy2': 2}.get(stage, 0)
    s = mg.SimulationCUDA(model, p, ncells=ncells, precision=precision,
                          rl=rl, diffusion=diffusion, stage_tiles=bool(stage),
                          **kw)
    s._stage_lazy = lazy
    s.set_step_size(0.01)
    if diffusion and conn is None:
        if isinstance(ncells, tuple):
            s.set_paced_cells(3, ncells[1])
        else:
            s.set_paced_cells(5)
    for name, v in (fields or {}).items():
        s.set_field(name, v)
    if gfield is not None:
        s.set_conductance_field(*gfield)
    if conn is not None:
        s.set_connections(conn)
        s.set_paced_cell_list(list(range(5)))
    n = ncells[0] * ncells[1] if isinstance(ncells, tuple) else ncells
    probes = sorted(set([0, n // 3, n - 1]))
    nx = ncells[0] if isinstance(ncells, tuple) else n
    keys = ['engine.time'] + [
        ('%d.%d.membrane.V' % (c % nx, c // nx)) if isinstance(ncells, tuple)
        else ('%d.membrane.V' % c) for c in probes]
    d = s.run(dur, log=keys, log_interval=0.5)
    return s.state_array(), d


def _same(a, b):
    assert np.array_equal(a[0], b[0])
    for k in a[1].keys():
        assert np.array_equal(np.asarray(a[1][k]), np.asarray(b[1][k])), k


def _close(a, b, tol):
    # Lazy staging moves the shared-memory reads next to their uses, so the
    # compiler may contract other multiply-add pairs into FMAs: results
    # agree to rounding (tol in mV for V; relative for the state)
    worst = 0.0
    for k in a[1].keys():
        x, y = np.asarray(a[1][k]), np.asarray(b[1][k])
        worst = max(worst, float(np.max(np.abs(x - y))))
    assert worst <= tol, worst
    s = np.abs(a[0] - b[0]) / np.maximum(np.abs(a[0]), 1e-6)
    assert float(np.max(s)) <= 1e3 * tol, float(np.max(s))


def _fields(m, shape, names, seed=0):
    rng = np.random.default_rng(seed)
    return {n: m.get(n).eval() * rng.lognormal(0, 0.2, shape) for n in names}


@pytest.mark.gpu
@pytest.mark.parametrize('shape', [(64, 20), (37, 23), (33, 9), 1000, 257])
@pytest.mark.parametrize('precision', [SP, DP])
def test_staged_equals_direct_grid(decker, shape, precision):
    sh = shape[::-1] if isinstance(shape, tuple) else shape
    f = _fields(decker, sh, ['ikr.Gbar', 'ina.Gbar'])
    out = [_run(decker, st, shape, precision, rl=True, fields=f)
           for st in (False, True, 'lazy', 'lazy2')]
    _same(out[0], out[1])
    _close(out[0], out[2], 1e-3 if precision == SP else 1e-9)
    _close(out[0], out[3], 1e-3 if precision == SP else 1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize('acc', ['kahan', 'double'])
@pytest.mark.parametrize('shape', [(48, 16), (45, 13)])
def test_staged_equals_direct_accumulate(decker, acc, shape):
    f = _fields(decker, shape[::-1], ['ikr.Gbar'])
    out = [_run(decker, st, shape, SP, rl=True, fields=f, accumulate=acc)
           for st in (False, True, 'lazy', 'lazy2')]
    _same(out[0], out[1])
    _close(out[0], out[2], 1e-3)
    _close(out[0], out[3], 1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize('block', [512, 640])
def test_lazy_staging_with_wide_ctas(decker, block):
    f = _fields(decker, (40, 70), ['ikr.Gbar'])
    out = [_run(decker, st, (70, 40), SP, rl=True, fields=f, block=block,
                min_blocks=1) for st in (False, 'lazy')]
    _close(out[0], out[1], 1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize('shape', [(40, 12), (41, 11), 700])
def test_staged_equals_direct_hetero(br77, shape):
    rng = np.random.default_rng(5)
    if isinstance(shape, tuple):
        nx, ny = shape
        g = (rng.uniform(5, 10, (ny, nx - 1)), rng.uniform(2, 6, (ny - 1, nx)))
    else:
        g = (rng.uniform(5, 10, shape - 1),)
        g[0][::97] = 0     # separate cables
    out = [_run(br77, st, shape, DP, gfield=g)
           for st in (False, True, 'lazy')]
    _same(out[0], out[1])
    _close(out[0], out[2], 1e-9)


@pytest.mark.gpu
def test_staged_equals_direct_connections_and_no_diffusion(br77):
    n = 600
    conn = [(i, i + 1, 7.0) for i in range(n - 1)] + [
        (i, i + 37, 1.5) for i in range(0, n - 37, 11)]
    out = [_run(br77, st, n, DP, conn=conn) for st in (False, True)]
    _same(out[0], out[1])
    out = [_run(br77, st, 512, DP, diffusion=False) for st in (False, True)]
    _same(out[0], out[1])


@pytest.mark.gpu
@pytest.mark.parametrize('shape', [(20, 16), (17, 19)])
def test_staged_matches_oracle_fp64(br77, shape):
    from oracle.refsim import ReferenceCpuSimulation
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=0.5)
    res = []
    for cls in (ReferenceCpuSimulation, mg.SimulationCUDA):
        s = cls(br77, p, ncells=shape, precision=DP)
        s.set_step_size(0.01)
        s.set_paced_cells(2, shape[1])
        s.set_conductance(9, 5)
        d = s.run(8, log=['engine.time', 'membrane.V'], log_interval=0.5)
        res.append(d)
        if cls is mg.SimulationCUDA:
            assert s._last_kernel.layout is not None
    worst = 0.0
    for k in res[0].keys():
        worst = max(worst, float(np.max(np.abs(
            np.asarray(res[0][k]) - np.asarray(res[1][k])))))
    assert worst < FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize('stage', [False, True, 'lazy', 'lazy2'])
@pytest.mark.parametrize('shape', [(64, 20), (37, 23), 1000, (2000, 1),
                                   (3, 400), 300])
def test_neighbour_sync_equals_grid_barrier(decker, stage, shape):
    # Waiting only for the warps that own a warp's halo tiles gives the
    # same results as a grid-wide barrier between steps
    out = []
    for sync in ('barrier', 'neighbors'):
        p = myokit.pacing.blocktrain(period=1000, duration=2, offset=0.5)
        s = mg.SimulationCUDA(decker, p, ncells=shape, rl=True,
                              stage_tiles=bool(stage), block=64,
                              min_blocks=1)
        s._stage_lazy = {'lazy': 1, 'lazy2': 2}.get(stage, 0)
        s._sync = sync
        if isinstance(shape, tuple):
            s.set_paced_cells(3, shape[1])
        else:
            s.set_paced_cells(5)
        s.set_step_size(0.01)
        d = s.run(4, log=['engine.time', 'membrane.V'], log_interval=0.5)
        assert s._last_kernel.sync == sync
        out.append((s.state_array(), d))
    _same(out[0], out[1])


@pytest.mark.gpu
@pytest.mark.parametrize('shape', [(64, 40), (64, 400), (32, 900)])
def test_neighbour_sync_nan_halt(shape):
    # A NaN halt stops every warp after the halting step, with neighbour
    # synchronisation as with the grid barrier. On tall grids most warps
    # are many halo rows away from the warp that records the halt (the
    # owner of cell 0); they must still leave after the halting step: no
    # timeout, and the same final state.
    import test_oracle as to
    msgs = []
    states = []
    for sync in ('barrier', 'neighbors'):
        p = myokit.Protocol()
        p.schedule(start=0, level=-80, duration=1.234)
        p.schedule(start=1.234, level=-47.13, duration=1000)
        s = mg.SimulationCUDA(to._nan_model(), p, ncells=shape, block=64,
                              min_blocks=1)
        s.set_paced_cell_list([[1, 1]])
        s._sync = sync
        s._steps_per_launch = 7
        with pytest.raises(myokit.SimulationError) as e:
            s.run(5)
        assert s._last_kernel.sync == sync
        msgs.append(str(e.value))
        s.reset()
        s.run(5, report_nan=False)
        states.append(s.state_array())
    assert 'Time:  1.23' in msgs[0]
    assert msgs[0] == msgs[1]
    assert np.array_equal(states[0], states[1], equal_nan=True)
