"""
Mixed precision: single precision right-hand side with selected states
accumulated in FP64 (``accumulate='double'``) or with a compensated FP32
update (``accumulate='kahan'``), checked against the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import load, myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib, metrics
from oracle.refsim import ReferenceCpuSimulation

SP = myokit.SINGLE_PRECISION
DP = myokit.DOUBLE_PRECISION


def _sheet(cls, precision, n=12, **kw):
    m = load('decker-2009.mmt')
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = cls(m, p, ncells=(n, n), precision=precision, rl=True, **kw)
    s.set_paced_cells(nx=3, ny=n)
    rng = np.random.default_rng(4)
    s.set_field('ikr.Gbar', 0.0138542 * rng.lognormal(0, 0.2, (n, n)))
    s.set_field('ina.Gbar', 9.075 * rng.lognormal(0, 0.2, (n, n)))
    return s


def test_accumulate_arguments():
    m = load('beeler-1977-model.mmt')
    with pytest.raises(ValueError, match='accumulate'):
        mg.SimulationCUDA(m, accumulate='quad')
    with pytest.raises(ValueError, match='single precision'):
        mg.SimulationCUDA(m, precision=DP, accumulate='double')
    with pytest.raises(ValueError, match='must be states'):
        mg.SimulationCUDA(m, accumulate='double',
                          accumulate_states=['ina.INa'])
    s = mg.SimulationCUDA(m, accumulate='kahan')
    names = [v.qname() for v in s.accumulated_states()]
    assert names == ['membrane.V', 'calcium.Cai']
    s = mg.SimulationCUDA(m, accumulate='double',
                          accumulate_states=['calcium.Cai'])
    assert [v.qname() for v in s.accumulated_states()] == ['calcium.Cai']


@pytest.mark.parametrize('acc', ['double', 'kahan'])
def test_accumulate_kernels_compile(acc):
    s = _sheet(mg.SimulationCUDA, SP, accumulate=acc)
    k = s._kernel([])
    assert len(k.hi_states) == 8
    assert k.bytes_per_cell_step() == 392 + 2 * 8 * 4
    cubin, _ = _lib.compile_source(k.source(), k.options())
    assert cubin[:4] == b'\x7fELF'


@pytest.mark.gpu
@pytest.mark.parametrize('acc', ['double', 'kahan'])
def test_accumulated_state_round_trip(acc):
    s = _sheet(mg.SimulationCUDA, SP, n=9, accumulate=acc)
    s.run(0.01)
    be = s._backend[1]
    n = s._nstate * s._ntotal
    rng = np.random.default_rng(0)
    x = np.ascontiguousarray(rng.normal(size=n) * 30)
    be.check(be.lib.mkg_set_state(be.h, _lib.dptr(x), n))
    y = np.empty(n)
    be.check(be.lib.mkg_get_state(be.h, _lib.dptr(y), n))
    hi = np.zeros(s._nstate, dtype=bool)
    hi[s._last_kernel.hi_states] = True
    hi = np.tile(hi, s._ntotal)
    # Accumulated states keep (nearly) all of their double precision
    if acc == 'double':
        assert np.array_equal(x[hi], y[hi])
    else:
        assert np.max(np.abs(x[hi] - y[hi]) / np.abs(x[hi])) < 1e-13
    # The others are rounded to single precision
    assert np.array_equal(y[~hi], x[~hi].astype(np.float32).astype(float))


@pytest.mark.gpu
def test_accumulation_against_fp64_oracle():
    keys = ['%d.%d.membrane.V' % (x, y) for x in (0, 5, 11)
            for y in (0, 6, 11)]
    log = ['engine.time'] + keys
    ref = _sheet(ReferenceCpuSimulation, DP).run(60, log=log,
                                                 log_interval=0.5)
    t = np.asarray(ref['engine.time'])
    tr = {k: np.asarray(ref[k]) for k in keys}
    res = {}
    for name, kw in (('fp32', {}), ('double', {'accumulate': 'double'}),
                     ('kahan', {'accumulate': 'kahan'})):
        d = _sheet(mg.SimulationCUDA, SP, **kw).run(60, log=log,
                                                     log_interval=0.5)
        res[name] = metrics.compare(t, {k: d[k] for k in keys}, tr)
    for name, r in res.items():
        assert r['max_abs_dV_mV'] < 0.5, (name, r)
        assert r['max_activation_error_ms'] < 0.05, (name, r)


def test_metrics_on_synthetic_action_potential():
    t = np.arange(0, 400, 0.5)
    v = -85 + 125 * ((t >= 10) & (t < 12)) * (t - 10) / 2
    v = np.where(t >= 12, -85 + 125 * np.exp(-(t - 12) / 80), v)
    v = np.where(t < 10, -85.0, v)
    assert abs(metrics.activation_time(t, v) - (10 + 2 * 55 / 125)) < 1e-9
    apd = metrics.apd90(t, v)
    # 90% repolarisation: exp(-(t-12)/80) = 0.1
    assert abs(apd - (12 + 80 * np.log(10) - (10 + 2 * 55 / 125))) < 0.5


@pytest.mark.gpu
@pytest.mark.parametrize('acc', [None, 'kahan'])
def test_conduction_drift_along_a_long_cable(acc):
    # A wave crossing 1000 Decker cells (one row of the paced-edge sheet):
    # single precision must not change the conduction velocity. Free Ca
    # from the trigonometric cubic formula loses most of its single
    # precision digits with a systematic bias; refined by Newton steps on
    # the cubic (exporter.cubic_root_coefficients) the activation times
    # stay within a microsecond of FP64 (with the formula alone they drift
    # by several, growing with distance).
    import bench
    n = 1000
    xs = list(range(0, n, 50)) + [n - 1]
    log = ['engine.time'] + ['%d.membrane.V' % x for x in xs]
    out = []
    for prec, kw in ((DP, {}), (SP, {'accumulate': acc})):
        s = bench.make_s1_cable(mg.SimulationCUDA, prec, n, **kw)
        if prec == SP:
            assert len(s._kernel([]).cubic) == 3
        out.append(s.run(220, log=log, log_interval=0.1))
    ref, got = out
    t = np.asarray(ref['engine.time'])
    errs = []
    for k in log[1:]:
        a = metrics.activation_time(t, np.asarray(got[k], dtype=float))
        b = metrics.activation_time(t, np.asarray(ref[k], dtype=float))
        assert np.isfinite(a) and np.isfinite(b), k
        errs.append(abs(a - b))
    assert max(errs) <= 1e-3          # ms
    c = metrics.compare(t, {k: np.asarray(got[k], dtype=float)
                            for k in log[1:]},
                        {k: np.asarray(ref[k], dtype=float)
                         for k in log[1:]})
    assert c['max_abs_dV_mV'] <= 0.5
