"""
FiberTissueSimulationCUDA against the oracle (the reference
FiberTissueSimulation with a CPU stand-in for its OpenCL module), following
the reference's own tests (``myokit/tests/test_simulation_fiber_tissue.py``):
argument checks, log keys, time and state handling, protocols, progress and
cancellation, NaN detection in fiber, tissue and diffusion current; and on
the GPU, double precision parity of every logged state and bound variable.
"""
import numpy as np
import pytest

from conftest import load, myokit
from myokit_gb300.fiber_tissue import FiberTissueSimulationCUDA
from oracle.ft_backend import ReferenceFiberTissueCpu

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION
CLASSES = {'oracle': ReferenceFiberTissueCpu,
           'cuda': FiberTissueSimulationCUDA}
RUN = ['oracle', pytest.param('cuda', marks=pytest.mark.gpu)]
NFX, NFY, NTX, NTY = 8, 4, 8, 6


class _Cancel(myokit.ProgressReporter):
    def __init__(self, okays=0):
        super().__init__()
        self.okays = okays

    def enter(self, msg=None):
        pass

    def exit(self):
        pass

    def update(self, progress):
        self.okays -= 1
        return self.okays >= 0


@pytest.fixture(scope='module')
def models():
    mf = load('dn-1985-normalised.mmt')
    mt = load('lr-1991.mmt')
    return mf, mt


def _p1():
    return myokit.pacing.blocktrain(1000, 2.0, offset=.01)


def _s1(cls, models, precision=SP, nx_paced=4, protocol=None):
    mf, mt = models
    return cls(mf, mt, protocol or _p1(), ncells_fiber=(NFX, NFY),
               ncells_tissue=(NTX, NTY), nx_paced=nx_paced,
               g_fiber=(235, 100), g_tissue=(9, 5), g_fiber_tissue=9,
               dt=0.0012, precision=precision)


def _s0(cls, models):
    mt = models[1]
    return cls(mt, mt, _p1(), ncells_fiber=(1, 1), ncells_tissue=(1, 1),
               nx_paced=1, g_fiber=(0, 0), g_tissue=(0, 0),
               g_fiber_tissue=0, precision=DP, dt=0.01)


@pytest.mark.parametrize('impl', ['oracle', 'cuda'])
def test_creation(impl, models):
    FT = CLASSES[impl]
    mf, mt = models
    p = _p1()
    m2 = mf.clone()
    m2.label('membrane_potential').set_rhs(None)
    with pytest.raises(myokit.MissingRhsError):
        FT(m2, mt)
    m2 = mf.clone()
    m2.get('ik').add_variable('xx').set_rhs('membrane.i_ion')
    with pytest.raises(ValueError, match='interdependent'):
        FT(m2, mt)
    s = FT(mf, mt, p, (5, 6), (7, 8))
    assert s.fiber_shape() == (6, 5) and s.tissue_shape() == (8, 7)
    for bad in (None, 12, (12,), (12, 12, 12)):
        with pytest.raises(ValueError, match=r'fiber size must be a tuple'):
            FT(mf, mt, ncells_fiber=bad)
        with pytest.raises(ValueError, match=r'tissue size must be a tuple'):
            FT(mf, mt, ncells_tissue=bad)
    for bad in ((0, 10), (10, 0), (-1, -1)):
        with pytest.raises(ValueError, match=r'fiber size must be at least'):
            FT(mf, mt, ncells_fiber=bad)
        with pytest.raises(ValueError, match=r'tissue size must be at least'):
            FT(mf, mt, ncells_tissue=bad)
    with pytest.raises(ValueError, match='exceed that of the tissue'):
        FT(mf, mt, p, (5, 6), (5, 5))
    FT(mf, mt, p, nx_paced=0)
    with pytest.raises(ValueError, match='must be non-negative'):
        FT(mf, mt, p, nx_paced=-1)
    with pytest.raises(ValueError, match=r'fiber conductivity must be a tup'):
        FT(mf, mt, p, g_fiber=1)
    with pytest.raises(ValueError, match='step size must be greater'):
        FT(mf, mt, p, dt=0)
    with pytest.raises(ValueError, match='single and double precision'):
        FT(mf, mt, p, precision=12)


@pytest.mark.parametrize('impl', RUN)
def test_basic_logs(impl, models):
    s = _s1(CLASSES[impl], models)
    logf, logt = s.run(
        .1, logf=['engine.time', 'membrane.V', 'isi.isiCa'],
        logt=['membrane.V', 'ica.Ca_i', 'ica.ICa'], log_interval=0.01)
    assert len(logf) == 1 + 2 * NFX * NFY
    assert len(logt) == 3 * NTX * NTY
    for key in ('engine.time', '0.0.membrane.V', '7.3.membrane.V',
                '0.0.isi.isiCa', '7.3.isi.isiCa'):
        assert key in logf
    for key in ('0.0.membrane.V', '7.5.membrane.V', '0.0.ica.Ca_i',
                '7.5.ica.Ca_i', '0.0.ica.ICa', '7.5.ica.ICa'):
        assert key in logt
    assert len(logf['engine.time']) == 10


@pytest.mark.parametrize('impl', RUN)
def test_pre_reset_and_states(impl, models):
    s = _s1(CLASSES[impl], models)
    assert s.time() == 0
    s.set_time(10)
    assert s.time() == 10
    s.reset()
    sf, st = s.fiber_state(), s.tissue_state()
    assert sf == s.default_fiber_state() and st == s.default_tissue_state()
    s.run(5, logf=myokit.LOG_NONE, logt=myokit.LOG_NONE)
    assert s.time() == 5
    assert s.fiber_state() != sf and s.tissue_state() != st
    assert s.default_fiber_state() == sf
    s.reset()
    assert s.fiber_state() == sf and s.tissue_state() == st
    s.pre(5)
    assert s.time() == 0
    assert s.fiber_state() != sf
    assert s.fiber_state() == s.default_fiber_state()
    assert s.tissue_state() == s.default_tissue_state()
    n = models[0].count_states()
    s.set_fiber_state([1.0] * n, 1, 2)
    assert s.fiber_state(1, 2) == [1.0] * n
    with pytest.raises(IndexError):
        s.fiber_state(NFX, 0)


@pytest.mark.parametrize('impl', RUN)
def test_protocol_and_negative_time(impl, models):
    s = _s0(CLASSES[impl], models)
    df, dt = s.run(5, logf=['membrane.V'], logt=myokit.LOG_NONE,
                   log_interval=1)
    assert df['membrane.V', 0, 0][-1] > 0
    s.reset()
    x = 0.0123
    s.set_protocol(myokit.pacing.blocktrain(level=x, duration=1000,
                                            period=1000))
    df, dt = s.run(3, logf=['engine.pace'])
    assert np.all(df.npview()['engine.pace'] == x)
    s.set_protocol(None)
    s.reset()
    df, dt = s.run(3, logf=['engine.pace'])
    assert np.all(df.npview()['engine.pace'] == 0)
    s.reset()
    s.set_protocol(myokit.pacing.blocktrain(duration=1, level=1, period=2))
    s.set_time(-10)
    df, dt = s.run(5, logf=['engine.pace'], logt=myokit.LOG_NONE)
    assert s.time() == -5
    assert np.all(df.npview()['engine.pace'] == 0)
    df, dt = s.run(6, logf=['engine.time', 'engine.pace'],
                   logt=myokit.LOG_NONE)
    df = df.npview()
    assert s.time() == 1
    assert np.all(df['engine.pace'][:-1] == 0)
    assert df['engine.pace'][-1] == 1


@pytest.mark.parametrize('impl', RUN)
def test_run_errors_and_progress(impl, models):
    s = _s1(CLASSES[impl], models)
    with pytest.raises(ValueError, match="can't be negative"):
        s.run(-1)
    s.run(1, log_interval=0)
    s.run(1, log_interval=-1)
    with pytest.raises(myokit.SimulationCancelledError):
        s.run(20, progress=_Cancel(0))
    with pytest.raises(ValueError, match='subclass of myokit.ProgressR'):
        s.run(1, progress=12)


@pytest.mark.parametrize('impl', RUN)
def test_nan_in_fiber_and_tissue(impl, models):
    cls = CLASSES[impl]
    p2 = myokit.Protocol()
    p2.schedule(period=0, duration=5, level=5e3, start=2)
    s = _s1(cls, models, nx_paced=10, protocol=p2)
    with pytest.raises(myokit.SimulationError,
                       match='numerical error in fiber simulation at t = 2.0'):
        s.run(10, log_interval=1)
    s.reset()
    df, dt = s.run(5, log_interval=0.1, report_nan=False)
    res = s.find_nan(df, dt)
    assert round(res[1], 1) == 2.0

    mf, mt = models
    mt = mt.clone()
    v = mt.get('ina.m')
    v.set_rhs('if(membrane.V < -100, 1e4, ' + v.rhs().code() + ')')
    p3 = myokit.Protocol()
    p3.schedule(period=0, duration=5, level=-1, start=1.234)
    s = cls(mf, mt, p3, ncells_fiber=(NFX, NFY), ncells_tissue=(NTX, NTY),
            nx_paced=10, g_fiber=(235, 100), g_tissue=(9, 5),
            g_fiber_tissue=9, dt=0.0012)
    with pytest.raises(myokit.SimulationError,
                       match='in tissue simulation at t = 1.7'):
        s.run(5)


@pytest.mark.parametrize('impl', RUN)
def test_nan_in_diffusion_current(impl, models):
    s = _s1(CLASSES[impl], models, nx_paced=10)
    s.set_step_size(0.01)
    with pytest.raises(myokit.SimulationError, match='when membrane.i_diff'):
        s.run(5)


@pytest.mark.gpu
@pytest.mark.parametrize('precision,tol', [(DP, 1e-9), (SP, 5e-3)])
def test_parity_with_oracle(models, precision, tol):
    # Every state and bound variable of every cell, both domains
    out = []
    for cls in (ReferenceFiberTissueCpu, FiberTissueSimulationCUDA):
        s = _s1(cls, models, precision=precision)
        out.append(s.run(12, log_interval=0.25))
    for a, b in zip(out[0], out[1]):
        assert set(a.keys()) == set(b.keys())
        worst = 0.0
        for k in a.keys():
            x, y = np.asarray(a[k]), np.asarray(b[k])
            assert x.shape == y.shape, k
            scale = max(1.0, float(np.max(np.abs(x))))
            worst = max(worst, float(np.max(np.abs(x - y))) / scale)
        assert worst <= tol, worst
    # The wave crossed the junction into the tissue
    vt = np.asarray(out[1][1]['0.2.membrane.V'])
    assert vt.max() > 0
