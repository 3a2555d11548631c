"""
The SimulationOpenCL API contract, checked on SimulationCUDA and on the CPU
oracle (the reference class itself) side by side.

Follows the reference's own tests in
``myokit/tests/test_simulation_opencl.py`` (argument checks and messages,
conductances, connections, fields, pacing, state handling, running,
progress and cancellation, NaN diagnosis). Tests that only exercise the
Python layer run on the CPU for both classes; tests that run a simulation
need a GPU for SimulationCUDA.
"""
import numpy as np
import pytest

from conftest import load, myokit
import myokit_gb300 as mg
from oracle.refsim import ReferenceCpuSimulation
import test_oracle as to

CLASSES = {'oracle': ReferenceCpuSimulation, 'cuda': mg.SimulationCUDA}
API = ['oracle', 'cuda']
RUN = ['oracle', pytest.param('cuda', marks=pytest.mark.gpu)]


class CancellingReporter(myokit.ProgressReporter):
    """Cancels after ``okays`` updates (myokit/tests/__init__.py:101)."""
    def __init__(self, okays=0):
        super().__init__()
        self.okays = int(okays)

    def enter(self, msg=None):
        pass

    def exit(self):
        pass

    def update(self, progress):
        self.okays -= 1
        return self.okays >= 0


@pytest.fixture(scope='module')
def m():
    return load('beeler-1977-model.mmt')


@pytest.fixture(scope='module')
def p():
    return myokit.pacing.blocktrain(duration=2, offset=1, period=1000)


def sims(impl, m, p):
    cls = CLASSES[impl]
    return (cls(m, p, ncells=1), cls(m, p, ncells=10),
            cls(m, p, ncells=(4, 3)))


# ---------------------------------------------------------------------------
# Python-layer contract (no simulation runs)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize('impl', API)
def test_creation(impl, m):
    cls = CLASSES[impl]
    m2 = m.clone()
    m2.label('membrane_potential').set_rhs(None)
    with pytest.raises(myokit.MissingRhsError):
        cls(m2)
    m2 = m.clone()
    m2.get('ix1').add_variable('xx').set_rhs('membrane.i_ion')
    with pytest.raises(ValueError, match='interdependent'):
        cls(m2)
    assert cls(m, ncells=1).shape() == 1
    assert cls(m, ncells=50).shape() == 50
    assert cls(m, ncells=(2, 1)).shape() == (1, 2)
    for bad in (None, (1,), (1, 1, 1)):
        with pytest.raises(ValueError, match=r'scalar or a tuple \(nx, ny\)'):
            cls(m, ncells=bad)
    for bad in (-1, 0, (0, 10), (10, 0), (-1, -1)):
        with pytest.raises(ValueError, match='at least 1'):
            cls(m, ncells=bad)
    with pytest.raises(ValueError, match='Only single and double'):
        cls(m, precision=myokit.SINGLE_PRECISION + myokit.DOUBLE_PRECISION)
    m2 = m.clone()
    m2.label('membrane_potential').set_label(None)
    with pytest.raises(ValueError, match='requires the membrane potential'):
        cls(m2)
    m2.get('ina.INa').set_label('membrane_potential')
    with pytest.raises(ValueError, match='must be a state variable'):
        cls(m2)


@pytest.mark.parametrize('impl', API)
def test_conductance_interface(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    gx = s1.conductance()
    assert isinstance(gx, float)
    s1.set_conductance(gx + 1)
    assert s1.conductance() == gx + 1
    gx, gy = s2.conductance()
    s2.set_conductance(gx + 1)
    assert s2.conductance() == (gx + 1, gy)
    s2.set_conductance(gx + 1, gx + 2)
    assert s2.conductance() == (gx + 1, gx + 2)
    with pytest.raises(ValueError, match='Invalid conductance gx'):
        s2.set_conductance(-1, 10)
    with pytest.raises(ValueError, match='Invalid conductance gy'):
        s2.set_conductance(10, -1)
    assert s0.monodomain_conductance(5.6, 2, 3.4, 7.8, 3) == \
        3.4 * 3 * 2 / (3 * 5.6 * 7.8 * 7.8)


@pytest.mark.parametrize('impl', API)
def test_conductance_field_interface(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    s1.set_conductance_field(list(range(9)))
    assert s1.conductance() is None
    for bad in (list(range(8)), list(range(10))):
        with pytest.raises(ValueError, match='must have length'):
            s1.set_conductance_field(bad)
    x = np.arange(9)
    x[3] = -1
    with pytest.raises(ValueError, match='negative'):
        s1.set_conductance_field(x)
    with pytest.raises(ValueError, match='must be None'):
        s1.set_conductance_field(np.arange(9), np.arange(9))
    x, y = np.ones((3, 3)), np.ones((2, 4))
    s2.set_conductance_field(x, y)
    assert s2.conductance() is None
    with pytest.raises(ValueError, match=r'dimensions \(3, 3\)'):
        s2.set_conductance_field(y, y)
    with pytest.raises(ValueError, match=r'dimensions \(2, 4\)'):
        s2.set_conductance_field(x, x)
    x[2, 2] = -1
    with pytest.raises(ValueError, match='negative'):
        s2.set_conductance_field(x, y)
    x[2, 2] = 1
    with pytest.raises(ValueError, match='must be set'):
        s2.set_conductance_field(x)


@pytest.mark.parametrize('impl', API)
def test_connections_interface(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    s1.set_connections([[0, 1, 1]])
    assert s1.conductance() is None
    with pytest.raises(RuntimeError, match='in 1d mode'):
        s2.set_connections([[0, 1, 1]])
    s1.set_connections(((0, 1, 1),))
    s1.set_connections(([0, 1, 1], (0, 2, 1)))
    with pytest.raises(ValueError, match='Connection list cannot be None'):
        s1.set_connections(None)
    for bad in ([[1, 1]], [1, 1, 1], 'hello'):
        with pytest.raises(ValueError, match='list of 3-tuples'):
            s1.set_connections(bad)
    for bad in ([[-1, 0, 1]], [[0, -2, 1]], [[10, 0, 1]], [[0, 10, 1]]):
        with pytest.raises(ValueError, match='Invalid connection'):
            s1.set_connections(bad)
    for bad in ([[1, 0, 1], [1, 0, 1]], [[1, 0, 1], [1, 0, 2]],
                [[1, 0, 1], [0, 1, 1]]):
        with pytest.raises(ValueError, match='Duplicate connection'):
            s1.set_connections(bad)
    with pytest.raises(ValueError, match='Invalid conductance'):
        s1.set_connections([[1, 0, 1], [0, 2, -1]])


@pytest.mark.parametrize('impl', API)
def test_diffusion_free_interface(impl, m, p):
    s = CLASSES[impl](m, p, ncells=3, diffusion=False)
    for f, args in ((s.conductance, ()), (s.is_paced, (0,)),
                    (s.neighbors, (0,)), (s.set_conductance, ()),
                    (s.set_connections, ([],)), (s.set_paced_cells, ()),
                    (s.set_paced_cell_list, ([],)),
                    (s.set_conductance_field, ([1, 1],))):
        with pytest.raises(RuntimeError, match='method is unavailable'):
            f(*args)


@pytest.mark.parametrize('impl', API)
def test_initial_value_expressions(impl):
    m = myokit.parse_model('''
        [[model]]
        c.x = 1 + sqrt(3)
        c.y = 1 / c.p
        c.z = 3

        [c]
        t = 0 bind time
        dot(x) = 1 label membrane_potential
        dot(y) = 2
        dot(z) = 3
        p = log(3)
        q = 0 bind diffusion_current
    ''')
    s = CLASSES[impl](m, ncells=2)
    x = s.state()
    assert all(isinstance(v, float) for v in x)
    assert x[:3] == x[3:]
    assert x == m.initial_values(True) * 2
    assert x == s.default_state()


@pytest.mark.parametrize('impl', API)
def test_neighbors(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    assert s0.neighbors(0) == []
    with pytest.raises(IndexError, match='out of range'):
        s0.neighbors(1)
    with pytest.raises(ValueError, match='1-dimensional'):
        s0.neighbors(0, 1)
    assert sorted(s1.neighbors(0)) == [1]
    assert sorted(s1.neighbors(1)) == [0, 2]
    assert sorted(s1.neighbors(9)) == [8]
    with pytest.raises(IndexError, match='out of range'):
        s1.neighbors(10)
    s1.set_connections([(0, 1, 1), (0, 2, 1), (3, 0, 1), (3, 2, 1)])
    assert sorted(s1.neighbors(0)) == [1, 2, 3]
    assert sorted(s1.neighbors(2)) == [0, 3]
    assert s1.neighbors(4) == []
    assert sorted(s2.neighbors(0, 0)) == [(0, 1), (1, 0)]
    assert sorted(s2.neighbors(1, 1)) == [(0, 1), (1, 0), (1, 2), (2, 1)]
    assert sorted(s2.neighbors(3, 1)) == [(2, 1), (3, 0), (3, 2)]
    with pytest.raises(IndexError, match='out of range'):
        s2.neighbors(0, 3)
    with pytest.raises(ValueError, match='2-dimensional'):
        s2.neighbors(0)


@pytest.mark.parametrize('impl', API)
def test_paced_cells(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    s1.set_paced_cells(3)
    assert [s1.is_paced(i) for i in range(5)] == [1, 1, 1, 0, 0]
    s1.set_paced_cells(nx=2, x=2)
    assert [s1.is_paced(i) for i in range(5)] == [0, 0, 1, 1, 0]
    s1.set_paced_cells(nx=-2)
    assert [s1.is_paced(i) for i in (0, 8, 9)] == [0, 1, 1]
    s1.set_paced_cells(nx=-2, x=4)
    assert [s1.is_paced(i) for i in range(5)] == [0, 0, 1, 1, 0]
    s1.set_paced_cells(nx=-2, x=-2)
    assert [s1.is_paced(i) for i in range(5, 10)] == [0, 1, 1, 0, 0]
    s1.set_paced_cell_list([0, 0, 3])
    assert [s1.is_paced(i) for i in range(5)] == [1, 0, 0, 1, 0]
    with pytest.raises(IndexError, match='out of range'):
        s1.set_paced_cell_list([10])
    with pytest.raises(ValueError, match='1-dimensional'):
        s1.is_paced(3, 3)
    s2.set_paced_cells(x=1, y=1, nx=1, ny=2)
    assert s2.is_paced(1, 1) and s2.is_paced(1, 2)
    assert not s2.is_paced(0, 0) and not s2.is_paced(2, 1)
    s2.set_paced_cells(x=1, y=2, nx=-1, ny=-2)
    assert s2.is_paced(0, 0) and s2.is_paced(0, 1)
    assert not s2.is_paced(0, 2)
    s2.set_paced_cell_list([(0, 0), (0, 2), (1, 1)])
    assert s2.is_paced(0, 2) and not s2.is_paced(0, 1)
    for bad in ([(-1, 0)], [(4, 0)], [(0, 4)], [(5, 5)]):
        with pytest.raises(IndexError, match='out of range'):
            s2.set_paced_cell_list(bad)
    with pytest.raises(ValueError, match='2-dimensional'):
        s2.is_paced(1)


@pytest.mark.parametrize('impl', API)
def test_set_state(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    n, k = 10, 8
    sm = m.initial_values(True)
    assert all(s1.state(i) == sm for i in range(n))
    sx = list(range(n * k))
    s1.set_state(sx)
    assert s1.state() == sx
    z = [0.0] * k
    s1.set_state(z)
    assert s1.state() == z * n
    s1.set_state(sm)
    s1.set_state(z, 3)
    assert s1.state(3) == z and s1.state(2) == sm
    with pytest.raises(ValueError, match='x was not None'):
        s1.set_state([0] * k * n, 3)
    with pytest.raises(ValueError, match='y was not None'):
        s1.set_state([0] * k * n, y=2)
    with pytest.raises(ValueError, match='must have the same size as'):
        s1.set_state([0] * (k * n + 1))
    with pytest.raises(IndexError, match='x-index out of range'):
        s1.set_state(sm, n)
    with pytest.raises(ValueError, match='1-dimensional'):
        s1.set_state(sm, 0, 1)
    with pytest.raises(IndexError, match='x-index out of range'):
        s1.state(-1)
    s1.set_default_state(list(range(k)), 3)
    assert s1.default_state(3) == list(range(k))
    # 2d: x first, then y
    s2.set_state(z)
    s2.set_state(sm, x=1, y=2)
    flat = s2.state()[::k]
    assert flat[9] == sm[0] and flat.count(0) == 11
    with pytest.raises(IndexError, match='y-index out of range'):
        s2.set_state(sm, 0, 3)
    with pytest.raises(IndexError, match='y-index out of range'):
        s2.default_state(1, 3)


@pytest.mark.parametrize('impl', API)
def test_set_constant_and_field(impl, m, p):
    cls = CLASSES[impl]
    m2 = m.clone()
    v = m2['membrane'].add_variable('calculated_constant')
    v.set_rhs('3 * C')
    s = cls(m2)
    s.set_constant('membrane.C', 3)
    s.set_constant(m2.get('membrane.C'), 2)
    for name in ('membrane.V', 'ina.INa', 'engine.time'):
        with pytest.raises(ValueError, match='not a literal'):
            s.set_constant(name, 1)
    s0, s1, s2 = sims(impl, m, p)
    x = list(range(10))
    s1.set_field('membrane.C', x)
    s1.set_field('membrane.C', x)
    s1.remove_field('membrane.C')
    with pytest.raises(KeyError):
        s1.remove_field('membrane.C')
    with pytest.raises(ValueError, match='constant'):
        s1.set_field('membrane.V', x)
    with pytest.raises(ValueError, match='Bound'):
        s1.set_field('engine.time', x)
    with pytest.raises(ValueError, match='length'):
        s1.set_field('membrane.C', list(range(9)))
    s2.set_field('membrane.C', np.zeros(s2.shape()))
    with pytest.raises(ValueError, match='dimensions'):
        s2.set_field('membrane.C', np.zeros((4, 4)))


@pytest.mark.parametrize('impl', API)
def test_shape_and_step_size(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    assert s1.shape() == 10 and s2.shape() == (3, 4)
    assert s2.is_2d() and not s1.is_2d()
    dt = s0.step_size() * 2 + 0.001
    s0.set_step_size(dt)
    assert s0.step_size() == dt
    for bad in (0, -1):
        with pytest.raises(ValueError, match='greater than zero'):
            s0.set_step_size(bad)


# ---------------------------------------------------------------------------
# Behaviour while running (SimulationCUDA on the GPU)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize('impl', RUN)
def test_conductance_effects(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    s1.set_paced_cells(5)
    s1.set_conductance()
    d = s1.run(10, log=['membrane.V']).npview()
    assert np.max(d['membrane.V', 9]) > 0
    s1.reset()
    s1.set_conductance(0)
    d = s1.run(10, log=['membrane.V']).npview()
    assert np.max(d['membrane.V', 9]) < 0
    s2.set_paced_cells(2, 2)
    for gx, gy, expect in ((10, 10, (1, 1, 1)), (10, 0, (1, 0, 0)),
                           (0, 10, (0, 1, 0))):
        s2.reset()
        s2.set_conductance(gx, gy)
        d = s2.run(5, log=['membrane.V']).npview()
        got = tuple(int(np.max(d['membrane.V', x, y]) > -80)
                    for x, y in ((3, 0), (0, 2), (3, 2)))
        assert got == expect, (gx, gy)


@pytest.mark.parametrize('impl', RUN)
def test_conductance_field_effects(impl, m, p):
    s0, s1, s2 = sims(impl, m, p)
    s1.set_paced_cells(x=3, nx=3)
    x = np.ones(9)
    x[0] = 0
    x[-2:] = 0
    s1.set_conductance_field(x)
    d = s1.run(15, log=['engine.time', 'membrane.V'],
               log_interval=0.1).npview()
    depol = [np.max(d['membrane.V', i]) > 0 for i in range(10)]
    assert depol == [0, 1, 1, 1, 1, 1, 1, 1, 0, 0]
    x = np.ones((3, 3))
    y = np.ones((2, 4))
    x[1, 1:3] = 0
    y[0:2, 2] = 0
    s2.set_paced_cells(2, 2)
    s2.set_conductance_field(x, y)
    d = s2.run(15, log=['engine.time', 'membrane.V'],
               log_interval=0.1).npview()
    for i in range(4):
        for j in range(3):
            up = np.max(d['membrane.V', i, j]) > 0
            assert up == (not (i == 2 and j == 1)), (i, j)


@pytest.mark.parametrize('impl', RUN)
def test_diffusion_free_run(impl, m, p):
    s = CLASSES[impl](m, p, ncells=3, diffusion=False)
    d = s.run(10, log=['membrane.V']).npview()
    assert np.all(d['membrane.V', 0] == d['membrane.V', 1])
    assert np.max(d['membrane.V', 2]) > 0
    s.reset()
    s.set_field('isi.gsBar', [0.05, 0.09, 0.14])
    d = s.run(10, log=['membrane.V']).npview()
    assert not np.all(d['membrane.V', 0] == d['membrane.V', 1])
    m2 = m.clone()
    m2.label('membrane_potential').set_label(None)
    s = CLASSES[impl](m2, p, ncells=3, diffusion=False)
    d = s.run(10, log=['membrane.V']).npview()
    assert np.all(d['membrane.V', 0] == d['membrane.V', 2])


@pytest.mark.parametrize('impl', RUN)
def test_negative_time(impl, m, p):
    s0 = CLASSES[impl](m, p, ncells=1)
    s0.set_protocol(myokit.pacing.blocktrain(duration=1, level=1, period=2))
    s0.set_time(-10)
    d = s0.run(5, log=['engine.pace']).npview()
    assert s0.time() == -5
    assert np.all(d['engine.pace'] == 0)
    d = s0.run(6, log=['engine.time', 'engine.pace']).npview()
    assert s0.time() == 1
    assert np.all(d['engine.pace'][:-1] == 0)
    assert d['engine.pace'][-1] == 1


@pytest.mark.parametrize('impl', RUN)
def test_protocol_changes(impl, m, p):
    s0 = CLASSES[impl](m, p, ncells=1)
    assert np.max(s0.run(3, log=['engine.pace']).npview()['engine.pace']) \
        == 1
    x = 0.0123
    s0.set_protocol(myokit.pacing.blocktrain(level=x, duration=1000,
                                             period=1000))
    s0.reset()
    d = s0.run(3, log=['engine.pace']).npview()
    assert np.all(d['engine.pace'] == np.float32(x))
    s0.reset()
    s0.set_protocol(None)
    assert np.all(s0.run(3, log=['engine.pace']).npview()['engine.pace']
                  == 0)
    s0.reset()
    s0.set_protocol(myokit.pacing.blocktrain(period=1000, duration=2,
                                             offset=3))
    assert np.max(s0.run(3, log=['engine.pace']).npview()['engine.pace']) \
        == 0
    assert np.max(s0.run(3, log=['engine.pace']).npview()['engine.pace']) \
        == 1


@pytest.mark.parametrize('impl', RUN)
def test_run_pre_reset(impl, m, p):
    s0 = CLASSES[impl](m, p, ncells=1)
    x0 = s0.default_state()
    assert x0 == s0.state() and s0.time() == 0
    s0.run(1)
    x1 = s0.state()
    assert x0 == s0.default_state() and x0 != x1 and s0.time() == 1
    s0.reset()
    assert x0 == s0.state() and s0.time() == 0
    s0.pre(1)
    assert x1 == s0.default_state() and x1 == s0.state()
    assert s0.time() == 0
    s0.run(1)
    assert x1 != s0.state() and s0.time() == 1
    s0.set_time(10)
    s0.run(1)
    assert s0.time() == 11
    with pytest.raises(ValueError, match='negative'):
        s0.run(-1)


@pytest.mark.parametrize('impl', RUN)
def test_progress_and_cancel(impl, m, p):
    s0 = CLASSES[impl](m, p, ncells=1)
    with myokit.tools.capture() as c:
        s0.run(3, progress=myokit.ProgressPrinter())
    assert c.text() != ''
    with pytest.raises(ValueError, match='progress'):
        s0.run(1, progress=True)
    before = s0.state()
    with pytest.raises(myokit.SimulationCancelledError):
        s0.run(20, progress=CancellingReporter(0))
    assert s0.state() == before


@pytest.mark.parametrize('impl', RUN)
def test_connections_equal_conductance(impl, m):
    pr = myokit.pacing.blocktrain(1000, 10, level=1)
    s1 = CLASSES[impl](m, pr, ncells=10)
    s1.set_paced_cells(3)
    log = ['engine.time', 'membrane.V', 'membrane.i_diff']
    s1.set_conductance(5, 0)
    a = s1.run(10, log=log, log_interval=0.1).npview()
    s1.reset()
    s1.set_connections([(i, i + 1, 5) for i in range(9)])
    b = s1.run(10, log=log, log_interval=0.1).npview()
    for c in (0, 9):
        assert np.max(np.abs(a['membrane.V', c] - b['membrane.V', c])) < 1e-4
    s = CLASSES[impl](m, pr, ncells=2, precision=myokit.DOUBLE_PRECISION)
    s.set_paced_cells(1)
    s.set_conductance(1)
    a = s.run(5, log=log, log_interval=0.1).npview()
    s.reset()
    s.set_connections([(0, 1, 1)])
    b = s.run(5, log=log, log_interval=0.1).npview()
    for c in (0, 1):
        assert np.max(np.abs(a['membrane.V', c] - b['membrane.V', c])) < 1e-9


@pytest.mark.parametrize('impl', RUN)
def test_find_nan_manual(impl):
    to.check_find_nan(CLASSES[impl])


@pytest.mark.parametrize('impl', RUN)
def test_find_nan_one_over_zero(impl):
    to.check_one_over_zero(CLASSES[impl])


@pytest.mark.parametrize('impl', RUN)
def test_find_nan_first_point(impl):
    s = to.nan_sim(CLASSES[impl])
    x = s.state(0, 0)
    x[3] = float('nan')
    s.set_state(x, 2, 2)
    with pytest.raises(myokit.SimulationError, match='met in the very first'):
        s.run(2)


@pytest.mark.parametrize('impl', RUN)
def test_find_nan_without_error(impl):
    s = to.nan_sim(CLASSES[impl])
    s.set_protocol(None)
    d = s.run(10)
    with pytest.raises(myokit.FindNanError, match='not found in log'):
        s.find_nan(d)


@pytest.mark.parametrize('impl', RUN)
def test_find_nan_big_steps(impl):
    s = CLASSES[impl](myokit.load_model('example'),
                      myokit.pacing.blocktrain(period=1000, duration=2),
                      ncells=10)
    s.set_step_size(1)
    with pytest.raises(myokit.SimulationError):
        s.run(10)
    for log in (['membrane.V'], myokit.LOG_STATE, myokit.LOG_BOUND):
        with pytest.raises(myokit.SimulationError, match='Unable to pinpoint'):
            s.run(10, log=log)
