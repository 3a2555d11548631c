"""
The double precision exp of the generated kernels (mkg_exp64, Tang's
table-driven method; see myokit_gb300.exporter._exp64_helper), through the
product path: one forward-Euler step of dx/dt = exp(a) from x = 0 with
dt = 1 leaves x = exp(a) exactly, for a per-cell field a. Compared in ulps
with numpy's exp (the host C library's, which the oracle's kernels use)
and with CUDA's exp (the kernels built with it).
"""
import numpy as np
import pytest

from conftest import myokit
import myokit_gb300 as mg

DP = myokit.DOUBLE_PRECISION


def _model():
    m = myokit.Model('expcheck')
    c = m.add_component('c')
    t = c.add_variable('t')
    t.set_binding('time')
    t.set_rhs(0)
    a = c.add_variable('a')
    a.set_rhs(0)
    x = c.add_variable('x')
    x.promote(0.0)
    x.set_rhs('exp(a)')
    m.validate()
    return m


def _inputs():
    rng = np.random.default_rng(12)
    parts = [
        rng.uniform(-700, 700, 600000),
        rng.uniform(-1, 1, 200000) * 10.0 ** rng.uniform(-20, 0, 200000),
        rng.uniform(-0.02, 0.02, 100000),
        np.array([0.0, -0.0, 1e-300, -1e-300, 699.999, -699.999, 700.0,
                  -700.0, 705.0, -705.0, 709.7, -745.0, 1000.0, -1000.0]),
    ]
    return np.concatenate(parts)


def _kernel_exp(a, exp64):
    s = mg.SimulationCUDA(_model(), ncells=len(a), diffusion=False,
                          precision=DP)
    s._exp64 = exp64
    s.set_step_size(1.0)
    s.set_field('c.a', a)
    s.run(1.0, log=myokit.LOG_NONE)
    assert ('mkg_exp64(' in s._last_kernel.source()) == exp64
    return s.state_array()


def _ulps(x, ref):
    with np.errstate(invalid='ignore', divide='ignore'):
        d = np.abs(x - ref) / np.spacing(np.abs(ref))
    d[x == ref] = 0
    return d


def test_exp64_helper_in_double_kernels_only(br77):
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    for prec, want in ((DP, True), (myokit.SINGLE_PRECISION, False)):
        s = mg.SimulationCUDA(br77, p, ncells=40, precision=prec)
        src = s._kernel([]).source()
        assert ('mkg_exp64(' in src) == want


@pytest.mark.gpu
def test_exp64_within_one_ulp():
    a = _inputs()
    ref = np.exp(a)
    got = _kernel_exp(a, True)
    cuda = _kernel_exp(a, False)
    # The table method's range; outside it CUDA's exp is used
    fin = np.abs(a) < 700
    e_tab = _ulps(got[fin], ref[fin])
    e_cuda = _ulps(cuda[fin], ref[fin])
    assert np.max(e_tab) <= 1.0, np.max(e_tab)
    assert np.max(e_cuda) <= 2.0
    # Outside (-700, 700): identical to CUDA's exp
    assert np.array_equal(got[~fin], cuda[~fin])
