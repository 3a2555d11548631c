"""
CPU tests of the CUDA exporter: expression writing, constant folding, the
op census, and that every kernel variant compiles for sm_103a with NVRTC
(which needs no GPU).
"""
import pytest

from conftest import load, myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib
from myokit_gb300.exporter import CudaExpressionWriter

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION


def test_writer_single_and_double():
    x = myokit.Name(myokit.Model().add_component('c').add_variable('x'))
    w = CudaExpressionWriter(single=True)
    w.set_lhs_function(lambda v: 'x')
    e = myokit.Exp(myokit.Multiply(myokit.Number(0.1), x))
    assert w.ex(e) == 'expf(0.1f * x)'
    assert w.ex(myokit.Power(x, myokit.Number(3))) == 'mkg_pow3(x)'
    assert w.ex(myokit.Power(x, myokit.Number(2.5))) == 'powf(x, 2.5f)'
    assert w.ex(myokit.Log(x, myokit.Number(10))) == \
        '(logf(x) / logf(10.0f))'
    assert w.ex(myokit.Abs(x)) == 'fabsf(x)'
    w = CudaExpressionWriter(single=False)
    w.set_lhs_function(lambda v: 'x')
    assert w.ex(e) == 'exp(0.1 * x)'
    assert w.ex(myokit.Power(x, myokit.Number(2.5))) == 'pow(x, 2.5)'
    w = CudaExpressionWriter(single=True, native_math=True)
    w.set_lhs_function(lambda v: 'x')
    assert w.ex(e) == '__expf(0.1f * x)'
    # Quotient and remainder round towards minus infinity
    q = myokit.Quotient(x, myokit.Number(2))
    assert 'floorf' in w.ex(q)


def _kernel(model, ncells, precision, **kw):
    rl = kw.pop('rl', False)
    diffusion = kw.pop('diffusion', True)
    s = mg.SimulationCUDA(model, ncells=ncells, precision=precision, rl=rl,
                          diffusion=diffusion)
    for f in kw.pop('fields', []):
        import numpy as np
        s.set_field(f, np.ones(s.shape()))
    if kw.pop('hetero', False):
        import numpy as np
        if isinstance(ncells, tuple):
            s.set_conductance_field(np.ones((ncells[1], ncells[0] - 1)),
                                    np.ones((ncells[1] - 1, ncells[0])))
        else:
            s.set_conductance_field(np.ones(ncells - 1))
    if kw.pop('conn', False):
        s.set_connections([(0, 1, 1.0)])
    inter = [s._model.get(v) for v in kw.pop('inter', [])]
    return s._kernel(inter)


CASES = [
    ('beeler-1977-model.mmt', 10, SP, {}),
    ('beeler-1977-model.mmt', 10, DP, {'rl': True}),
    ('beeler-1977-model.mmt', (8, 4), SP, {'hetero': True,
                                           'inter': ['isi.Isi']}),
    ('beeler-1977-model.mmt', 6, DP, {'conn': True}),
    ('beeler-1977-model.mmt', 3, DP, {'diffusion': False,
                                      'fields': ['isi.gsBar']}),
    ('lr-1991.mmt', (5, 5), SP, {'rl': True}),
    ('dn-1985-normalised.mmt', 20, SP, {'rl': True}),
    ('decker-2009.mmt', (16, 16), SP, {'rl': True,
                                       'fields': ['ikr.Gbar', 'ina.Gbar']}),
]


@pytest.mark.parametrize('name,ncells,precision,kw', CASES)
def test_kernels_compile_for_sm103a(name, ncells, precision, kw):
    k = _kernel(load(name), ncells, precision, **dict(kw))
    src = k.source()
    assert 'mkg_tissue_step' in src
    assert ('typedef float Real;' in src) == (precision == SP)
    cubin, log = _lib.compile_source(src, k.options())
    assert len(cubin) > 1000
    assert cubin[:4] == b'\x7fELF'


def test_constants_are_folded_and_fields_are_per_cell():
    m = load('decker-2009.mmt')
    k = _kernel(m, (8, 8), SP, rl=True, fields=['ikr.Gbar'])
    src = k.source()
    # ikr.G depends on the field ikr.Gbar: computed per cell
    assert 'field[(long long)0 * pitch + cid]' in src
    g = k._name(k.model.get('ikr.G'))
    assert 'const Real ' + g + ' =' in src
    # ina.Gbar is not a field: folded to its literal
    assert k._name(k.model.get('ina.Gbar')) not in src


def test_census_counts_work():
    k = _kernel(load('decker-2009.mmt'), (8, 8), SP, rl=True)
    c = k.census.as_dict()
    assert c['arith'] > 500 and c['trans'] > 50
    assert k.bytes_per_cell_step() == 2 * 48 * 4
    k = _kernel(load('beeler-1977-model.mmt'), 10, DP)
    assert k.bytes_per_cell_step() == 2 * 8 * 8


def test_cubic_root_refinement_single_precision_only():
    # Decker 2009 computes free Ca_i, Ca_sr and Ca_cal with the
    # trigonometric solution of a cubic; single precision kernels refine
    # each with Newton steps on that cubic, double precision kernels keep
    # the reference's expressions
    from myokit_gb300.exporter import cubic_root_coefficients
    m = load('decker-2009.mmt')
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    ks = {}
    for prec in (myokit.SINGLE_PRECISION, myokit.DOUBLE_PRECISION):
        s = mg.SimulationCUDA(m, p, ncells=64, precision=prec, rl=True)
        ks[prec] = s._kernel([])
    k = ks[myokit.SINGLE_PRECISION]
    assert sorted(k.cubic) == ['v_Ca_cal', 'v_Ca_i', 'v_Ca_sr']
    assert k.cubic['v_Ca_i'] == ('v_calciumb_Ca_i_b', 'v_calciumb_Ca_i_c',
                                 'v_calciumb_Ca_i_d')
    assert 'v_Ca_i = mkg_cubic_root(' in k.source()
    assert ks[myokit.DOUBLE_PRECISION].cubic == {}
    assert 'mkg_cubic_root(' not in ks[myokit.DOUBLE_PRECISION].source()
    # Not a cubic root: other expressions with acos and sqrt
    x = myokit.Name(m.get('calciumb.Ca_i.b'))
    y = myokit.Name(m.get('calciumb.Ca_i.c'))
    z = myokit.Name(m.get('calciumb.Ca_i.d'))
    e = myokit.Plus(myokit.ACos(myokit.Divide(x, myokit.Number(10))),
                    myokit.Sqrt(myokit.Plus(myokit.Multiply(y, y),
                                            myokit.Multiply(z, z))))
    assert cubic_root_coefficients(e) is None
    assert cubic_root_coefficients(m.get('ina.INa').rhs()) is None
