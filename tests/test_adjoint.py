"""
The discrete adjoint: local symbolic partials (CPU), kernel generation for
sm_103a (CPU, NVRTC), and on the GPU the gradients of a loss on probe V
against central finite differences (relative step 1e-4, double precision),
checkpoint-length independence and the torch.autograd.Function.
"""
import numpy as np
import pytest

from conftest import load, myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib, adjoint, exporter

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION


def _numeric_partial(e, ref, values):
    h = 1e-6 * max(abs(values[ref]), 1e-9)

    def ev(delta):
        sub = {k: myokit.Number(v + (delta if k == ref else 0))
               for k, v in values.items()}
        return e.eval(subst=sub)
    return (ev(h) - ev(-h)) / (2 * h)


@pytest.mark.parametrize('name', ['beeler-1977-model.mmt', 'lr-1991.mmt'])
def test_local_partials_match_numerical(name):
    m = load(name)
    rng = np.random.default_rng(0)
    checked = 0
    for v in m.variables(deep=True):
        if v.is_state() or v.is_constant() or v.is_bound():
            continue
        e = v.rhs()
        refs = [r for r in adjoint._references(e)]
        if not refs:
            continue
        values = {}
        for r in refs:
            rv = r.var()
            if rv.is_state():
                values[r] = rv.initial_value(True) * (1 + 0.1 * rng.normal())
            else:
                values[r] = rv.eval() if rv.is_constant() else rng.uniform(
                    0.5, 2)
        for r in refs:
            dp = adjoint.local_partial(e, r)
            sub = {k: myokit.Number(x) for k, x in values.items()}
            a = 0.0 if dp is None else dp.eval(subst=sub)
            b = _numeric_partial(e, r, values)
            assert abs(a - b) <= 1e-5 * max(1e-8, abs(b)), (v.qname(), r)
            checked += 1
    assert checked > 20


def _sim(model, precision, shape=(6, 5), rl=False, fields=None, cls=None):
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1)
    cls = cls or mg.SimulationCUDA
    s = cls(model, p, ncells=shape, precision=precision, rl=rl)
    s.set_paced_cells(2, shape[1] if isinstance(shape, tuple) else 1)
    s.set_conductance(9, 6)
    for name, values in (fields or {}).items():
        s.set_field(name, values)
    return s


@pytest.mark.parametrize('name,field', [
    ('beeler-1977-model.mmt', 'isi.gsBar'),
    ('decker-2009.mmt', 'ikr.Gbar'),
])
@pytest.mark.parametrize('precision', [SP, DP])
def test_adjoint_kernels_compile(name, field, precision):
    m = load(name)
    base = m.get(field).eval()
    s = _sim(m, precision, rl=True, fields={field: np.full((5, 6), base)})
    k = s._kernel([])
    fwd = exporter.TissueKernel(
        s._model, s._precision, False, s._bound_variables, [], k.diffusion,
        k.two_d, list(s._fields.keys()), s._rl_states, k.block, traj=True)
    ak = adjoint.AdjointKernel(fwd)
    cubin, _ = _lib.compile_source(ak.source(), ak.options())
    assert cubin[:4] == b'\x7fELF'
    assert 'mkg_tissue_adjoint' in ak.source()


def _fields(m, shape, seed):
    rng = np.random.default_rng(seed)
    return {
        'isi.gsBar': m.get('isi.gsBar').eval() * rng.lognormal(0, 0.2, shape),
        'ina.gNaBar': m.get('ina.gNaBar').eval() * rng.lognormal(0, 0.2,
                                                                  shape),
    }


PROBES = [(0, 0), (3, 2), (5, 4), (1, 4)]


def _loss(s, adj, target, dur=12):
    v = adj.forward(dur, 0.5)
    return float(np.sum((v - target) ** 2))


@pytest.mark.gpu
@pytest.mark.parametrize('rl', [False, True])
def test_adjoint_matches_finite_differences(br77, rl):
    shape = (5, 6)
    f0 = _fields(br77, shape, 1)
    ft = _fields(br77, shape, 2)
    s = _sim(br77, DP, rl=rl, fields=ft)
    adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=150)
    target = adj.forward(12, 0.5)
    for k, v in f0.items():
        s.set_field(k, v)
    s.set_conductance(8, 5)
    L, grads = adj.loss_and_gradient(12, target, 0.5)
    assert L > 0
    rng = np.random.default_rng(3)
    checks = []
    for name in f0:
        for _ in range(3):
            iy, ix = rng.integers(0, shape[0]), rng.integers(0, shape[1])
            checks.append((name, (iy, ix)))
    checks += [('gx', None), ('gy', None)]
    for name, idx in checks:
        if name in ('gx', 'gy'):
            g0 = 8.0 if name == 'gx' else 5.0
            h = 1e-4 * g0
            vals = []
            for sgn in (1, -1):
                gx = g0 + sgn * h if name == 'gx' else 8.0
                gy = g0 + sgn * h if name == 'gy' else 5.0
                s.set_conductance(gx, gy)
                vals.append(_loss(s, adj, target))
            s.set_conductance(8, 5)
            fd = (vals[0] - vals[1]) / (2 * h)
            ad = grads[name]
        else:
            base = f0[name].copy()
            h = 1e-4 * base[idx]
            vals = []
            for sgn in (1, -1):
                f = base.copy()
                f[idx] += sgn * h
                s.set_field(name, f)
                vals.append(_loss(s, adj, target))
            s.set_field(name, base)
            fd = (vals[0] - vals[1]) / (2 * h)
            ad = grads[name][idx]
        scale = max(abs(fd), 1e-6 * abs(L))
        assert abs(ad - fd) <= 1e-4 * scale, (name, idx, ad, fd)


@pytest.mark.gpu
def test_adjoint_checkpoint_length_independent(br77):
    shape = (5, 6)
    s = _sim(br77, DP, fields=_fields(br77, shape, 1))
    target = np.zeros((24, len(PROBES))) - 80
    out = []
    for k in (7, 64, 1000):
        adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=k)
        L, g = adj.loss_and_gradient(12, target, 0.5)
        out.append((L, g))
    for L, g in out[1:]:
        assert L == out[0][0]
        for k in g:
            assert np.array_equal(np.asarray(g[k]), np.asarray(out[0][1][k]))


@pytest.mark.gpu
def test_torch_function_gradients(br77):
    import torch
    shape = (5, 6)
    f0 = _fields(br77, shape, 1)
    s = _sim(br77, DP, fields=f0)
    adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=100)
    target = torch.full((24, len(PROBES)), -80.0, dtype=torch.float64)
    g = torch.tensor(7.0, dtype=torch.float64, requires_grad=True)
    fields = [torch.tensor(f0[n], requires_grad=True)
              for n in adj.field_names()]
    loss = adjoint.tissue_loss(adj, 12, target, g, fields, 0.5)
    loss.backward()
    s.set_conductance(7, 7)
    L, ref = adj.loss_and_gradient(12, target.numpy(), 0.5)
    assert abs(loss.item() - L) <= 1e-12 * abs(L)
    assert abs(float(g.grad) - (ref['gx'] + ref['gy'])) <= 1e-12 * abs(
        ref['gx'] + ref['gy'])
    for t, n in zip(fields, adj.field_names()):
        np.testing.assert_allclose(t.grad.numpy(), ref[n], rtol=1e-12)


@pytest.mark.gpu
def test_guarded_and_straight_line_sweeps_agree(br77):
    shape = (5, 6)
    s = _sim(br77, DP, fields=_fields(br77, shape, 1))
    target = np.zeros((24, len(PROBES))) - 80
    out = []
    for guards in (True, False):
        adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=50,
                                    guards=guards)
        out.append(adj.loss_and_gradient(12, target, 0.5))
    assert out[0][0] == out[1][0]
    for k in out[0][1]:
        np.testing.assert_allclose(np.asarray(out[0][1][k]),
                                   np.asarray(out[1][1][k]), rtol=1e-12,
                                   atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize('acc', ['double', 'kahan'])
def test_adjoint_with_accumulation_modes(br77, acc):
    # FP32 forward with FP64 (or compensated) V and concentrations: the
    # adjoint's forward equals the simulation's own run, and its gradients
    # agree with the double precision adjoint to the FP32 forward's accuracy
    shape = (5, 6)
    f0 = _fields(br77, shape, 1)
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1)
    res = {}
    for key, kw in (('fp64', {'precision': DP}),
                    (acc, {'precision': SP, 'accumulate': acc})):
        s = mg.SimulationCUDA(br77, p, ncells=(6, 5), **kw)
        s.set_paced_cells(2, 5)
        s.set_conductance(9, 6)
        for k, v in f0.items():
            s.set_field(k, v)
        adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=70)
        target = np.zeros((24, len(PROBES))) - 80
        L, g = adj.loss_and_gradient(12, target, 0.5)
        res[key] = (L, g)
        if key == acc:
            keys = ['engine.time'] + ['%d.%d.membrane.V' % q for q in PROBES]
            va = adj.forward(12, 0.5)
            d = s.run(12, log=keys, log_interval=0.5)
            v = np.stack([np.asarray(d[k]) for k in keys[1:]], axis=1)
            assert np.array_equal(v, va)
    L64, g64 = res['fp64']
    L32, g32 = res[acc]
    assert abs(L32 - L64) <= 1e-3 * L64
    for k in g64:
        a, b = np.asarray(g32[k]), np.asarray(g64[k])
        err = np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)
        assert err <= 2e-2, (k, err)


@pytest.mark.gpu
def test_adjoint_matches_oracle_finite_differences(br77):
    # Gradients of the loss as the reference computes it: central finite
    # differences of the oracle's (reference SimulationOpenCL) loss
    from oracle.refsim import ReferenceCpuSimulation
    shape = (5, 6)
    f0 = _fields(br77, shape, 1)
    target = np.zeros((24, len(PROBES))) - 80
    s = _sim(br77, DP, fields=f0)
    adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=100)
    L, grads = adj.loss_and_gradient(12, target, 0.5)
    keys = ['%d.%d.membrane.V' % q for q in PROBES]

    def oracle_loss(fields, gx=9.0):
        o = _sim(br77, DP, fields=fields, cls=ReferenceCpuSimulation)
        o.set_conductance(gx, 6)
        d = o.run(12, log=['engine.time'] + keys, log_interval=0.5)
        v = np.stack([np.asarray(d[k]) for k in keys], axis=1)
        return float(np.sum((v - target) ** 2))

    assert abs(oracle_loss(f0) - L) <= 1e-9 * L
    for name, idx in (('isi.gsBar', (0, 0)), ('isi.gsBar', (2, 3)),
                      ('ina.gNaBar', (4, 5)), ('ina.gNaBar', (1, 1))):
        h = 1e-4 * f0[name][idx]
        vals = []
        for sgn in (1, -1):
            f = {k: v.copy() for k, v in f0.items()}
            f[name][idx] += sgn * h
            vals.append(oracle_loss(f))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(grads[name][idx] - fd) <= 1e-4 * max(abs(fd), 1e-6 * L)
    h = 1e-4 * 9.0
    fd = (oracle_loss(f0, 9.0 + h) - oracle_loss(f0, 9.0 - h)) / (2 * h)
    assert abs(grads['gx'] - fd) <= 1e-4 * abs(fd)


def _dep_model():
    # Other equations refer to dot(m) of a Rush-Larsen state (ina.x) and to
    # dot(V) (test.t1); the file has no membrane_potential label
    m = load('lr-1991-dep.mmt')
    m.get('membrane.V').set_label('membrane_potential')
    return m


def test_adjoint_kernel_with_derivative_references_compiles():
    m = _dep_model()
    s = _sim(m, DP, rl=True, fields={'ina.gNa': np.full((5, 6), 16.0)})
    k = s._kernel([])
    # m and h update by Rush-Larsen; other equations see dot(m) = dot(h) = 0,
    # as in the reference's kernel
    assert 'const Real d_m = 0' in k.source()
    assert 'const Real d_h = 0' in k.source()
    fwd = exporter.TissueKernel(
        s._model, s._precision, False, s._bound_variables, [], k.diffusion,
        k.two_d, list(s._fields.keys()), s._rl_states, k.block, traj=True)
    ak = adjoint.AdjointKernel(fwd, guards=False)
    cubin, _ = _lib.compile_source(ak.source(), ak.options())
    assert cubin[:4] == b'\x7fELF'


@pytest.mark.gpu
def test_adjoint_with_derivative_references():
    m = _dep_model()
    shape = (5, 6)
    rng = np.random.default_rng(4)
    f0 = 16.0 * rng.lognormal(0, 0.2, shape)
    ft = 16.0 * rng.lognormal(0, 0.2, shape)
    s = _sim(m, DP, rl=True, fields={'ina.gNa': ft})
    adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=150)
    target = adj.forward(12, 0.5)
    s.set_field('ina.gNa', f0)
    L, grads = adj.loss_and_gradient(12, target, 0.5)
    assert L > 0
    # Probe cells (0, 0) and (1, 4) are paced; (3, 2) is a probe at rest;
    # (2, 2) is no probe (the model has no diffusion current)
    for idx in ((0, 0), (4, 1), (2, 3), (2, 2)):
        h = 1e-4 * f0[idx]
        vals = []
        for sgn in (1, -1):
            f = f0.copy()
            f[idx] += sgn * h
            s.set_field('ina.gNa', f)
            vals.append(_loss(s, adj, target))
        s.set_field('ina.gNa', f0)
        fd = (vals[0] - vals[1]) / (2 * h)
        ad = grads['ina.gNa'][idx]
        assert abs(ad - fd) <= 1e-4 * max(abs(fd), 1e-6 * L), (idx, ad, fd)


# ---------------------------------------------------------------------------
# Per-edge conductances and connections (diff_hetero, openclsim.cl:452-487;
# diff_arb_step, openclsim.cl:537-556): gradients with respect to every
# edge's conductance, against central differences of the oracle's loss
# ---------------------------------------------------------------------------

def _edge_case(kind):
    """(ncells, setter(sim), parameters {name: (array, index list)})."""
    rng = np.random.default_rng(21)
    if kind == 'hetero2d':
        gx = 9.0 * rng.lognormal(0, 0.2, (5, 5))
        gy = 6.0 * rng.lognormal(0, 0.2, (4, 6))

        def setter(s, gx=gx, gy=gy):
            s.set_conductance_field(gx, gy)
        return (6, 5), setter, {'gx': gx, 'gy': gy}
    if kind == 'hetero1d':
        gx = 9.0 * rng.lognormal(0, 0.2, 39)

        def setter(s, gx=gx):
            s.set_conductance_field(gx)
        return 40, setter, {'gx': gx}
    # A chain with a few long-range links
    n = 30
    conns = [(i, i + 1, 9.0 * rng.lognormal(0, 0.2)) for i in range(n - 1)]
    conns += [(0, 12, 2.5), (5, 25, 1.5), (17, 29, 3.0)]
    g = np.array([c[2] for c in conns])

    def setter(s, g=g):
        s.set_connections([(i, j, float(x)) for (i, j, _), x in
                           zip(conns, g)])
    return n, setter, {'connections': g}


def _edge_sim(model, cls, shape, setter, fields):
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1)
    s = cls(model, p, ncells=shape, precision=DP)
    if isinstance(shape, tuple):
        s.set_paced_cells(2, shape[1])
    else:
        s.set_paced_cells(3)
    setter(s)
    for name, values in fields.items():
        s.set_field(name, values)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize('kind', ['hetero2d', 'hetero1d', 'connections'])
def test_adjoint_edges_match_oracle_finite_differences(br77, kind):
    from oracle.refsim import ReferenceCpuSimulation
    shape, setter, params = _edge_case(kind)
    fshape = (shape[1], shape[0]) if isinstance(shape, tuple) else (shape,)
    f0 = _fields(br77, fshape, 1)
    probes = PROBES if isinstance(shape, tuple) else [0, 7, 20, 29]
    keys = ['%d.%d.membrane.V' % q if isinstance(q, tuple) else
            '%d.membrane.V' % q for q in probes]
    target = np.zeros((24, len(probes))) - 80
    s = _edge_sim(br77, mg.SimulationCUDA, shape, setter, f0)
    adj = adjoint.TissueAdjoint(s, probes, segment_steps=70)
    L, grads = adj.loss_and_gradient(12, target, 0.5)

    def oracle_loss(p):
        def set_(o):
            if kind == 'hetero2d':
                o.set_conductance_field(p['gx'], p['gy'])
            elif kind == 'hetero1d':
                o.set_conductance_field(p['gx'])
            else:
                setter(o, p['connections'])
        o = _edge_sim(br77, ReferenceCpuSimulation, shape, set_, f0)
        d = o.run(12, log=['engine.time'] + keys, log_interval=0.5)
        v = np.stack([np.asarray(d[k]) for k in keys], axis=1)
        return float(np.sum((v - target) ** 2))

    assert abs(oracle_loss(params) - L) <= 1e-9 * L
    rng = np.random.default_rng(8)
    checked = 0
    for name, arr in params.items():
        got = grads[name]
        assert np.shape(got) == arr.shape
        for _ in range(4):
            idx = tuple(int(rng.integers(0, k)) for k in arr.shape)
            h = 1e-4 * arr[idx]
            vals = []
            for sgn in (1, -1):
                p = {k: v.copy() for k, v in params.items()}
                p[name][idx] += sgn * h
                vals.append(oracle_loss(p))
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(got[idx] - fd) <= 1e-4 * max(abs(fd), 1e-6 * L), (
                name, idx, got[idx], fd)
            checked += 1
    assert checked >= 4
    # Field gradients are unchanged by the diffusion mode's bookkeeping
    name = 'isi.gsBar'
    idx = (0,) * len(fshape)
    h = 1e-4 * f0[name][idx]
    vals = []
    for sgn in (1, -1):
        f = f0[name].copy()
        f[idx] += sgn * h
        s.set_field(name, f)
        v = adj.forward(12, 0.5)
        vals.append(float(np.sum((v - target) ** 2)))
    s.set_field(name, f0[name])
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(grads[name][idx] - fd) <= 1e-4 * max(abs(fd), 1e-6 * L)


@pytest.mark.gpu
def test_adjoint_uniform_edges_sum_to_homogeneous(br77):
    # A grid with every x edge 9 and every y edge 6, given as per-edge
    # conductances: the edge gradients sum to the homogeneous gradients
    # dL/dgx, dL/dgy, and fields get the same gradients
    f0 = _fields(br77, (5, 6), 1)
    target = np.zeros((24, len(PROBES))) - 80
    out = []
    for hetero in (False, True):
        s = _sim(br77, DP, fields=f0)
        if hetero:
            s.set_conductance_field(np.full((5, 5), 9.0),
                                    np.full((4, 6), 6.0))
        adj = adjoint.TissueAdjoint(s, PROBES, segment_steps=100)
        out.append(adj.loss_and_gradient(12, target, 0.5))
    (L0, g0), (L1, g1) = out
    assert abs(L1 - L0) <= 1e-12 * L0
    assert abs(np.sum(g1['gx']) - g0['gx']) <= 1e-9 * abs(g0['gx'])
    assert abs(np.sum(g1['gy']) - g0['gy']) <= 1e-9 * abs(g0['gy'])
    for k in f0:
        np.testing.assert_allclose(g1[k], g0[k], rtol=1e-9, atol=1e-12 * L0)


@pytest.mark.gpu
@pytest.mark.parametrize('kind', ['hetero2d', 'connections'])
def test_torch_function_edge_gradients(br77, kind):
    import torch
    shape, setter, params = _edge_case(kind)
    fshape = (shape[1], shape[0]) if isinstance(shape, tuple) else (shape,)
    f0 = _fields(br77, fshape, 1)
    probes = PROBES if isinstance(shape, tuple) else [0, 7, 20, 29]
    s = _edge_sim(br77, mg.SimulationCUDA, shape, setter, f0)
    adj = adjoint.TissueAdjoint(s, probes, segment_steps=100)
    target = torch.full((24, len(probes)), -80.0, dtype=torch.float64)
    flat = np.concatenate([np.ravel(v) for v in params.values()])
    g = torch.tensor(flat, requires_grad=True)
    fields = [torch.tensor(f0[n], requires_grad=True)
              for n in adj.field_names()]
    loss = adjoint.tissue_loss(adj, 12, target, g, fields, 0.5)
    loss.backward()
    L, ref = adj.loss_and_gradient(12, target.numpy(), 0.5)
    assert abs(loss.item() - L) <= 1e-12 * abs(L)
    want = np.concatenate([np.ravel(ref[k]) for k in params])
    np.testing.assert_allclose(g.grad.numpy(), want, rtol=1e-12)
    for t, n in zip(fields, adj.field_names()):
        np.testing.assert_allclose(t.grad.numpy(), ref[n], rtol=1e-12)


@pytest.mark.parametrize('kind', ['hetero2d', 'hetero1d', 'connections'])
@pytest.mark.parametrize('precision', [SP, DP])
def test_adjoint_edge_kernels_compile(br77, kind, precision):
    shape, setter, params = _edge_case(kind)
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1)
    s = mg.SimulationCUDA(br77, p, ncells=shape, precision=precision)
    setter(s)
    k = s._kernel([])
    assert k.diffusion == {'hetero2d': 2, 'hetero1d': 2,
                           'connections': 3}[kind]
    fwd = exporter.TissueKernel(
        s._model, s._precision, False, s._bound_variables, [], k.diffusion,
        k.two_d, [], s._rl_states, k.block, traj=True)
    ak = adjoint.AdjointKernel(fwd)
    cubin, _ = _lib.compile_source(ak.source(), ak.options())
    assert cubin[:4] == b'\x7fELF'
