"""
Every cell model in myokit's test data through both implementations.

- CPU: for every model file, ``SimulationCUDA`` accepts it exactly when the
  reference ``SimulationOpenCL`` (the oracle class) does, and otherwise
  raises the same exception with the same message
  (``myokit/_sim/openclsim.py:195-260``); every accepted model's generated
  kernel compiles with NVRTC in double precision with forward Euler and in
  single precision with Rush-Larsen.
- GPU: every accepted model on a small paced sheet, every state,
  intermediary (double precision) and bound variable of every cell logged, against the oracle in double precision
  (forward Euler and Rush-Larsen; with and without diffusion; bar 1e-9
  relative, observed at most 1.4e-13) and in single precision (bar 1e-3
  relative, observed at most 1.5e-4).

Three files have no ``membrane_potential`` label (``beeler-1977-units``,
``lr-1991-dep``, ``conditional``); they are also run with ``membrane.V``
labelled, which covers units, references to state derivatives from other
equations (``dot(m)`` of a Rush-Larsen state in ``lr-1991-dep``) and
``if``/``piecewise`` expressions.
"""
import os

import numpy as np
import pytest

from conftest import DATA, myokit
import myokit_gb300 as mg
from myokit_gb300 import _lib
from oracle.refsim import ReferenceCpuSimulation

DP = myokit.DOUBLE_PRECISION
SP = myokit.SINGLE_PRECISION
# Everything SimulationOpenCL can log: states, intermediaries, bound
LOG = myokit.LOG_STATE + myokit.LOG_INTER + myokit.LOG_BOUND

FILES = sorted(f for f in os.listdir(DATA) if f.endswith('.mmt'))
LABELLED = ['beeler-1977-units.mmt', 'lr-1991-dep.mmt', 'conditional.mmt']
ACCEPTED = [
    'beeler-1977-model-compare-a.mmt', 'beeler-1977-model-compare-b.mmt',
    'beeler-1977-model.mmt', 'cv1d.mmt', 'decker-2009.mmt',
    'dn-1985-normalised.mmt', 'lr-1991-testing.mmt', 'lr-1991.mmt',
    'noble-1962.mmt'] + ['label:' + f for f in LABELLED]


def _model(name):
    if name.startswith('label:'):
        m = myokit.load_model(os.path.join(DATA, name[6:]))
        m.get('membrane.V').set_label('membrane_potential')
        return m
    return myokit.load_model(os.path.join(DATA, name))


def _outcome(cls, m):
    try:
        cls(m, ncells=(4, 2))
    except Exception as e:
        return type(e).__name__, str(e)
    return 'ok', ''


@pytest.mark.parametrize('name', FILES)
def test_same_acceptance_as_reference(name):
    try:
        m = myokit.load_model(os.path.join(DATA, name))
    except myokit.SectionNotFoundError:
        pytest.skip('protocol or script file, no model')
    ref = _outcome(ReferenceCpuSimulation, m)
    assert _outcome(mg.SimulationCUDA, m) == ref
    assert (ref[0] == 'ok') == (name in ACCEPTED)


@pytest.mark.parametrize('name', ACCEPTED)
def test_kernels_compile(name):
    m = _model(name)
    for prec, rl in ((DP, False), (SP, True)):
        s = mg.SimulationCUDA(m, ncells=(8, 2), precision=prec, rl=rl)
        k = s._kernel([])
        cubin, _ = _lib.compile_source(k.source(), k.options())
        assert len(cubin) > 0


def _run(cls, m, prec, rl, diffusion=True, log=LOG):
    # Half the sheet paced, so that the models fire and (where they have a
    # diffusion current) the wave crosses the other half within 30 ms.
    # Without diffusion every cell is paced.
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=1, level=1)
    s = cls(m, p, ncells=(6, 3), precision=prec, rl=rl, diffusion=diffusion)
    if diffusion:
        s.set_paced_cells(3, 3)
        s.set_conductance(2, 2)
    return s.run(30, log=log, log_interval=0.25)


def _worst(a, b):
    assert set(a.keys()) == set(b.keys())
    worst = 0.0
    for k in a.keys():
        x, y = np.asarray(a[k], dtype=float), np.asarray(b[k], dtype=float)
        assert x.shape == y.shape, k
        if len(x):
            scale = max(1.0, float(np.max(np.abs(x))))
            worst = max(worst, float(np.max(np.abs(x - y))) / scale)
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize('name', ACCEPTED)
@pytest.mark.parametrize('prec,rl,diffusion,tol', [
    (DP, False, True, 1e-9), (DP, True, True, 1e-9), (SP, True, True, 1e-3),
    (DP, False, False, 1e-9)],
    ids=['fp64', 'fp64-rl', 'fp32-rl', 'fp64-no-diffusion'])
def test_model_parity(name, prec, rl, diffusion, tol):
    # Single precision: states and bound variables. Some intermediaries
    # lose most of their digits in single precision, in both implementations
    # alike: Decker 2009's ical.zz = (0.003 / Ca_cal)^4, with Ca_cal from a
    # cubic-root formula that cancels, differs by 0.47 of its maximum. They
    # are compared in double precision.
    m = _model(name)
    log = LOG if prec == DP else myokit.LOG_STATE + myokit.LOG_BOUND
    ref = _run(ReferenceCpuSimulation, m, prec, rl, diffusion, log)
    out = _run(mg.SimulationCUDA, m, prec, rl, diffusion, log)
    assert _worst(ref, out) <= tol
