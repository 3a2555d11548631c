"""
Discrete adjoint of the fused tissue step.

For a loss on logged membrane potentials,
``L = sum over probes p and log points j of (V_p(t_j) - target_pj)^2``,
the gradients with respect to per-cell scalar fields (for example GKr and
GNa scale fields) and to the diffusion conductances gx, gy are computed by
reverse-mode differentiation of the discrete forward map (forward Euler or
Rush-Larsen, plus the diffusion stencil), not of the ODEs: they are the
exact gradients of what the forward kernel computes, up to rounding.

- :func:`local_partial` differentiates one equation's right-hand side with
  respect to one referenced variable, all other references held fixed (the
  reference's ``Expression.diff``, ``myokit/_expressions.py:243``, expands
  intermediate variables instead; here every equation is differentiated
  locally and the chain rule runs through the generated reverse sweep).
- :class:`AdjointKernel` emits, from the forward :class:`TissueKernel`'s
  equation list, a CUDA kernel that re-evaluates the model at step k from a
  recorded trajectory and sweeps the equations in reverse.
- :class:`TissueAdjoint` runs forward with checkpoints every K steps, then
  per segment (last first) recomputes the trajectory and runs the adjoint
  kernel; :class:`TissueLossFunction` wraps this as a
  ``torch.autograd.Function``.
"""
import math

import numpy as np

from ._deps import myokit
from . import exporter as _exp
from . import _lib

_N = myokit.Number


def _mul(a, b):
    if a is None or b is None:
        return None
    return myokit.Multiply(a, b)


def _add(a, b):
    if a is None:
        return b
    if b is None:
        return a
    return myokit.Plus(a, b)


def _sub(a, b):
    if b is None:
        return a
    if a is None:
        return myokit.PrefixMinus(b)
    return myokit.Minus(a, b)


def local_partial(e, ref):
    """
    Partial derivative of expression ``e`` with respect to the
    :class:`myokit.Name` (or ``Derivative``) ``ref``, treating every other
    reference as a constant. Returns an expression or ``None`` for zero.
    Conditionals differentiate their branches (right derivatives at the
    switching points), as ``Expression.diff`` does.
    """
    d = lambda x: local_partial(x, ref)  # noqa: E731
    if isinstance(e, (myokit.Name, myokit.Derivative)):
        return _N(1) if e == ref else None
    if isinstance(e, myokit.Number):
        return None
    if isinstance(e, myokit.PrefixPlus):
        return d(e[0])
    if isinstance(e, myokit.PrefixMinus):
        x = d(e[0])
        return None if x is None else myokit.PrefixMinus(x)
    if isinstance(e, myokit.Plus):
        return _add(d(e[0]), d(e[1]))
    if isinstance(e, myokit.Minus):
        return _sub(d(e[0]), d(e[1]))
    if isinstance(e, myokit.Multiply):
        return _add(_mul(d(e[0]), e[1]), _mul(e[0], d(e[1])))
    if isinstance(e, myokit.Divide):
        a, b = e[0], e[1]
        da, db = d(a), d(b)
        out = None if da is None else myokit.Divide(da, b)
        if db is not None:
            out = _sub(out, myokit.Divide(myokit.Multiply(a, db),
                                          myokit.Power(b, _N(2))))
        return out
    if isinstance(e, myokit.Power):
        a, b = e[0], e[1]
        da, db = d(a), d(b)
        out = None
        if da is not None:
            if isinstance(b, myokit.Number):
                p = b.eval()
                out = myokit.Multiply(
                    myokit.Multiply(_N(p), myokit.Power(a, _N(p - 1))), da)
            else:
                out = myokit.Multiply(
                    myokit.Multiply(b, myokit.Power(a, myokit.Minus(b, _N(1)))),
                    da)
        if db is not None:
            out = _add(out, myokit.Multiply(
                myokit.Multiply(e, myokit.Log(a)), db))
        return out
    if isinstance(e, myokit.Exp):
        x = d(e[0])
        return None if x is None else myokit.Multiply(e, x)
    if isinstance(e, myokit.Log):
        if len(e) == 1:
            x = d(e[0])
            return None if x is None else myokit.Divide(x, e[0])
        # log_b(a) = ln a / ln b
        return d(myokit.Divide(myokit.Log(e[0]), myokit.Log(e[1])))
    if isinstance(e, myokit.Log10):
        x = d(e[0])
        return None if x is None else myokit.Divide(
            x, myokit.Multiply(e[0], _N(math.log(10))))
    if isinstance(e, myokit.Sqrt):
        x = d(e[0])
        return None if x is None else myokit.Divide(
            x, myokit.Multiply(_N(2), e))
    if isinstance(e, myokit.Sin):
        x = d(e[0])
        return None if x is None else myokit.Multiply(myokit.Cos(e[0]), x)
    if isinstance(e, myokit.Cos):
        x = d(e[0])
        return None if x is None else myokit.PrefixMinus(
            myokit.Multiply(myokit.Sin(e[0]), x))
    if isinstance(e, myokit.Tan):
        x = d(e[0])
        return None if x is None else myokit.Divide(
            x, myokit.Power(myokit.Cos(e[0]), _N(2)))
    if isinstance(e, myokit.ASin):
        x = d(e[0])
        return None if x is None else myokit.Divide(x, myokit.Sqrt(
            myokit.Minus(_N(1), myokit.Power(e[0], _N(2)))))
    if isinstance(e, myokit.ACos):
        x = d(e[0])
        return None if x is None else myokit.PrefixMinus(myokit.Divide(
            x, myokit.Sqrt(myokit.Minus(_N(1), myokit.Power(e[0], _N(2))))))
    if isinstance(e, myokit.ATan):
        x = d(e[0])
        return None if x is None else myokit.Divide(x, myokit.Plus(
            _N(1), myokit.Power(e[0], _N(2))))
    if isinstance(e, (myokit.Floor, myokit.Ceil, myokit.Quotient)):
        return None
    if isinstance(e, myokit.Remainder):
        return _sub(d(e[0]), _mul(d(e[1]), myokit.Floor(
            myokit.Divide(e[0], e[1]))))
    if isinstance(e, myokit.Abs):
        x = d(e[0])
        return None if x is None else myokit.If(
            myokit.MoreEqual(e[0], _N(0)), x, myokit.PrefixMinus(x))
    if isinstance(e, myokit.If):
        t, f = d(e._t), d(e._e)
        if t is None and f is None:
            return None
        return myokit.If(e._i, t or _N(0), f or _N(0))
    if isinstance(e, myokit.Piecewise):
        parts = [d(x) for x in e._e]
        if all(p is None for p in parts):
            return None
        args = []
        for c, p in zip(e._i, parts[:-1]):
            args.extend([c, p or _N(0)])
        args.append(parts[-1] or _N(0))
        return myokit.Piecewise(*args)
    if isinstance(e, (myokit.Condition,)):
        return None
    raise NotImplementedError(
        'No local derivative for ' + type(e).__name__)


def _references(e):
    """Names and derivatives referenced in e (unique, stable order)."""
    seen = []
    for x in e.walk():
        if isinstance(x, (myokit.Name, myokit.Derivative)) and x not in seen:
            seen.append(x)
    return seen


class AdjointKernel(object):
    """
    CUDA source for the adjoint of a forward :class:`TissueKernel`: the
    trajectory-writing forward kernel and the reverse kernel, in one module.
    Supports forward-Euler and Rush-Larsen updates, every diffusion mode
    (homogeneous or per-edge conductances on a 1D or 2D grid, arbitrary
    connections, none) and scalar fields.
    """
    def __init__(self, fwd, min_blocks=1, threads=None, guards=True):
        self.fwd = fwd
        self.single = fwd.single
        self.min_blocks = int(min_blocks)
        self.threads = int(threads or fwd.block[0])
        if self.threads % 32 or not 32 <= self.threads <= 1024:
            raise ValueError('threads must be a multiple of 32 up to 1024')
        self.guards = bool(guards)
        self._source = self._generate()

    def _generate(self):
        fwd = self.fwd
        w = fwd.writer
        name = fwd._name
        tab = '            '
        states = fwd.states
        # Forward values at step k, from the trajectory
        fw = []
        for i, s in enumerate(states):
            fw.append(f'{tab}const Real {name(s)} = xk[(long long){i}'
                      f' * pitch + cid];')
        for k, var in enumerate(fwd.fields):
            fw.append(f'{tab}const Real {name(var)} = '
                      f'field[(long long){k} * pitch + cid];')
        for lhs, rhs in fwd.cell_const_eqs:
            fw.append(f'{tab}const Real {name(lhs)} = {w.ex(rhs)};')
        for lhs, rhs in fwd.rhs_eqs:
            fw.append(f'{tab}const Real {name(lhs)} = '
                      f'{fwd.rhs_code(lhs, rhs)};')

        # Adjoint accumulators: every state, field, per-cell constant,
        # equation left-hand side and the diffusion current
        acc = []

        def A(n):
            return 'A' + n

        accs = [name(s) for s in states] + [name(v) for v in fwd.fields]
        accs += [name(lhs) for lhs, _ in fwd.cell_const_eqs]
        accs += [name(lhs) for lhs, _ in fwd.rhs_eqs]
        accs.append(_exp._IDIFF)
        seen = set()
        for n in accs:
            if n not in seen:
                acc.append(f'{tab}Real {A(n)} = 0;')
                seen.add(n)

        def ref(var):
            x = fwd.literal_subst.get(myokit.Name(var))
            return w.ex(x) if x is not None else name(var)

        # Seeds: lambda_{k+1} through the update of each state
        seeds = list(acc)
        expf = w._fn('exp')
        for i, s in enumerate(states):
            lam = f'lam[(long long){i} * pitch + cid]'
            if i == fwd.i_vm:
                lam = f'({lam} + gather)'
            n = name(s)
            seeds.append(f'{tab}{{ const Real l_ = {lam};')
            if s in fwd.rl_states:
                inf, tau = fwd.rl_states[s]
                ri, rt = ref(inf), ref(tau)
                seeds.append(f'{tab}  const Real E_ = {expf}(-dt_ / {rt});')
                seeds.append(f'{tab}  {A(n)} += l_ * E_;')
                if myokit.Name(inf) not in fwd.literal_subst:
                    seeds.append(f'{tab}  {A(name(inf))} += l_ * (1 - E_);')
                if myokit.Name(tau) not in fwd.literal_subst:
                    seeds.append(
                        f'{tab}  {A(name(tau))} += -l_ * ({ri} - {n}) * E_'
                        f' * dt_ / ({rt} * {rt});')
            else:
                seeds.append(f'{tab}  {A(n)} += l_;')
                seeds.append(f'{tab}  {A(name(s.lhs()))} += l_ * dt_;')
            seeds.append(f'{tab}}}')

        # Reverse sweep: equations in reverse evaluation order
        rev = []
        valid = set(seen)
        for lhs, rhs in reversed(fwd.rhs_eqs + []):
            a = A(name(lhs))
            terms = []
            bcd = fwd.cubic.get(name(lhs))
            if bcd is not None:
                # A refined root x of x^3 + b x^2 + c x + d: by the implicit
                # function theorem dx/db = -x^2/g, dx/dc = -x/g, dx/dd = -1/g
                # with g = 3x^2 + 2bx + c
                x = name(lhs)
                b, c, d = bcd
                terms.append(f'{tab}    const Real g_ = (3 * {x} + 2 * {b})'
                             f' * {x} + {c};')
                terms.append(f'{tab}    const Real r_ = (g_ != 0) ? a_ / g_'
                             ' : (Real)0;')
                for rn, dx in ((b, f'{x} * {x}'), (c, x), (d, '1')):
                    if rn in valid:
                        terms.append(f'{tab}    {A(rn)} -= r_ * ({dx});')
                rhs = myokit.Number(0)   # no further terms
            for r in _references(rhs):
                rn = name(r)
                if rn in (_exp._T, _exp._PACE):
                    continue
                if rn not in valid:
                    continue
                dp = local_partial(rhs, r)
                if dp is None:
                    continue
                terms.append(f'{tab}    {A(rn)} += a_ * ({w.ex(dp)});')
            if terms:
                # With guards an equation whose adjoint is still zero is
                # skipped; without, the sweep is straight-line code
                if self.guards:
                    rev.append(f'{tab}if ({a} != 0) {{ const Real a_ = {a};')
                else:
                    rev.append(f'{tab}{{ const Real a_ = {a};')
                rev.extend(terms)
                rev.append(f'{tab}}}')
        for lhs, rhs in reversed(fwd.cell_const_eqs):
            a = A(name(lhs))
            for r in _references(rhs):
                rn = name(r)
                if rn not in valid:
                    continue
                dp = local_partial(rhs, r)
                if dp is None:
                    continue
                rev.append(f'{tab}{A(rn)} += {a} * ({w.ex(dp)});')

        # Outputs
        out = []
        for i, s in enumerate(states):
            n = name(s)
            extra = ''
            if i == fwd.i_vm and fwd.diffusion != _exp.DIFF_NONE:
                extra = f' + {A(_exp._IDIFF)} * cdiag'
            out.append(f'{tab}lam[(long long){i} * pitch + cid] = '
                       f'{A(n)}{extra};')
        for k, var in enumerate(fwd.fields):
            out.append(f'{tab}gfield[(long long){k} * pitch + cid] += '
                       f'{A(name(var))};')
        if fwd.diffusion != _exp.DIFF_NONE:
            out.append(f'{tab}mu_out[cid] = {A(_exp._IDIFF)};')
            out.append(f'{tab}gg[cid] += {A(_exp._IDIFF)} * xterm;')
            out.append(f'{tab}gg[pitch + cid] += {A(_exp._IDIFF)} * yterm;')

        loss_target = A(name(states[fwd.i_vm])) if fwd.i_vm >= 0 else \
            A(name(fwd.vm))
        subs = {
            '@ADJ_MINB@': str(self.min_blocks),
            '@ADJ_BX@': str(self.threads),
            '@FORWARD@': '\n'.join(fw),
            '@SEEDS@': '\n'.join(seeds),
            '@LOSS_TARGET@': loss_target,
            '@REVERSE@': '\n'.join(rev),
            '@OUTPUTS@': '\n'.join(out),
            '@IDIFF_ADJ@': A(_exp._IDIFF),
        }
        text = _exp._read('tissue_adjoint.cu.in')
        for k, v in subs.items():
            text = text.replace(k, v)
        # The forward kernel with trajectory output, in the same module
        return self._join(fwd.source(), text)

    @staticmethod
    def _join(fsrc, text):
        """Appends the adjoint kernel (the template from its declaration
        on) to the forward module, which defines what it uses."""
        start = text.index('extern "C" __global__')
        return fsrc + '\n' + text[start:]

    def source(self):
        return self._source

    def options(self):
        return self.fwd.options()

    def key(self):
        import hashlib
        h = hashlib.sha256()
        h.update(self._source.encode())
        h.update('\0'.join(self.options()).encode())
        return h.hexdigest()


class TissueAdjoint(object):
    """
    Forward runs and loss gradients for a :class:`SimulationCUDA`.

    ``sim``
        A simulation in any diffusion mode: homogeneous conductances gx, gy,
        per-edge conductances (``set_conductance_field``), connections
        (``set_connections``) or none. Its fields and its conductances are
        the parameters the gradients refer to. With an accumulation mode the
        forward
        runs (and is recomputed) exactly as the simulation's own, FP64 or
        compensated states included; the reverse sweep is in the
        simulation precision and takes the rounding of those states to it
        as the identity.
    ``probes``
        Cells whose V enters the loss: integers (1D) or ``(x, y)`` (2D).
    ``segment_steps``
        Steps between checkpoints: the backward pass recomputes each segment
        from its checkpoint, so memory is one segment's trajectory plus one
        state per segment.
    ``min_blocks``, ``threads``
        Resident CTAs per SM asked of the compiler for the reverse kernel,
        and its CTA size (default: the simulation's); the register cap is
        64K / (threads * min_blocks).
    ``guards``
        Skip the reverse of equations whose adjoint is still zero (one
        branch per equation). The default, straight-line code, lets the
        compiler schedule across equations and keeps the reverse kernel
        free of register spills; results are the same while the partial
        derivatives are finite.

    The simulation's state and time are not changed by :meth:`forward`.
    """
    def __init__(self, sim, probes, segment_steps=200, min_blocks=1,
                 threads=None, guards=False):
        self.sim = sim
        self.segment_steps = int(segment_steps)
        self.min_blocks = int(min_blocks)
        self.threads = threads
        self.guards = bool(guards)
        self._generated = {}
        vm = sim._vm
        if vm is None:
            raise ValueError('The adjoint needs a membrane potential.')
        self.cells = []
        for p in probes:
            if len(sim._dims) == 2:
                x, y = int(p[0]), int(p[1])
                if not (0 <= x < sim._nx and 0 <= y < sim._ny):
                    raise IndexError('Probe out of range: ' + str(p))
                self.cells.append(x + y * sim._nx)
            else:
                x = int(p)
                if not 0 <= x < sim._nx:
                    raise IndexError('Probe out of range: ' + str(p))
                self.cells.append(x)
        if len(set(self.cells)) != len(self.cells):
            raise ValueError('Duplicate probe cells.')
        self._attached = None
        self.rows = 0

    def field_names(self):
        """Qualified names of the fields, in gradient order."""
        return [v.qname() for v in self.sim._fields]

    def _prepare(self):
        from .simulation import compile_kernel
        sim = self.sim
        kernel = sim._kernel([])
        be = sim._get_backend(kernel)
        # Generated once per forward kernel (the forward kernel's key covers
        # the model version, precision, fields and launch shape)
        akey = (kernel.key(), self.min_blocks, self.threads, self.guards)
        ak = self._generated.get(akey)
        if ak is None:
            # The trajectory-writing forward kernel has the launch shape,
            # register cap and tile staging of the simulation's own kernel
            fwd = _exp.TissueKernel(
                sim._model, sim._precision, sim._native_math,
                sim._bound_variables, [], kernel.diffusion, kernel.two_d,
                list(sim._fields.keys()), sim._rl_states, kernel.block,
                min_blocks=kernel.min_blocks, math=sim._fp32_math,
                accumulate=kernel.accumulate,
                accumulate_states=sim.accumulated_states(), traj=True,
                stage=kernel.stage, row_pad=kernel.row_pad,
                stage_lazy=kernel.stage_lazy, sync=kernel.sync)
            ak = AdjointKernel(fwd, self.min_blocks, self.threads,
                               self.guards)
            self._generated = {akey: ak}
        key = (id(be), akey, self.segment_steps)
        if self._attached != key:
            cubin = compile_kernel(ak)
            be.check(be.lib.mkg_adj_attach(be.h, cubin, len(cubin),
                                           self.segment_steps))
            self._attached = key
        return be

    def forward(self, duration, log_interval=1.0):
        """
        Runs ``duration`` time units from the simulation's state and time,
        and returns the probes' V as an array (log points x probes).
        """
        sim = self.sim
        be = self._prepare()
        lib, h = be.lib, be.h
        saved = (sim._state.copy(), sim._time)
        sim._upload(be)
        items = np.full(len(self.cells), sim._vm.index(), dtype=np.int32)
        cells = np.ascontiguousarray(self.cells, dtype=np.int64)
        be.log_sig = None
        be.check(lib.mkg_set_log(h, _lib.i32ptr(items), _lib.i64ptr(cells),
                                 len(cells), 0))
        be.check(lib.mkg_set_tuning(h, 0, 0, 0))
        rows = _lib.ctypes.c_int64()
        be.check(lib.mkg_adj_forward(
            h, sim._time, sim._time + duration, sim._step_size,
            float(log_interval), _lib.ctypes.byref(rows)))
        self.rows = rows.value
        out = np.empty((self.rows, len(self.cells)))
        be.check(lib.mkg_adj_read_log(h, _lib.dptr(out), self.rows))
        sim._state, sim._time = saved
        return out

    def backward(self, dl_dv):
        """
        Gradients for ``dl_dv = dL/dV`` at the logged points (the array
        returned by :meth:`forward`). Returns ``{field qname: gradient with
        the field's shape, 'gx': ..., 'gy': ...}`` where, by diffusion mode,

        - homogeneous conductances: ``gx`` and ``gy`` are floats;
        - per-edge conductances: ``gx`` has the shape of the simulation's
          gx field, ``(ny, nx - 1)`` in 2D or ``(nx - 1,)`` in 1D, and
          ``gy`` the shape ``(ny - 1, nx)`` (an empty array in 1D);
        - connections: ``'connections'`` holds one gradient per connection,
          in the order of the simulation's connection list, and ``gx`` is
          their sum (``gy`` is 0).
        """
        sim = self.sim
        be = self._prepare()
        g = np.ascontiguousarray(dl_dv, dtype=np.float64)
        if g.shape != (self.rows, len(self.cells)):
            raise ValueError('dl_dv must have shape %s' % (
                (self.rows, len(self.cells)),))
        nf = len(sim._fields)
        gf = np.zeros(max(nf, 1) * sim._ntotal)
        gg = np.zeros(2)
        be.check(be.lib.mkg_adj_backward(
            be.h, _lib.dptr(g), self.rows, _lib.dptr(gf), _lib.dptr(gg)))
        out = {}
        shape = (sim._ny, sim._nx) if len(sim._dims) == 2 else (sim._nx,)
        gf = gf[:nf * sim._ntotal].reshape(sim._ntotal, max(nf, 1))
        for k, name in enumerate(self.field_names()):
            out[name] = gf[:, k].reshape(shape)
        out['gx'] = float(gg[0])
        out['gy'] = float(gg[1])
        mode = sim._diffusion_mode()
        if mode in (_exp.DIFF_HETERO, _exp.DIFF_CONN):
            nx, ny = sim._nx, sim._ny
            two_d = len(sim._dims) == 2
            if mode == _exp.DIFF_HETERO:
                n = ny * (nx - 1) + ((ny - 1) * nx if two_d else 0)
            else:
                n = len(sim._connections)
            ge = np.zeros(max(n, 1))
            be.check(be.lib.mkg_adj_conductance_gradient(
                be.h, _lib.dptr(ge), n))
            if mode == _exp.DIFF_CONN:
                out['connections'] = ge[:n]
            elif two_d:
                out['gx'] = ge[:ny * (nx - 1)].reshape(ny, nx - 1)
                out['gy'] = ge[ny * (nx - 1):n].reshape(ny - 1, nx)
            else:
                out['gx'] = ge[:n]
                out['gy'] = np.zeros(0)
        return out

    def loss_and_gradient(self, duration, target, log_interval=1.0):
        """Sum of squared V errors against ``target`` and its gradients."""
        v = self.forward(duration, log_interval)
        d = v - np.asarray(target, dtype=float)
        return float(np.sum(d * d)), self.backward(2 * d)


def _make_function():
    import torch

    class TissueLossFunction(torch.autograd.Function):
        """
        ``loss = TissueLossFunction.apply(adjoint, duration, log_interval,
        target, g, *fields)``: the sum of squared V errors at the probes of
        a :class:`TissueAdjoint`, as a function of the scalar fields (tensors
        shaped like the grid, in ``adjoint.field_names()`` order) and of the
        diffusion conductances ``g``:

        - homogeneous conductances: a scalar tensor (gx = gy = g in 2D) or a
          two-element tensor (gx, gy);
        - per-edge conductances: one tensor of the gx field's values
          followed, in 2D, by the gy field's (the layout of
          ``set_conductance_field``, flattened);
        - connections: one tensor of per-connection conductances, in the
          order of the simulation's connection list.

        Gradients come from the discrete adjoint.
        """
        @staticmethod
        def forward(ctx, adj, duration, log_interval, target, g, *fields):
            sim = adj.sim
            for name, f in zip(adj.field_names(), fields):
                sim.set_field(name, f.detach().cpu().double().numpy())
            gv = g.detach().cpu().double().reshape(-1).numpy()
            mode = sim._diffusion_mode()
            ctx.mode = mode
            if mode == _exp.DIFF_HETERO:
                nx, ny = sim._nx, sim._ny
                n = ny * (nx - 1)
                if len(sim._dims) == 2:
                    sim.set_conductance_field(
                        gv[:n].reshape(ny, nx - 1), gv[n:].reshape(ny - 1, nx))
                else:
                    sim.set_conductance_field(gv[:n])
            elif mode == _exp.DIFF_CONN:
                sim.set_connections([(i, j, float(x)) for (i, j, _), x in
                                     zip(sim._connections, gv)])
            elif sim._diffusion_enabled:
                gx = float(gv[0])
                gy = float(gv[1]) if len(gv) > 1 else gx
                sim.set_conductance(gx, gy)
            v = adj.forward(duration, log_interval)
            tgt = target.detach().cpu().double().numpy() \
                if hasattr(target, 'detach') else np.asarray(target)
            d = v - tgt
            ctx.adj = adj
            ctx.lgrad = 2 * d
            ctx.g_len = len(gv)
            ctx.g_dtype = g.dtype
            ctx.f_meta = [(f.dtype, f.device) for f in fields]
            return torch.tensor(float(np.sum(d * d)), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            adj = ctx.adj
            grads = adj.backward(ctx.lgrad)
            s = float(grad_out)
            if ctx.mode == _exp.DIFF_HETERO:
                gg = torch.as_tensor(np.concatenate(
                    [np.ravel(grads['gx']), np.ravel(grads['gy'])]) * s,
                    dtype=ctx.g_dtype)
            elif ctx.mode == _exp.DIFF_CONN:
                gg = torch.as_tensor(grads['connections'] * s,
                                     dtype=ctx.g_dtype)
            elif ctx.g_len > 1:
                gg = torch.tensor([grads['gx'] * s, grads['gy'] * s],
                                  dtype=ctx.g_dtype)
            else:
                gg = torch.tensor((grads['gx'] + grads['gy']) * s,
                                  dtype=ctx.g_dtype)
            out = [None, None, None, None, gg]
            for name, (dt, dev) in zip(adj.field_names(), ctx.f_meta):
                out.append(torch.as_tensor(grads[name] * s, dtype=dt,
                                           device=dev))
            return tuple(out)

    return TissueLossFunction


_FUNCTION = None


def tissue_loss(adj, duration, target, g, fields, log_interval=1.0):
    """
    Differentiable loss (see ``TissueLossFunction``): returns a 0-d torch
    tensor whose ``backward()`` fills ``g.grad`` and the fields' ``.grad``.
    """
    global _FUNCTION
    if _FUNCTION is None:
        _FUNCTION = _make_function()
    return _FUNCTION.apply(adj, duration, log_interval, target, g, *fields)
