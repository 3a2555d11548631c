"""
CUDA exporter: turns a myokit model into one fused tissue-step kernel.

The reference renders ``myokit/_sim/openclsim.cl`` once per run into an
OpenCL program with a ``cell_step`` kernel (model right-hand side plus the
forward-Euler or Rush-Larsen update, ``openclsim.cl:298-367``) and separate
diffusion kernels (``diff_step`` ``:384``, ``diff_hetero`` ``:452``,
``diff_arb_step`` ``:537``). This exporter emits a single CUDA kernel,
``mkg_tissue_step``, that for every cell and step

1. computes the diffusion current from V(t) of the neighbours (warp tiles
   staged in shared memory by TMA tensor copies, or loaded directly;
   neighbour lists for arbitrary connections),
2. evaluates the model right-hand side in registers,
3. writes the logged values of that step to the device log, and
4. updates every state to t + dt, writing V(t + dt) to the second plane of a
   ping-pong buffer so that neighbours still read V(t).

Several steps run in one launch, separated by a bounded grid barrier or by
bounded waits on the warps owning the neighbouring tiles. State is stored
structure-of-arrays, so every load and store is coalesced.

Differences from the reference kernel text that do not change results:

- constants that do not depend on a scalar field are evaluated once on the
  host (in the simulation precision, with ``Expression.eval``) and written as
  literals, where the reference writes them as macros (``openclsim.cl:174-186``);
- subexpressions of literals only are evaluated on the host as well;
- small integer powers ``x^2`` .. ``x^16`` are written as products.
"""
import hashlib
import os

import numpy as np

from ._deps import myokit
from myokit.formats.ansic import CBasedExpressionWriter

_HERE = os.path.dirname(os.path.abspath(__file__))
_CSRC = os.path.join(_HERE, 'csrc')

# Diffusion modes (match include/mkg_tissue.h)
DIFF_NONE = 0
DIFF_GRID = 1
DIFF_HETERO = 2
DIFF_CONN = 3

# Bound-variable internal names used in the generated code
_T = 't_'
_PACE = 'pace_'
_IDIFF = 'idiff_'


def _fmt_number(x, single):
    """Formats a float as a C literal of the simulation precision."""
    x = float(x)
    if np.isnan(x):
        return '(0.0f/0.0f)' if single else '(0.0/0.0)'
    if np.isinf(x):
        s = '(1.0f/0.0f)' if single else '(1.0/0.0)'
        return s if x > 0 else '(-' + s + ')'
    # Shortest text that rounds back to the same value in the precision
    s = str(np.float32(x)) if single else repr(x)
    if 'e' not in s and '.' not in s:
        s += '.0'
    return s + 'f' if single else s


class CudaExpressionWriter(CBasedExpressionWriter):
    """
    Writes myokit expressions as CUDA C++ for one precision.

    Functions are written with explicit single or double precision names
    (``expf``/``exp``); with ``native_math`` the single precision versions
    use the fast hardware approximations (``__expf`` etc.), the CUDA
    counterpart of OpenCL's ``native_*`` functions
    (``myokit/formats/opencl/_ewriter.py:59-93``).
    """
    def __init__(self, single, native_math=False, fast_divide=False):
        super().__init__()
        self._single = bool(single)
        self._native = bool(native_math) and self._single
        self._fast_div = bool(fast_divide) and self._single
        self.int_powers = set()

    def _ex_divide(self, e):
        if not self._fast_div:
            return super()._ex_divide(e)
        # Single precision fast division: a constant denominator becomes a
        # multiplication by its rounded reciprocal (within 1.5 ulp of the
        # quotient), any other one uses the 2-ulp hardware reciprocal.
        num = self.ex(e[0])
        if isinstance(e[1], myokit.Number):
            d = float(e[1].eval())
            if d != 0 and np.isfinite(d):
                r = _fmt_number(float(np.float32(1.0) / np.float32(d)), True)
                return f'(({num}) * {r})'
        return f'__fdividef({num}, {self.ex(e[1])})'

    def _fn(self, name):
        if not self._single:
            return name
        if self._native and name in ('exp', 'log', 'sin', 'cos', 'tan',
                                     'log10'):
            return '__' + name + 'f'
        return name + 'f'

    def _ex_number(self, e):
        return _fmt_number(e.eval(), self._single)

    def _ex_power(self, e):
        base, exponent = e[0], e[1]
        if isinstance(exponent, myokit.Number):
            p = float(exponent.eval())
            # Small integer powers by repeated squaring (the exporter emits
            # mkg_pow<n> helpers), half-integer powers through sqrt.
            if p == int(p) and 2 <= p <= 16:
                self.int_powers.add(int(p))
                return f'mkg_pow{int(p)}({self.ex(base)})'
            if p == 0.5:
                return self._ex_function(myokit.Sqrt(base), self._fn('sqrt'))
            if p == 1.5:
                b = self.ex(base)
                return f'mkg_pow1p5({b})'
        return f'{self._fn("pow")}({self.ex(base)}, {self.ex(exponent)})'

    def _ex_sqrt(self, e):
        return self._ex_function(e, self._fn('sqrt'))

    def _ex_sin(self, e):
        return self._ex_function(e, self._fn('sin'))

    def _ex_cos(self, e):
        return self._ex_function(e, self._fn('cos'))

    def _ex_tan(self, e):
        return self._ex_function(e, self._fn('tan'))

    def _ex_asin(self, e):
        return self._ex_function(e, self._fn('asin'))

    def _ex_acos(self, e):
        return self._ex_function(e, self._fn('acos'))

    def _ex_atan(self, e):
        return self._ex_function(e, self._fn('atan'))

    def _ex_exp(self, e):
        return self._ex_function(e, self._fn('exp'))

    def _ex_log(self, e):
        f = self._fn('log')
        if len(e) == 1:
            return self._ex_function(e, f)
        return f'({f}({self.ex(e[0])}) / {f}({self.ex(e[1])}))'

    def _ex_log10(self, e):
        return self._ex_function(e, self._fn('log10'))

    def _ex_floor(self, e):
        return self._ex_function(e, self._fn('floor'))

    def _ex_ceil(self, e):
        return self._ex_function(e, self._fn('ceil'))

    def _ex_abs(self, e):
        return self._ex_function(e, self._fn('fabs'))


class OpCensus(object):
    """
    Counts the work in one cell-step of a generated kernel: arithmetic
    operations (``+ - * /``, an FMA counted as two), transcendental calls and
    conditionals. Used for the compute roofline.
    """
    _TRANS = (
        myokit.Exp, myokit.Log, myokit.Log10, myokit.Sqrt, myokit.Sin,
        myokit.Cos, myokit.Tan, myokit.ASin, myokit.ACos, myokit.ATan)

    def __init__(self):
        self.arith = 0
        self.divide = 0
        self.trans = 0
        self.power = 0
        self.cond = 0

    def cost(self):
        """Estimated instructions: an arithmetic operation 1, a division
        8, a transcendental function 20, a general power 25."""
        return (self.arith + 7 * self.divide + 20 * self.trans +
                25 * self.power)

    def add(self, e):
        for x in e.walk():
            if isinstance(x, (myokit.Plus, myokit.Minus, myokit.Multiply,
                              myokit.PrefixMinus)):
                self.arith += 1
            elif isinstance(x, (myokit.Divide, myokit.Quotient,
                                myokit.Remainder)):
                self.arith += 1
                self.divide += 1
            elif isinstance(x, myokit.Power):
                p = x[1].eval() if isinstance(x[1], myokit.Number) else None
                if p is not None and p == int(p) and 2 <= p <= 16:
                    self.arith += int(p).bit_length() + bin(int(p)).count(
                        '1') - 2
                elif p in (0.5, 1.5):
                    self.trans += 1
                    self.arith += 1 if p == 1.5 else 0
                else:
                    self.power += 1
            elif isinstance(x, self._TRANS):
                self.trans += 1
            elif isinstance(x, (myokit.If, myokit.Piecewise)):
                self.cond += 1

    def as_dict(self):
        return {
            'arith': self.arith, 'divide': self.divide, 'trans': self.trans,
            'power': self.power, 'cond': self.cond,
        }


# Writes the logged items of one class for this cell at a log row.
_LOG_BLOCK = '''
        if (row >= 0) {{
            Real *lg = (Real *)a.log + (long long)row * a.log_ncol;
            for (int j = 0; j < a.n_log_items; ++j) {{
                const int item = a.log_items[j];
                if (!({cond})) continue;
                const int c = a.log_cols[(long long)j * pitch + cid];
                if (c < 0) continue;
                Real val = 0;
                switch (item) {{
                {cases}
                default: break;
                }}
                lg[c] = val;
            }}
        }}'''


_CUBIC_HELPER = '''
// Two Newton steps on x^3 + b x^2 + c x + d = 0 from the estimate x: a
// root given by the trigonometric cubic formula differs from the sum of
// two nearly equal terms, which keeps few correct digits in single
// precision; two steps restore them (see cubic_root_coefficients)
static __device__ __forceinline__ Real mkg_cubic_root(Real x, Real b, Real c,
                                                      Real d)
{
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const Real f = ((x + b) * x + c) * x + d;
        const Real g = (3 * x + 2 * b) * x + c;
        if (g != 0) x = x - f / g;
    }
    return x;
}'''


def cubic_root_coefficients(rhs):
    """
    If ``rhs`` computes a root of ``x^3 + b x^2 + c x + d`` from three
    referenced variables (b, c, d) by a closed formula with ``acos`` and
    ``sqrt`` (the trigonometric solution some buffering models use for a
    free concentration), returns their references ``(b, c, d)``; else None.
    Detected numerically: for each assignment of the three references, the
    expression must return a root of test cubics with three real roots.
    """
    import itertools
    import warnings
    kinds = set(type(x) for x in rhs.walk())
    if myokit.ACos not in kinds or myokit.Sqrt not in kinds:
        return None
    refs = []
    for r in rhs.references():
        if r not in refs:
            refs.append(r)
    if len(refs) != 3 or not all(isinstance(r, myokit.Name) for r in refs):
        return None
    tests = [(1e-4, -0.05, -0.3), (2e-3, -0.01, -0.7), (0.5, -1.0, -2.0),
             (3.0, 1.0, -4.0), (2.5e-7, -0.003, -0.04)]
    for perm in itertools.permutations(refs):
        ok = True
        for r1, r2, r3 in tests:
            b = -(r1 + r2 + r3)
            c = r1 * r2 + r1 * r3 + r2 * r3
            d = -r1 * r2 * r3
            sub = {perm[0]: myokit.Number(b), perm[1]: myokit.Number(c),
                   perm[2]: myokit.Number(d)}
            try:
                with np.errstate(all='ignore'), warnings.catch_warnings():
                    warnings.simplefilter('ignore')
                    x = rhs.eval(subst=sub)
                x = float(x) if np.isreal(x) else float('nan')
            except Exception:
                ok = False
                break
            # Constants folded in single precision (2/3 and the like) move
            # the formula's value by a few parts in 1e8 of the roots' scale
            scale = max(abs(r1), abs(r2), abs(r3))
            if not (np.isfinite(x) and min(abs(x - r) for r in (r1, r2, r3))
                    <= 1e-5 * scale):
                ok = False
                break
        if ok:
            return tuple(perm)
    return None


def _pow_helpers(single):
    """Inline helpers for x^n (n = 2..16, by repeated squaring) and x^1.5
    and, in single precision, the cubic root refinement."""
    out = []
    for n in range(2, 17):
        lines = []
        # binary exponentiation, most significant bit first
        bits = bin(n)[3:]
        cur = 'x'
        k = 0
        for b in bits:
            lines.append(f'    const Real s{k} = {cur} * {cur};')
            cur = f's{k}'
            k += 1
            if b == '1':
                lines.append(f'    const Real s{k} = {cur} * x;')
                cur = f's{k}'
                k += 1
        out.append(
            f'static __device__ __forceinline__ Real mkg_pow{n}(Real x)\n'
            '{\n' + '\n'.join(lines) + f'\n    return {cur};\n}}')
    sq = 'sqrtf' if single else 'sqrt'
    out.append('static __device__ __forceinline__ Real mkg_pow1p5(Real x)'
               f' {{ return x * {sq}(x); }}')
    if single:
        out.append(_CUBIC_HELPER)
    return '\n'.join(out)


def _constant_subtrees(e):
    """The largest subexpressions of ``e`` that reference no variable and
    are more than a number (conditions are kept, their operands searched)."""
    if isinstance(e, myokit.Number):
        return []
    if not isinstance(e, myokit.Condition) and not any(
            True for _ in e.references()):
        return [e]
    out = []
    for op in e:
        out.extend(_constant_subtrees(op))
    return out


def _read(name):
    with open(os.path.join(_CSRC, name), 'r') as f:
        return f.read()


# Shared-memory staging of warp-tile inputs with TMA (tensor copies). The
# same rule is restated by stage_layout() in csrc/mkg_host.cu, which builds
# the tensor maps and sizes the dynamic shared memory; the kernel refuses
# to run when the two disagree on the bytes per tile.
STAGE_VW = 40            # staged V / conductance row: 32 cells + halo + pad
STAGE_MAX_BOX = 256      # planes per tensor copy
STAGE_MAX_CTA = 200 * 1024


def stage_layout(real_bytes, n_state, i_vm, n_field, n_hi, hi_bytes, v_bytes,
                 v_rows, gx, row_pad):
    """
    Per-warp shared-memory layout of one staged warp tile. Tile inputs are
    copied from x = the tile's first cell, rounded down to a multiple of 4
    cells when rows are not 4-cell aligned (``row_pad``; the copy is then
    36 cells wide, else 32), so that every copy starts on a 16-byte
    boundary. V rows (and 1D conductances) start one cell earlier, rounded
    down the same way, and are 40 wide. Every copy lands on a 128-byte
    aligned address: regions, and each V row within its region
    (``v_row_bytes`` apart), are padded to multiples of 128 bytes.

    Returns a dict with the tile width ``sw``, the first staged state plane
    ``lo`` and count ``np`` (the membrane potential plane is skipped when it
    is the first or last state), region offsets, ``bytes`` per warp and
    ``tx``, the bytes the copies of one tile deliver.
    """
    sw = 36 if row_pad else 32
    v_row = (STAGE_VW * v_bytes + 127) // 128 * 128
    lo, hi = 0, n_state
    if i_vm >= 0:
        if i_vm == 0:
            lo = 1
        if i_vm == n_state - 1:
            hi = n_state - 1
    npl = max(0, hi - lo)
    sizes = [
        ('state', npl * sw * real_bytes),
        ('hi', n_hi * sw * hi_bytes),
        ('field', n_field * sw * real_bytes),
        ('v', v_rows * STAGE_VW * v_bytes),
        ('gx', STAGE_VW * real_bytes if gx else 0),
    ]
    out = {'sw': sw, 'vw': STAGE_VW, 'lo': lo, 'np': npl, 'v_rows': v_rows,
           'gx': 1 if gx else 0, 'v_row_bytes': v_row}
    off = 0
    tx = 0
    for name, n in sizes:
        out[name + '_off'] = off
        room = v_rows * v_row if name == 'v' else n
        off += (room + 127) // 128 * 128
        tx += n
    out['bytes'] = off
    out['tx'] = tx
    return out


class TissueKernel(object):
    """
    The generated CUDA source for one simulation configuration, with the
    metadata the host needs (state order, logged intermediaries, census).

    Arguments:

    ``model``
        A cloned model with unique names created and bindings prepared, as
        held by :class:`SimulationCUDA` (``openclsim.py:276-290``).
    ``precision``
        ``myokit.SINGLE_PRECISION`` or ``myokit.DOUBLE_PRECISION``.
    ``native_math``
        Use fast hardware approximations for single precision functions.
    ``bound_variables``
        Map from bound variables to ``'time'``, ``'pace'`` or ``'idiff'``.
    ``inter_log``
        Intermediary variables whose values are logged.
    ``diffusion``
        One of ``DIFF_NONE``, ``DIFF_GRID``, ``DIFF_HETERO``, ``DIFF_CONN``.
    ``two_d``
        True for an ``(nx, ny)`` grid.
    ``fields``
        Variables replaced by per-cell scalar fields, in field order.
    ``rl_states``
        Map ``{state: (inf, tau)}`` of Rush-Larsen states.
    ``block``
        CTA shape ``(bx, by)``.
    ``fast_divide``
        Single precision only: use the 2-ulp division of the hardware,
        within the 2.5 ulp that OpenCL allows for ``x / y`` by default.
    ``math``
        Single precision only: ``'default'`` (the above), ``'ieee'``
        (correctly rounded division), or ``'fast'`` (reciprocal
        multiplication for constant denominators, the hardware reciprocal
        elsewhere, denormals flushed to zero).
    ``stage``
        Copy each warp tile's states, accumulation planes, fields and V
        rows into shared memory with TMA tensor copies, one tile ahead of
        the computation (ignored when the layout does not fit).
    ``row_pad``
        Rows of the grid are not a multiple of 4 cells (2D only): staged
        copies are then 36 cells wide.
    ``sync``
        ``'barrier'``: a grid-wide barrier between steps; ``'neighbors'``:
        each warp waits only for the warps owning its halo tiles (per-warp
        step counters). Connection graphs always use the barrier.
    ``stage_lazy``
        With staging: read staged values from shared memory where they are
        used, instead of reading them all into registers first and copying
        the next tile ahead. Needs fewer registers, so more warps fit on an
        SM. ``1`` (or True): one buffer per warp, the next tile's copies
        start after the computation; ``2``: two buffers per warp, the tile
        after the next is copied while a tile computes (twice the shared
        memory).
    """
    def __init__(self, model, precision, native_math, bound_variables,
                 inter_log, diffusion, two_d, fields, rl_states, block,
                 fast_divide=True, min_blocks=1, math='default',
                 accumulate=None, accumulate_states=(), traj=False,
                 stage=False, row_pad=False, stage_lazy=False,
                 sync='barrier', split=1):
        self.model = model
        self.single = (precision == myokit.SINGLE_PRECISION)
        self.native_math = bool(native_math)
        self.bound = dict(bound_variables)
        self.inter_log = list(inter_log)
        self.diffusion = int(diffusion)
        self.two_d = bool(two_d) and self.diffusion in (DIFF_GRID, DIFF_HETERO)
        self.fields = list(fields)
        self.rl_states = dict(rl_states)
        self.block = (int(block[0]), int(block[1]))
        self.math = str(math) if self.single else 'ieee'
        if self.math not in ('default', 'ieee', 'fast'):
            raise ValueError('math must be default, ieee or fast')
        self.fast_divide = (bool(fast_divide) and self.single
                            and self.math != 'ieee')
        self.min_blocks = int(min_blocks)
        self.states = list(model.states())
        self.n_state = len(self.states)
        self.vm = model.label('membrane_potential')
        if self.diffusion != DIFF_NONE:
            self.i_vm = self.vm.index()
        else:
            self.i_vm = -1
        # States accumulated in FP64 or with a Kahan-compensated FP32 update
        # (single precision only; Rush-Larsen gates never need it)
        if accumulate not in (None, 'double', 'kahan'):
            raise ValueError('accumulate must be None, "double" or "kahan"')
        self.accumulate = accumulate if self.single else None
        self.hi_states = []
        if self.accumulate:
            chosen = set(accumulate_states)
            for i, st in enumerate(self.states):
                if st in chosen and st not in self.rl_states:
                    self.hi_states.append(i)
        self.hi_index = {i: j for j, i in enumerate(self.hi_states)}
        self.v_double = (self.accumulate == 'double' and
                         self.i_vm in self.hi_index)
        self.traj = bool(traj)
        # Warps per warp tile (1, 2, 4, 8 or 16). Split teams read their
        # states themselves and meet at a team barrier, so they take none
        # of tile staging, accumulation planes, trajectory output or
        # neighbour synchronisation; where one of those is asked for the
        # kernel is not split. A team is either part of one CTA (at most
        # 15 teams per CTA: named barriers 1-15) or a cluster of 2 to 8
        # whole CTAs (split_cl CTAs: a team larger than the CTA); other
        # shapes are not split either.
        self.split = int(split)
        if self.split not in (1, 2, 4, 8, 16):
            raise ValueError('split must be 1, 2, 4, 8 or 16')
        nwarp = self.block[0] // 32
        if self.split > 1 and (
                self.accumulate or self.traj or self.block[1] != 1):
            self.split = 1
        if self.split > nwarp:
            if self.split % nwarp or self.split // nwarp > 8:
                self.split = 1
        elif self.split > 1 and (nwarp % self.split or
                                 nwarp // self.split > 15):
            self.split = 1
        self.split_cl = max(1, self.split // nwarp)
        self.split_nslot = 0
        self.split_terms = {}
        self.split_term_exprs = {}
        if self.split > 1:
            stage = False
            sync = 'barrier'
        self.stage = bool(stage)
        self.row_pad = bool(row_pad) and self.two_d
        self.stage_lazy = int(stage_lazy)
        if self.stage_lazy not in (0, 1, 2):
            raise ValueError('stage_lazy must be 0, 1 or 2')
        if sync not in ('barrier', 'neighbors'):
            raise ValueError('sync must be "barrier" or "neighbors"')
        # Connection graphs have arbitrary neighbours: grid barrier only
        self.sync = sync if self.diffusion != DIFF_CONN else 'barrier'
        self.layout = None
        if self.stage:
            real = 4 if self.single else 8
            v_rows = 0
            if self.diffusion in (DIFF_GRID, DIFF_HETERO):
                v_rows = 3 if self.two_d else 1
            lay = stage_layout(
                real, self.n_state, self.i_vm, len(self.fields),
                len(self.hi_states),
                8 if self.accumulate == 'double' else real,
                8 if self.v_double else real, v_rows,
                self.diffusion == DIFF_HETERO and not self.two_d,
                bool(row_pad) and self.two_d)
            per_cta = lay['bytes'] * (self.block[0] // 32)
            if (max(lay['np'], len(self.hi_states), len(self.fields))
                    <= STAGE_MAX_BOX and per_cta <= STAGE_MAX_CTA):
                self.layout = lay
                # Two buffers per warp only where they fit
                if self.stage_lazy == 2 and 2 * per_cta > STAGE_MAX_CTA:
                    self.stage_lazy = 1
        # Staging buffers per warp (mkg_config.stage)
        self.stage_buffers = 2 if self.layout and self.stage_lazy == 2 \
            else 1
        self.census = OpCensus()
        # Single precision: variables computed by the trigonometric cubic
        # formula, refined by mkg_cubic_root: name -> (b, c, d) names
        self.cubic = {}
        self._source = self._generate()

    # -- naming ------------------------------------------------------------

    def _name(self, x):
        """C name of a variable or LhsExpression."""
        if isinstance(x, myokit.Derivative):
            return 'd_' + x.var().uname()
        if isinstance(x, myokit.Name):
            x = x.var()
        b = self.bound.get(x)
        if b == 'time':
            return _T
        if b == 'pace':
            return _PACE
        if b == 'idiff':
            return _IDIFF
        if x.is_state():
            return 'x_' + x.uname()
        return 'v_' + x.uname()

    # -- generation --------------------------------------------------------

    def _generate(self):
        m = self.model
        w = CudaExpressionWriter(self.single, self.native_math,
                                 self.math == 'fast')
        w.set_lhs_function(self._name)
        real = 'float' if self.single else 'double'
        prec = myokit.SINGLE_PRECISION if self.single else \
            myokit.DOUBLE_PRECISION

        order = m.solvable_order()
        remaining = order.pop('*remaining*', None)
        if remaining is not None and len(remaining) > 0:
            raise ValueError(
                'This simulation requires models without interdependent'
                ' components.')

        field_set = set(self.fields)

        # Constants that depend (directly or not) on a field must be computed
        # per cell; all others are folded to literals on the host.
        percell_const = set()
        const_eqs = []
        for group in order.values():
            for eq in group.equations(const=True):
                const_eqs.append(eq)
        changed = True
        while changed:
            changed = False
            for eq in const_eqs:
                var = eq.lhs.var()
                if var in percell_const:
                    continue
                if var in field_set:
                    percell_const.add(var)
                    changed = True
                    continue
                for ref in eq.rhs.references():
                    if ref.var() in percell_const:
                        percell_const.add(var)
                        changed = True
                        break

        # Host-folded constant values (in the simulation precision)
        literal_subst = {}
        for eq in const_eqs:
            var = eq.lhs.var()
            if var in percell_const or var in self.bound:
                continue
            value = eq.rhs.eval(precision=prec)
            literal_subst[myokit.Name(var)] = myokit.Number(float(value))

        def fold(e):
            if literal_subst:
                e = e.clone(subst=literal_subst)
            # Subexpressions of literals only (e.g. sqrt(Ko / 5.4) beside a
            # per-cell field) are evaluated here, like the folded constants
            sub = {}
            for c in _constant_subtrees(e):
                sub[c] = myokit.Number(float(c.eval(precision=prec)))
            return e.clone(subst=sub) if sub else e

        body = []
        tab = '        '

        # Per-cell constants (fields and what depends on them), in order
        # Recorded for the adjoint exporter: per-cell constant equations and
        # the right-hand side equations, in evaluation order, with constants
        # folded (lists of (lhs, folded rhs)).
        self.writer = w
        self.literal_subst = literal_subst
        self.cell_const_eqs = []
        self.rhs_eqs = []
        # Scalar fields are read with the states (below); constants that
        # depend on them are computed per cell here.
        lay = self.layout
        sw = lay['sw'] if lay else 0
        # Lazy staging binds names to the staged values in shared memory
        amp = '&' if lay and self.stage_lazy else ''
        field_loads = []
        for k, var in enumerate(self.fields):
            src = (f's_fd[{k * sw}]' if lay else
                   f'field[(long long){k} * pitch + cid]')
            field_loads.append(
                f'{tab}const Real {amp}{self._name(var)} = {src};')
        # (name, referenced names, line, cost) of every equation in body
        # order, for kernels that divide a tile's work among warps
        items = []

        def item(lhs, rhs, line):
            refs = set(self._name(r) for r in rhs.references())
            c = OpCensus()
            c.add(rhs)
            items.append((self._name(lhs), refs, line, c.cost()))

        body.append(tab + '// Per-cell constants (scalar fields)')
        for eq in const_eqs:
            var = eq.lhs.var()
            if var in percell_const and var not in field_set:
                rhs = fold(eq.rhs)
                self.cell_const_eqs.append((eq.lhs, rhs))
                self.census.add(rhs)
                line = f'{tab}const Real {self._name(var)} = {w.ex(rhs)};'
                body.append(line)
                item(var, rhs, line)

        def ref(var):
            # Name of a variable, or its literal when it was folded
            x = literal_subst.get(myokit.Name(var))
            return w.ex(x) if x is not None else self._name(var)

        # State loads, and the update of each state, emitted as soon as its
        # inputs exist so that derivatives do not stay live to the end.
        # States in self.hi_states live in the accumulation planes (hi):
        # FP64 values ('double') or FP32 compensation terms ('kahan'; the
        # state is x - c, updated with Kahan's compensated sum).
        loads = []
        updates = []
        state_src = []       # (name, value at t) per state, plain loads
        # (target, new value) of each plain update, for split kernels,
        # which write the states after the team has read them
        self._upd_expr = {}
        hiD = '((double *)hi)'
        hiR = '((Real *)hi)'
        for i, s in enumerate(self.states):
            n = self._name(s)
            j = self.hi_index.get(i)
            plane = f'(long long){i} * pitch + cid'
            if j is not None:
                hplane = f'(long long){j} * pitch + cid'
            if lay:
                # Staged in shared memory (see stage_layout)
                src = f's_st[{(i - lay["lo"]) * sw}]'
                hsrc = f's_hi[{j * sw}]' if j is not None else None
            else:
                src = f'state[{plane}]'
                hsrc = None
            state_src.append((n, '(Real)V_' if i == self.i_vm else src))
            if i == self.i_vm:
                loads.append(f'{tab}const Real {n} = (Real)V_;')
            elif j is not None and self.accumulate == 'double':
                loads.append(
                    f'{tab}const double {amp}X{n} = '
                    f'{hsrc or hiD + "[" + hplane + "]"};')
                loads.append(f'{tab}const Real {n} = (Real)X{n};')
            else:
                loads.append(f'{tab}const Real {amp}{n} = {src};')
            if j is not None and self.accumulate == 'kahan':
                loads.append(
                    f'{tab}const Real {amp}C{n} = '
                    f'{hsrc or hiR + "[" + hplane + "]"};')
            target = 'vout[cid]' if i == self.i_vm else f'state[{plane}]'
            if s in self.rl_states:
                inf, tau = self.rl_states[s]
                need = set(
                    self._name(v) for v in (inf, tau)
                    if myokit.Name(v) not in literal_subst)
                inf, tau = ref(inf), ref(tau)
                expf = w._fn('exp')
                upd = f'{inf} - ({inf} - {n}) * {expf}(-dt_ / {tau})'
                text = f'{tab}{target} = {upd};'
                self._upd_expr[i] = (target, upd)
                self.census.arith += 4
                self.census.trans += 1
            else:
                d = self._name(s.lhs())
                need = set([d])
                self.census.arith += 2
                if j is None:
                    text = f'{tab}{target} = {n} + dt_ * {d};'
                    self._upd_expr[i] = (target, f'{n} + dt_ * {d}')
                elif self.accumulate == 'double':
                    cur = 'V_' if i == self.i_vm else f'X{n}'
                    dst = target if i == self.i_vm else f'{hiD}[{hplane}]'
                    text = f'{tab}{dst} = {cur} + (double)(dt_ * {d});'
                else:
                    text = (
                        f'{tab}{{ const Real y_ = dt_ * {d} - C{n};\n'
                        f'{tab}  const Real s_ = {n} + y_;\n'
                        f'{tab}  {hiR}[{hplane}] = (s_ - {n}) - y_;\n'
                        f'{tab}  {target} = s_; }}')
                    self.census.arith += 3
            updates.append((i, need, text))

        defined = set(self._name(v) for v in self.fields)
        for eq in const_eqs:
            if eq.lhs.var() in percell_const:
                defined.add(self._name(eq.lhs.var()))
        emitted = set()

        def flush():
            for i, need, text in updates:
                if i not in emitted and need <= defined:
                    body.append(text)
                    emitted.add(i)

        # The derivative of a Rush-Larsen state is not needed for its update.
        # The reference skips its equation but still declares it, as a
        # component output initialised to zero (openclsim.cl:236-238,
        # 341-343), so other equations that refer to dot(x) see 0. The same
        # zero is defined here for the derivatives that are referred to.
        used_dots = set()
        for group in order.values():
            for eq in group.equations(const=False):
                for r in eq.rhs.references():
                    if isinstance(r, myokit.Derivative):
                        used_dots.add(r.var())

        # Equations in solvable order (the reference calls one function per
        # component in this order, openclsim.cl:336-352).
        body.append(tab + '// Model right-hand side at time t')
        flush()
        for group in order.values():
            for eq in group.equations(const=False):
                var = eq.lhs.var()
                if var in self.bound:
                    continue
                if isinstance(eq.lhs, myokit.Derivative) and \
                        var in self.rl_states:
                    if var not in used_dots:
                        continue
                    rhs = myokit.Number(0)
                else:
                    rhs = fold(eq.rhs)
                self.rhs_eqs.append((eq.lhs, rhs))
                self.census.add(rhs)
                name = self._name(eq.lhs)
                if self.single and isinstance(eq.lhs, myokit.Name):
                    bcd = cubic_root_coefficients(rhs)
                    if bcd is not None:
                        self.cubic[name] = tuple(self._name(r) for r in bcd)
                        self.census.arith += 20
                line = f'{tab}const Real {name} = {self.rhs_code(eq.lhs, rhs)};'
                body.append(line)
                item(eq.lhs, rhs, line)
                defined.add(name)
                flush()
        if len(emitted) != len(updates):   # pragma: no cover
            raise ValueError('Could not order the state updates.')
        self._inter_names = [self._name(v) for v in self.inter_log]

        if self.traj:
            # The adjoint's forward pass records the states at t of every
            # step of the launch: traj[k][state][pitch]
            for i, st in enumerate(self.states):
                loads.append(
                    f'{tab}((Real *)a.traj)[((long long)k * {self.n_state}'
                    f' + {i}) * pitch + cid] = {self._name(st)};')

        # Logging: states and idiff right after the loads, intermediaries
        # at the end (item ids as in include/mkg_tissue.h).
        t2 = tab + '    '
        cases = [f'case {i}: val = {self._name(s)}; break;'
                 for i, s in enumerate(self.states)]
        cases.append(f'case {self.n_state}: val = {_IDIFF}; break;')
        log_a = _LOG_BLOCK.format(
            cond=f'item <= {self.n_state}',
            cases=('\n' + t2 + '        ').join(cases))
        first = self._name(self.states[0])
        log_a += (
            f'\n{tab}if (row >= 0 && a.nan_check && cid == 0 && '
            f'isnan({first}))\n{tab}    atomicMin(&a.status->halt_step, a.step0 + k);')
        log_b = ''
        if self.inter_log:
            cases = [f'case {self.n_state + 1 + k}: val = {name}; break;'
                     for k, name in enumerate(self._inter_names)]
            log_b = _LOG_BLOCK.format(
                cond=f'item > {self.n_state}',
                cases=('\n' + t2 + '        ').join(cases))

        split_body = ''
        if self.split > 1:
            split_body = self._split_body(
                items, updates, state_src, field_loads, log_a, log_b)
        self.split_body = split_body

        subs = {
            '@SPLIT@': str(self.split),
            '@SPLIT_CL@': str(self.split_cl),
            '@SPLIT_NSLOT@': str(self.split_nslot),
            '@SPLIT_BODY@': split_body,
            '@REAL@': real,
            '@VREAL@': 'double' if self.v_double else real,
            '@SINGLE@': '1' if self.single else '0',
            '@N_STATE@': str(self.n_state),
            '@N_FIELD@': str(len(self.fields)),
            '@N_INTER@': str(len(self.inter_log)),
            '@I_VM@': str(self.i_vm),
            '@DIFF@': str(self.diffusion),
            '@TWO_D@': '1' if self.two_d else '0',
            '@BX@': str(self.block[0]),
            '@BY@': str(self.block[1]),
            '@MINB@': str(self.min_blocks),
            '@POW_HELPERS@': _pow_helpers(self.single),
            '@LOADS@': '\n'.join(loads + field_loads),
            '@LOG_A@': log_a,
            '@BODY@': '\n'.join(body),
            '@LOG_B@': log_b,
        }
        # The per-cell pieces, for kernels that assemble several models
        self.parts = {
            'loads': subs['@LOADS@'], 'log_a': log_a,
            'body': subs['@BODY@'], 'log_b': log_b,
        }
        lay = self.layout or {}
        subs.update({
            '@NBR_SYNC@': '1' if self.sync == 'neighbors' else '0',
            '@STAGE@': '1' if self.layout else '0',
            '@STAGE_LAZY@': '1' if self.layout and self.stage_lazy else '0',
            '@STAGE_BUFS@': '2' if self.layout and self.stage_lazy == 2
            else '1',
            '@SW@': str(lay.get('sw', 32)),
            '@VW@': str(STAGE_VW),
            '@ST_LO@': str(lay.get('lo', 0)),
            '@ST_NP@': str(lay.get('np', 0)),
            '@HI_NP@': str(len(self.hi_states) if lay else 0),
            '@FD_NP@': str(len(self.fields) if lay else 0),
            '@V_ROWS@': str(lay.get('v_rows', 0)),
            '@GX_STAGE@': str(lay.get('gx', 0)),
            '@ST_OFF@': str(lay.get('state_off', 0)),
            '@HI_OFF@': str(lay.get('hi_off', 0)),
            '@FD_OFF@': str(lay.get('field_off', 0)),
            '@V_OFF@': str(lay.get('v_off', 0)),
            '@GX_OFF@': str(lay.get('gx_off', 0)),
            '@V_ROW_BYTES@': str(lay.get('v_row_bytes', 0)),
            '@STAGE_BYTES@': str(lay.get('bytes', 0)),
            '@TX_BYTES@': str(lay.get('tx', 0)),
            '@HREAL@': 'double' if self.accumulate == 'double' else real,
        })
        text = _read('tissue_kernel.cu.in')
        for k, v in subs.items():
            text = text.replace(k, v)
        abi = _read('mkg_kernel_abi.h')
        return (
            '// Generated by myokit_gb300.exporter for model '
            + str(m.name()) + '\n' + abi + '\n' + text)

    def _split_terms(self, rhs_of):
        """
        Additive decomposition of an expression into (coefficient, term)
        pairs: through sums, differences, negation, multiplication and
        division by literals, and references to intermediary variables
        whose own right-hand sides decompose (cubic roots excluded, their
        refinement needs the whole expression).
        """
        def terms(e, c):
            if isinstance(e, myokit.PrefixPlus):
                return terms(e[0], c)
            if isinstance(e, myokit.PrefixMinus):
                return terms(e[0], -c)
            if isinstance(e, myokit.Plus):
                return terms(e[0], c) + terms(e[1], c)
            if isinstance(e, myokit.Minus):
                return terms(e[0], c) + terms(e[1], -c)
            if isinstance(e, myokit.Multiply):
                for i in (0, 1):
                    if isinstance(e[i], myokit.Number):
                        return terms(e[1 - i], c * float(e[i].eval()))
            if isinstance(e, myokit.Divide) and \
                    isinstance(e[1], myokit.Number):
                den = float(e[1].eval())
                if den != 0:
                    return terms(e[0], c / den)
            if isinstance(e, myokit.Name):
                n = self._name(e)
                if n in rhs_of and n not in self.cubic:
                    return terms(rhs_of[n], c)
            return [(c, e)]
        return terms

    def _split_body(self, items, updates, state_src, field_loads, log_a,
                    log_b):
        """
        The per-warp code of a split tile. The work units are the updates
        of the states, except that the derivative of a forward-Euler state
        that no other equation uses is divided into its additive terms
        (the currents of dV/dt, the alpha and beta terms of a gate), each a
        unit of its own. Units are assigned greedily, from the costliest
        down, to the warp whose share (every equation it needs, counted
        once per warp that needs it) then stays smallest. A warp that holds
        terms of another warp's state sums them and hands the partial sum
        over in shared memory (distributed shared memory of the owner's
        CTA when the team spans a cluster); the owner adds the partial sums
        in a fixed order (the order of the warps), so results do not
        depend on timing. Every warp reads the states it needs at t,
        computes, and hands its partial sums over; the team then meets at
        its barrier, and each warp writes its own states at t + dt. Warp 0
        also logs and checks the NaN halt, so it reads every state and
        computes the logged intermediaries.
        """
        P = self.split
        nwarp = self.block[0] // 32
        w = self.writer
        refs = {name: r for name, r, _, _ in items}
        cost = {name: c for name, _, _, c in items}
        rhs_of = {self._name(lhs): rhs for lhs, rhs in self.rhs_eqs
                  if isinstance(lhs, myokit.Name)}
        terms = self._split_terms(rhs_of)

        def closure(roots):
            out = set()
            todo = list(roots)
            while todo:
                n = todo.pop()
                if n in out or n not in refs:
                    continue
                out.add(n)
                todo.extend(refs[n])
            return out

        # Derivatives another equation (or the log) refers to are computed
        # whole
        used = set(self._inter_names)
        for r in refs.values():
            used |= r
        dexpr = {self._name(lhs): rhs for lhs, rhs in self.rhs_eqs
                 if isinstance(lhs, myokit.Derivative)}

        # Units: (state, term index or None, needed equations, own cost)
        units = []
        split_terms = {}     # state -> [(coefficient, term), ...]
        for i, need, text in updates:
            s = self.states[i]
            d = self._name(s.lhs())
            tl = None
            if s not in self.rl_states and d not in used and d in dexpr:
                tl = terms(dexpr[d], 1.0)
                if len(tl) < 2 or len(tl) > 256:
                    tl = None
            if tl is None:
                own = 24 if s in self.rl_states else 2
                units.append((i, None, closure(need), own))
                continue
            split_terms[i] = tl
            for k, (c, e) in enumerate(tl):
                cen = OpCensus()
                cen.add(e)
                r = set(self._name(x) for x in e.references())
                units.append((i, k, closure(r), cen.cost() + 2))

        groups = [set() for _ in range(P)]
        owns = [0] * P
        assign = [[] for _ in range(P)]     # units per warp
        groups[0] |= closure(self._inter_names)

        def gcost(g, extra=frozenset()):
            return sum(cost[n] for n in groups[g] | extra)
        for u in sorted(units,
                        key=lambda u: -(sum(cost[n] for n in u[2]) + u[3])):
            g = min(range(P), key=lambda g: (gcost(g, u[2]) + owns[g] + u[3],
                                             g))
            groups[g] |= u[2]
            owns[g] += u[3]
            assign[g].append(u)

        # Owner of each divided state: the warp holding its costliest term
        holders = {i: [] for i in split_terms}
        for g in range(P):
            for i, k, _, own in assign[g]:
                if k is not None and g not in holders[i]:
                    holders[i].append(g)
        owner = {}
        for i in split_terms:
            best = max((own, -g) for g in range(P)
                       for j, k, _, own in assign[g] if j == i and k is not None)
            owner[i] = -best[1]
            holders[i].sort()
            owns[owner[i]] += len(holders[i])
        # Shared-memory slots: one per (state, warp other than the owner)
        slot = {}
        for i in sorted(split_terms):
            for g in holders[i]:
                if g != owner[i]:
                    slot[(i, g)] = len(slot)
        self.split_nslot = len(slot)
        self.split_terms = {self.states[i].qname(): len(t)
                            for i, t in split_terms.items()}
        # The (coefficient, term) lists themselves, per divided state
        self.split_term_exprs = {self.states[i].qname(): list(t)
                                 for i, t in split_terms.items()}
        self.split_costs = [gcost(g) + owns[g] for g in range(P)]

        def coef_term(c, e, first, acc):
            t = w.ex(e)
            if c == 1.0:
                return f'{acc} = {t};' if first else f'{acc} += {t};'
            if c == -1.0:
                return f'{acc} = -({t});' if first else f'{acc} -= {t};'
            cc = w.ex(myokit.Number(c))
            return (f'{acc} = {cc} * ({t});' if first
                    else f'{acc} += {cc} * ({t});')

        tab = '            '
        out = []
        for p in range(P):
            whole = [i for i, k, _, _ in assign[p] if k is None]
            mine_terms = {}
            for i, k, _, _ in assign[p]:
                if k is not None:
                    mine_terms.setdefault(i, []).append(k)
            owned = [i for i in split_terms if owner[i] == p]
            # States read: those the part's equations and updates use
            read = set(self._name(self.states[i]) for i in whole + owned)
            for n in groups[p]:
                read |= refs[n]
            for i, ks in mine_terms.items():
                for k in ks:
                    read |= set(self._name(x)
                                for x in split_terms[i][k][1].references())
            sts = [(n, src) for n, src in state_src
                   if p == 0 or n in read]
            out.append(f'{tab}{"if" if p == 0 else "else if"} (part_ == {p})'
                       ' {')
            for n, _ in sts:
                out.append(f'{tab}    Real {n} = 0;')
            for i in whole:
                out.append(f'{tab}    Real n{i}_ = 0;')
            for i in sorted(mine_terms):
                out.append(f'{tab}    Real q{i}_ = 0;')
            out.append(f'{tab}    if (live) {{')
            for n, src in sts:
                out.append(f'{tab}        {n} = {src};')
            out.append(f'{tab}    const Real idiff_ = (Real)id_;')
            out.append(f'{tab}    (void)idiff_;')
            out.append(f'{tab}    const Real pace_ = mkg_cell_pace(a, ix, iy,'
                       ' cid, pace_in);')
            out.append(f'{tab}    (void)pace_;')
            out.extend(field_loads)
            if p == 0:
                out.append(log_a)
            defined = set()
            done = set()
            pend = [(i, k) for i in sorted(mine_terms)
                    for k in mine_terms[i]]
            started = set()

            def flush():
                for i, need, text in updates:
                    if i in whole and i not in done and need <= defined:
                        out.append(f'{tab}    n{i}_ = '
                                   f'{self._upd_expr[i][1]};')
                        done.add(i)
                for ik in list(pend):
                    i, k = ik
                    c, e = split_terms[i][k]
                    r = set(self._name(x) for x in e.references())
                    if (r & set(refs)) <= defined:
                        out.append(f'{tab}    ' + coef_term(
                            c, e, i not in started, f'q{i}_'))
                        started.add(i)
                        pend.remove(ik)
            flush()
            for name, _, line, _ in items:
                if name in groups[p]:
                    out.append(line)
                    defined.add(name)
                    flush()
            if done != set(whole) or pend:   # pragma: no cover
                raise ValueError('Could not order the state updates.')
            if p == 0:
                out.append(log_b)
            # Partial sums of other warps' states
            for i in sorted(mine_terms):
                if owner[i] == p:
                    continue
                s = slot[(i, p)]
                r = owner[i] // nwarp
                if P > nwarp and r != p // nwarp:
                    out.append(f'{tab}    MKG_PP_PUT({s}, {r}, q{i}_);')
                else:
                    out.append(f'{tab}    MKG_PP_LOCAL({s}, q{i}_);')
            out.append(f'{tab}    }}')
            out.append(f'{tab}    // the team read its states at t and'
                       ' handed its partial sums over')
            out.append(f'{tab}    mkg_team_sync();')
            out.append(f'{tab}    if (live) {{')
            for i in whole:
                out.append(f'{tab}        {self._upd_expr[i][0]} = n{i}_;')
            for i in owned:
                parts = [f'q{i}_' if g == p else f'MKG_PP_GET({slot[(i, g)]})'
                         for g in holders[i]]
                acc = parts[0]
                for t in parts[1:]:
                    acc = f'({acc} + {t})'
                n = self._name(self.states[i])
                out.append(f'{tab}        {self._upd_expr[i][0]} = '
                           f'{n} + dt_ * {acc};')
            out.append(f'{tab}    }}')
            out.append(f'{tab}}}')
        return '\n'.join(out)

    def rhs_code(self, lhs, rhs):
        """CUDA expression for an equation's right-hand side, with the
        cubic root refinement where it applies."""
        text = self.writer.ex(rhs)
        bcd = self.cubic.get(self._name(lhs))
        if bcd is not None:
            text = f'mkg_cubic_root({text}, {bcd[0]}, {bcd[1]}, {bcd[2]})'
        return text

    # -- public ------------------------------------------------------------

    def source(self):
        """Returns the CUDA C++ source text."""
        return self._source

    def options(self):
        """NVRTC options for this kernel."""
        opts = [
            '--gpu-architecture=sm_103a',
            '--std=c++17',
            '-lineinfo',
            '--extra-device-vectorization',
        ]
        if self.single:
            if self.fast_divide:
                opts.append('--prec-div=false')
            opts.append('--prec-sqrt=false' if self.native_math else
                        '--prec-sqrt=true')
            opts.append('--ftz=true' if self.math == 'fast' else '--ftz=false')
        opts.append('--fmad=true')
        return opts

    def key(self):
        """A hash identifying the source and options, for the cubin cache."""
        h = hashlib.sha256()
        h.update(self._source.encode())
        h.update('\0'.join(self.options()).encode())
        return h.hexdigest()

    def bytes_per_cell_step(self):
        """
        Algorithmic bytes per cell-step: one read and one write of every
        state, one read of every field and, for heterogeneous grids, of two
        conductances. Neighbour V reads count as on-chip hits.
        """
        r = 4 if self.single else 8
        b = 2 * self.n_state * r + len(self.fields) * r
        # FP64 storage doubles a state's bytes; a Kahan term adds a Real
        b += 2 * len(self.hi_states) * (8 - r if self.accumulate == 'double'
                                        else r)
        if self.diffusion == DIFF_HETERO:
            b += 2 * r
        return b

    def flops_per_cell_step(self):
        """Arithmetic operations per cell-step (excluding transcendentals),
        plus about 8 for the diffusion current."""
        return self.census.arith + (8 if self.diffusion else 0)


class FiberTissueKernel(object):
    """
    One fused kernel for ``FiberTissueSimulationCUDA``: the fiber's and the
    tissue's generated cell code (from two :class:`TissueKernel` objects,
    both for homogeneous 2D grid diffusion without staging) in one launch,
    with the junction current between the fiber's last column and the
    tissue's first (``openclsim.cl:601-628``).
    """
    def __init__(self, fiber, tissue):
        if fiber.single != tissue.single:
            raise ValueError('Both kernels must have the same precision.')
        if fiber.block != tissue.block:
            raise ValueError('Both kernels must have the same CTA shape.')
        for k in (fiber, tissue):
            if k.diffusion != DIFF_GRID or not k.two_d or k.layout:
                raise ValueError('Fiber-tissue kernels use 2D homogeneous'
                                 ' diffusion without tile staging.')
        self.fiber = fiber
        self.tissue = tissue
        self.single = fiber.single
        self.block = fiber.block
        self.min_blocks = fiber.min_blocks
        text = _read('fiber_tissue_kernel.cu.in')
        subs = {
            '@REAL@': 'float' if self.single else 'double',
            '@SINGLE@': '1' if self.single else '0',
            '@BX@': str(self.block[0]),
            '@MINB@': str(self.min_blocks),
            '@POW_HELPERS@': _pow_helpers(self.single),
        }
        for name, k in (('FIBER', fiber), ('TISSUE', tissue)):
            for part in ('loads', 'log_a', 'body', 'log_b'):
                subs['@%s_%s@' % (name, part.upper())] = k.parts[part]
        for key, v in subs.items():
            text = text.replace(key, v)
        self._source = (
            '// Generated by myokit_gb300.exporter for models '
            + str(fiber.model.name()) + ' (fiber) and '
            + str(tissue.model.name()) + ' (tissue)\n'
            + _read('mkg_kernel_abi.h') + '\n' + text)

    def source(self):
        return self._source

    def options(self):
        return self.fiber.options()

    def key(self):
        h = hashlib.sha256()
        h.update(self._source.encode())
        h.update('\0'.join(self.options()).encode())
        return h.hexdigest()
