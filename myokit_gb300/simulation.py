"""
``SimulationCUDA``: a drop-in for ``myokit.SimulationOpenCL`` that runs on
one GB300 through the host library in ``include/mkg_tissue.h``.

The public API, argument checks and error messages follow
``myokit/_sim/openclsim.py`` (class ``SimulationOpenCL``, line 23), so that
code and tests written for the reference run unchanged. What differs is the
backend: the model is exported to one fused CUDA kernel per configuration
(``myokit_gb300.exporter``), compiled once with NVRTC and cached, and the run
loop executes many steps per launch with the schedule, pacing and logging
kept on the device.
"""
import array
import hashlib
import os
import threading
from collections import OrderedDict

import numpy as np

from ._deps import myokit
from . import _lib
from . import exporter as _exp

# Cubin cache shared by all simulations in this process (key -> bytes)
_CUBIN_CACHE = {}
_CUBIN_LOCK = threading.Lock()


def _cache_dir():
    d = os.environ.get('MYOKIT_GB300_CACHE')
    if d is None:
        d = os.path.join(os.path.expanduser('~'), '.cache', 'myokit_gb300')
    return d


def compile_kernel(kernel):
    """
    Returns the sm_103a cubin for a :class:`TissueKernel`, compiling it with
    NVRTC on a cache miss. Cubins are cached in memory and on disk by the
    hash of source and options.
    """
    key = kernel.key()
    with _CUBIN_LOCK:
        data = _CUBIN_CACHE.get(key)
        if data is not None:
            return data
        path = os.path.join(_cache_dir(), key + '.cubin')
        try:
            with open(path, 'rb') as f:
                data = f.read()
        except OSError:
            data = None
        if not data:
            data, _ = _lib.compile_source(kernel.source(), kernel.options())
            try:
                os.makedirs(_cache_dir(), exist_ok=True)
                tmp = path + '.%d' % os.getpid()
                with open(tmp, 'wb') as f:
                    f.write(data)
                os.replace(tmp, path)
            except OSError:   # pragma: no cover
                pass
        _CUBIN_CACHE[key] = data
        return data


class _Backend(object):
    """One host-library handle plus the kernel it was created with."""
    def __init__(self, kernel, cfg):
        self.kernel = kernel
        self.lib = _lib.load()
        cubin = compile_kernel(kernel)
        handle = _lib.ctypes.c_void_p()
        _lib.check(self.lib.mkg_create(
            _lib.ctypes.byref(cfg), cubin, len(cubin),
            _lib.ctypes.byref(handle)))
        self.h = handle
        self.cfg = cfg
        # What the handle's log columns were last set to by run_frames
        # (None after any other setting): the frame columns of a large
        # grid are then not rebuilt and uploaded again for the next call
        self.log_sig = None

    def check(self, code):
        return _lib.check(code, self.h)

    def close(self):
        if self.h is not None and self.h.value:
            self.lib.mkg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:   # pragma: no cover
            pass


class SimulationCUDA(object):
    """
    Runs multi-cellular simulations of a myokit model on one NVIDIA GB300
    (sm_103a), with the API of :class:`myokit.SimulationOpenCL`.

    Arguments are those of ``SimulationOpenCL`` (``openclsim.py:149``):
    ``model``, ``protocol``, ``ncells`` (scalar for 1d, ``(nx, ny)`` for 2d),
    ``diffusion``, ``precision`` (``myokit.SINGLE_PRECISION`` or
    ``myokit.DOUBLE_PRECISION``), ``native_maths`` and ``rl``
    (Rush-Larsen updates for Hodgkin-Huxley gates). The cell update is a
    forward-Euler (or Rush-Larsen) step with a fixed step size, preceded by
    the diffusion current ``i = sum[g * (V - V_j)]`` over the neighbours
    ``j``; variables can bind to ``time``, ``pace`` and
    ``diffusion_current``.

    GPU-only keyword arguments:

    ``block``
        CTA shape ``(bx, by)`` of the generated kernel (2d grids) or the
        number of threads per CTA (1d). ``None`` picks a default.
    ``steps_per_launch``
        Time steps fused into one kernel launch (0 = a whole chunk).
    ``device``
        CUDA device ordinal.
    ``min_blocks``
        Minimum resident CTAs per SM asked of the compiler (caps registers).
    ``fp32_math``
        Single precision arithmetic. ``'fast'`` (the default): a division by
        a constant becomes a multiplication by its reciprocal (1.5 ulp),
        other divisions use the 2-ulp hardware reciprocal, denormals flush
        to zero -- all within what OpenCL allows single precision by
        default. ``'default'``: the compiler's 2-ulp division, denormals
        kept. ``'ieee'``: correctly rounded division.
    ``accumulate``
        Single precision only. ``None``: every state in FP32. ``'double'``:
        the selected states are stored and updated in FP64 while the
        right-hand side is evaluated in FP32. ``'kahan'``: the selected
        states stay FP32 and are updated with a compensated (Kahan) sum.
    ``accumulate_states``
        The states to accumulate; by default the membrane potential, states
        with concentration units and non-gating states of magnitude >= 1,
        whose per-step increments are smallest relative to their value.
    ``stage_tiles``
        Copy each warp tile's states, fields and V rows into shared memory
        with TMA tensor copies, one tile ahead of the computation (grids of
        256 cells or more). Results are identical either way.
    """
    _index = 0

    def __init__(
            self, model, protocol=None, ncells=256, diffusion=True,
            precision=myokit.SINGLE_PRECISION, native_maths=False, rl=False,
            block=None, steps_per_launch=0, device=0, min_blocks=None,
            fp32_math='fast', accumulate=None, accumulate_states=None,
            stage_tiles=True):

        # Model checks (openclsim.py:155-167)
        if not model.is_valid():
            model.validate()
        if model.has_interdependent_components():
            cycles = '\n'.join([
                '  ' + ' > '.join([x.name() for x in c])
                for c in model.component_cycles()])
            raise ValueError(
                'This simulation requires models without interdependent'
                ' components. Please restructure the model and re-run.'
                '\nCycles:\n' + cycles)

        self.set_protocol(protocol)

        # Dimensions (openclsim.py:172-189)
        try:
            self._nx = int(ncells)
            self._ny = 1
            self._dims = (self._nx,)
        except TypeError:
            try:
                assert len(ncells) == 2
            except (TypeError, AssertionError):
                raise ValueError(
                    'The argument "ncells" must be either a scalar or a tuple'
                    ' (nx, ny).')
            self._nx = int(ncells[0])
            self._ny = int(ncells[1])
            self._dims = (self._nx, self._ny)
        if self._nx < 1 or self._ny < 1:
            raise ValueError(
                'The number of cells in any direction must be at least 1.')
        self._ntotal = self._nx * self._ny

        self._diffusion_enabled = bool(diffusion)
        if precision not in (myokit.SINGLE_PRECISION,
                             myokit.DOUBLE_PRECISION):
            raise ValueError('Only single and double precision are supported.')
        self._precision = precision
        self._native_math = bool(native_maths)
        self._rl = bool(rl)

        # Membrane potential (openclsim.py:206-215)
        vm = model.label('membrane_potential')
        if self._diffusion_enabled or self._rl:
            if vm is None:
                raise ValueError(
                    'This simulation requires the membrane potential'
                    ' variable to be labelled as "membrane_potential".')
            if not vm.is_state():
                raise ValueError(
                    'The variable labelled as membrane potential must'
                    ' be a state variable.')

        # Rush-Larsen conversion and model clone (openclsim.py:217-246)
        self._rl_states = {}
        if self._rl:
            import myokit.lib.hh as hh
            self._model = hh.convert_hh_states_to_inf_tau_form(model, vm)
            self._vm = self._model.get(vm.qname())
            for state in self._model.states():
                res = hh.get_inf_and_tau(state, self._vm)
                if res is not None:
                    self._rl_states[state] = res
        else:
            self._model = model.clone()
            self._vm = None if vm is None else self._model.get(vm.qname())
        del model, vm

        # Defaults (openclsim.py:248-267)
        self._gx = self._gy = None
        if self._diffusion_enabled:
            self.set_conductance()
        self._gx_field = None
        self._gy_field = None
        self._g_arrays = None      # (key, gx, gy) arrays of the above
        self._connections = None
        self._paced_cells = None
        if self._diffusion_enabled:
            self.set_paced_cells()
        self._fields = OrderedDict()
        self._field_block = None    # fields interleaved per cell, pinned
        self._pinned = {}           # page-locked host buffers by use
        self.set_step_size()
        self._time = 0
        self._nstate = self._model.count_states()

        # State, kept as a float64 array (x fastest, then y; state minor)
        init = np.array(self._model.initial_values(True), dtype=float)
        self._state = np.tile(init, self._ntotal)
        self._default_state = self._state.copy()

        # Bindings (openclsim.py:281-287)
        self._global = ['time', 'pace']
        inputs = {'time': 'time', 'pace': 'pace'}
        if self._diffusion_enabled:
            inputs['diffusion_current'] = 'idiff'
        self._bound_variables = myokit._prepare_bindings(self._model, inputs)
        self._model.create_unique_names()

        # GPU options
        self._block = block
        self._min_blocks = min_blocks
        self._fp32_math = fp32_math
        self._stage_tiles = bool(stage_tiles)
        self._stage_lazy = None     # set by the autotuner
        # Between steps: 'barrier' (grid-wide) or 'neighbors' (each warp
        # waits for the warps whose cells it reads); None: tuned or barrier
        self._sync = None
        # Warps per warp tile (1, 2, 4, 8 or 16); None: tuned or 1
        self._split = None
        if accumulate not in (None, 'double', 'kahan'):
            raise ValueError(
                'The argument "accumulate" must be None, "double" or'
                ' "kahan".')
        if accumulate is not None and precision != myokit.SINGLE_PRECISION:
            raise ValueError(
                'Accumulation modes apply to single precision simulations.')
        self._accumulate = accumulate
        self._acc_names = None
        if accumulate_states is not None:
            self._acc_names = [
                v.qname() if isinstance(v, myokit.Variable) else str(v)
                for v in accumulate_states]
            for name in self._acc_names:
                if not self._model.get(name).is_state():
                    raise ValueError(
                        'Accumulated variables must be states: ' + name)
        self._steps_per_launch = int(steps_per_launch)
        self._blocks_per_sm = 0
        self._graphs = 1
        self._tune_sig = None
        self._tune_hit = None
        self._model_version = 0
        self._log_templates = {}
        self._kernels = {}
        self._device = int(device)
        self._backend = None
        self._last_stats = None
        self._last_kernel = None

        SimulationCUDA._index += 1

    # ------------------------------------------------------------------
    # Conductance and geometry
    # ------------------------------------------------------------------

    def calculate_conductance(self, r, sx, chi, dx):
        """
        Deprecated alias: ``calculate_conductance(r, sx, chi, dx)`` equals
        ``monodomain_conductance(1 / chi, r, sx, dx, 1)``.
        """
        import warnings
        warnings.warn('The method SimulationOpenCL.calculate_conductance() is'
                      ' deprecated. Please use monodomain_conductance()'
                      ' instead.')
        return self.monodomain_conductance(1 / chi, r, sx, dx, 1)

    def _require_diffusion(self):
        if not self._diffusion_enabled:
            raise RuntimeError(
                'This method is unavailable when diffusion is disabled.')

    def conductance(self):
        """
        Returns the cell-to-cell conductance: a float in 1d, ``(gx, gy)`` in
        2d, or ``None`` when conductance fields or connections are set.
        """
        self._require_diffusion()
        if (self._gx_field is not None) or (self._connections is not None):
            return None
        if len(self._dims) == 1:
            return self._gx
        return (self._gx, self._gy)

    def monodomain_conductance(self, chi, k, D, dx, A=1):
        """
        Conductance ``g = D * A * k / ((k + 1) * chi * dx^2)`` from monodomain
        parameters (zero-flux boundaries, regular grid, homogeneous D).
        """
        return D * A * k / ((k + 1) * chi * dx * dx)

    def set_conductance(self, gx=10, gy=5):
        """
        Sets homogeneous cell-to-cell conductances ``gx`` (and ``gy`` in 2d);
        clears conductance fields and connections.
        """
        self._require_diffusion()
        gx, gy = float(gx), float(gy)
        if gx < 0:
            raise ValueError('Invalid conductance gx=' + str(gx))
        if gy < 0:
            raise ValueError('Invalid conductance gy=' + str(gy))
        self._gx, self._gy = gx, gy
        self._gx_field = self._gy_field = None
        self._g_arrays = None
        self._connections = None

    def set_conductance_field(self, gx, gy=None):
        """
        Sets per-edge conductances: ``gx`` of length ``nx - 1`` in 1d, or
        ``gx`` with shape ``(ny, nx - 1)`` and ``gy`` with shape
        ``(ny - 1, nx)`` in 2d.
        """
        self._require_diffusion()
        gx = np.asarray(gx, dtype=float)
        if len(self._dims) == 1:
            s = self._nx - 1
            if gx.shape != (s, ):
                raise ValueError(
                    'The argument `gx` must have length ' + str(s) + '.')
            if gy is not None:
                raise ValueError(
                    'For 1-d simulations the argument `gy` must be None.')
        else:
            s = (self._ny, self._nx - 1)
            if gx.shape != s:
                raise ValueError(
                    'The argument `gx` must have dimensions ' + str(s) + '.')
            if gy is None:
                raise ValueError(
                    'The argument `gy` must be set for 2-d simulations.')
            gy = np.asarray(gy, dtype=float)
            s = (self._ny - 1, self._nx)
            if gy.shape != s:
                raise ValueError(
                    'The argument `gy` must have dimensions ' + str(s) + '.')
        if np.any(gx < 0):
            raise ValueError(
                'The argument `gx` can not contain negative values.')
        if (gy is not None) and np.any(gy < 0):
            raise ValueError(
                'The argument `gy` can not contain negative values.')
        self._g_arrays = None
        self._gx_field = list(gx.reshape((self._nx - 1) * self._ny))
        if gy is None:
            self._gy_field = None
        else:
            self._gy_field = list(gy.reshape(self._nx * (self._ny - 1)))
        self._connections = None

    def set_connections(self, connections):
        """
        Sets an arbitrary geometry as a list of ``(cell_1, cell_2, g)``
        tuples (1d mode only); clears other conductances.
        """
        self._require_diffusion()
        if len(self._dims) != 1:
            raise RuntimeError('Connections can only be specified in 1d mode.')
        if connections is None:
            raise ValueError(
                'Connection list cannot be None. To unset connections, call '
                ' set_conductance() with the new conductance value.')
        conns = []
        seen = set()
        for x in connections:
            try:
                i, j, c = x
            except Exception:
                raise ValueError(
                    'Connections must be a list of 3-tuples'
                    ' (cell_index_1, cell_index_2, conductance).')
            i, j = int(i), int(j)
            if i == j or i < 0 or j < 0 or i >= self._nx or j >= self._nx:
                raise ValueError(
                    'Invalid connection: (' + str(i) + ', ' + str(j) + ', '
                    + str(c) + ')')
            i, j = (i, j) if i < j else (j, i)
            if (i, j) in seen:
                raise ValueError(
                    'Duplicate connection: (' + str(i) + ', ' + str(j) + ', '
                    + str(c) + ')')
            seen.add((i, j))
            c = float(c)
            if c < 0:
                raise ValueError('Invalid conductance: ' + str(c))
            conns.append((i, j, c))
        self._connections = conns
        self._gx_field = self._gy_field = None
        self._g_arrays = None

    def neighbors(self, x, y=None):
        """
        Returns the neighbours of cell ``x`` (or ``(x, y)`` in 2d): integers
        in 1d and for connections, tuples in 2d.
        """
        self._require_diffusion()
        x = int(x or 0)
        if x < 0 or x >= self._dims[0]:
            raise IndexError('X-coordinate out of range: ' + str(x) + '.')
        if len(self._dims) == 2:
            if y is None:
                raise ValueError(
                    'No y-coordinate specified in 2-dimensional simulation.')
            y = int(y)
            if y < 0 or y >= self._dims[1]:
                raise IndexError('Y-coordinate out of range: ' + str(y) + '.')
        elif not (y is None or y == 0):
            raise ValueError(
                'Y-coordinate specified for 1-dimensional simulation.')
        if self._connections is not None:
            out = []
            for i, j, c in self._connections:
                if i == x:
                    out.append(j)
                elif j == x:
                    out.append(i)
            return out
        out = []
        if x > 0:
            out.append(x - 1)
        if x + 1 < self._dims[0]:
            out.append(x + 1)
        if len(self._dims) == 2:
            out = [(i, y) for i in out]
            if y > 0:
                out.append((x, y - 1))
            if y + 1 < self._dims[1]:
                out.append((x, y + 1))
        return out

    def neighbours(self, x, y=None):
        """Deprecated alias of :meth:`neighbors`."""
        import warnings
        warnings.warn('The method SimulationOpenCL.neighbours() is deprecated.'
                      ' Please use neighbors() instead.')
        return self.neighbors(x, y)

    def is2d(self):
        """Deprecated alias of :meth:`is_2d()`."""
        import warnings
        warnings.warn('The method SimulationOpenCL.is2d() is deprecated.'
                      ' Please use is_2d() instead.')
        return self.is_2d()

    def is_2d(self):
        """True for a 2d simulation."""
        return len(self._dims) == 2

    def shape(self):
        """``(ny, nx)`` in 2d, ``nx`` in 1d."""
        if len(self._dims) == 2:
            return (self._ny, self._nx)
        return self._nx

    # ------------------------------------------------------------------
    # Pacing
    # ------------------------------------------------------------------

    def is_paced(self, x, y=None):
        """True if cell ``x`` (or ``(x, y)``) receives the pacing signal."""
        self._require_diffusion()
        x = int(x)
        if x < 0 or x >= self._dims[0]:
            raise IndexError('X-coordinate out of range: ' + str(x) + '.')
        if len(self._dims) == 2:
            if y is None:
                raise ValueError(
                    'No y-coordinate specified in 2-dimensional simulation.')
            y = int(y)
            if y < 0 or y >= self._dims[1]:
                raise IndexError('Y-coordinate out of range: ' + str(y) + '.')
        elif y is None:
            y = 0
        elif y != 0:
            raise ValueError(
                'Y-coordinate specified for 1-dimensional simulation.')
        if type(self._paced_cells) == tuple:
            nx, ny, xmin, ymin = self._paced_cells
            return (x >= xmin and x < xmin + nx and
                    y >= ymin and y < ymin + ny)
        return (x + y * self._dims[0]) in self._paced_cells

    def set_paced_cells(self, nx=5, ny=5, x=0, y=0):
        """
        Paces a rectangle of ``nx`` by ``ny`` cells at offset ``(x, y)``.
        Negative sizes extend left/down from the offset; negative offsets
        count from the right/top (``openclsim.py:1534-1593``).
        """
        self._require_diffusion()
        nx = int(nx)
        x = int(x)
        if nx < 0:
            nx = -nx
            x -= nx
        if x < 0:
            x += self._nx
        if len(self._dims) == 1:
            ny = 1
            y = 0
        else:
            ny = int(ny)
            if ny < 0:
                ny = -ny
                y -= ny
            if y < 0:
                y += self._ny
        self._paced_cells = (nx, ny, x, y)

    def set_paced_cell_list(self, cells):
        """Paces the listed cells: integers in 1d, ``(x, y)`` in 2d."""
        self._require_diffusion()
        paced = []
        if len(self._dims) == 1:
            for cell in cells:
                cell = int(cell)
                if cell < 0 or cell >= self._nx:
                    raise IndexError(
                        'Cell index out of range: ' + str(cell) + '.')
                paced.append(cell)
        else:
            for i, j in cells:
                i, j = int(i), int(j)
                if i < 0 or j < 0 or i >= self._nx or j >= self._ny:
                    raise IndexError(
                        'Cell index out of range: (' + str(i) + ', ' + str(j)
                        + ').')
                paced.append(i + j * self._nx)
        self._paced_cells = paced

    def set_protocol(self, protocol=None):
        """Sets (a clone of) the pacing protocol, or ``None``."""
        self._protocol = None if protocol is None else protocol.clone()

    # ------------------------------------------------------------------
    # Constants and fields
    # ------------------------------------------------------------------

    def set_constant(self, var, value):
        """Changes a literal constant of the simulation's model."""
        value = float(value)
        if isinstance(var, myokit.Variable):
            var = var.qname()
        var = self._model.get(var)
        if not var.is_literal():
            raise ValueError(
                'The given variable <' + var.qname() + '> is not a literal.')
        self._model.set_value(var.qname(), value)
        self._model_version += 1

    def set_field(self, var, values):
        """
        Replaces a constant with a per-cell scalar field of shape ``(ny, nx)``
        (or length ``nx`` in 1d).
        """
        if isinstance(var, myokit.Variable):
            var = var.qname()
        var = self._model.get(var)
        if var.is_bound():
            raise ValueError('Bound values cannot be replaced by fields.')
        if not var.is_constant():
            raise ValueError('Only constants can be used for fields.')
        values = np.asarray(values, dtype=float)
        if len(self._dims) == 1:
            if values.shape != (self._nx, ):
                raise ValueError(
                    'The argument `values` must have length ' + str(self._nx)
                    + '.')
        else:
            shape = (self._ny, self._nx)
            if values.shape != shape:
                raise ValueError(
                    'The argument `values` must have dimensions ' + str(shape)
                    + '.')
        self._fields[var] = values.reshape(self._nx * self._ny).copy()
        self._field_block = None

    def remove_field(self, var):
        """Removes the field set for ``var``."""
        if isinstance(var, myokit.Variable):
            var = var.qname()
        var = self._model.get(var)
        del self._fields[var]
        self._field_block = None

    # ------------------------------------------------------------------
    # State and time
    # ------------------------------------------------------------------

    def _cell_offset(self, x, y, yname):
        x = int(x or 0)
        if x < 0 or x >= self._nx:
            raise IndexError('Given x-index out of range.')
        y = int(y or 0)
        if len(self._dims) == 2:
            if y < 0 or y >= self._ny:
                raise IndexError('Given y-index out of range.')
            x += y * self._nx
        elif y != 0:
            raise ValueError(
                yname + ' specified for 1-dimensional simulation.')
        return x * self._nstate

    def state(self, x=None, y=None):
        """
        The current state as a list of ``n_states * n_cells`` floats (x
        fastest), or one cell's state when ``x`` (and ``y``) are given.
        """
        if x is None:
            return self._state.tolist()
        o = self._cell_offset(x, y, 'Y-coordinate')
        return self._state[o:o + self._nstate].tolist()

    def state_array(self):
        """
        The current state as a float64 numpy array (a copy), laid out as
        :meth:`state`; avoids building a Python list for large grids.
        """
        return np.array(self._state, dtype=float)

    def default_state(self, x=None, y=None):
        """The default state, indexed as :meth:`state`."""
        if x is None:
            return self._default_state.tolist()
        o = self._cell_offset(x, y, 'Y-coordinate')
        return self._default_state[o:o + self._nstate].tolist()

    def _set_state(self, state, x, y, update):
        n = len(state)
        if n == self._nstate * self._ntotal:
            if x is not None:
                raise ValueError(
                    'A state for all cells was passed in, but argument x'
                    ' was not None.')
            if y is not None:
                raise ValueError(
                    'A state for all cells was passed in, but argument y'
                    ' was not None.')
            return np.array(state, dtype=float)
        elif n != self._nstate:
            raise ValueError(
                'Given state must have the same size as a single'
                ' cell state or a full simulation state')
        if x is None:
            return np.tile(np.asarray(state, dtype=float), self._ntotal)
        o = self._cell_offset(x, y, 'Y-index given')
        update = np.array(update, dtype=float)
        update[o:o + self._nstate] = np.asarray(state, dtype=float)
        return update

    def set_state(self, state, x=None, y=None):
        """
        Sets the state of all cells (one cell state or a full state) or of
        cell ``(x, y)``.
        """
        self._state = self._set_state(state, x, y, self._state)

    def set_default_state(self, state, x=None, y=None):
        """Sets the default state, as :meth:`set_state`."""
        self._default_state = self._set_state(
            state, x, y, self._default_state)

    def reset(self):
        """Sets the time to 0 and the state to the default state."""
        self._time = 0
        self._state = self._default_state.copy()

    def set_step_size(self, step_size=0.005):
        """Sets the forward-Euler step size."""
        step_size = float(step_size)
        if step_size <= 0:
            raise ValueError('Step size must be greater than zero.')
        self._step_size = step_size

    def step_size(self):
        """The current step size."""
        return self._step_size

    def set_time(self, time=0):
        """Sets the simulation time."""
        self._time = float(time)

    def time(self):
        """The current simulation time."""
        return self._time

    # ------------------------------------------------------------------
    # Running
    # ------------------------------------------------------------------

    def pre(self, duration, report_nan=True, progress=None,
            msg='Pre-pacing SimulationOpenCL'):
        """
        Runs without logging and without advancing the time; the final state
        becomes the new default state.
        """
        self._run(duration, myokit.LOG_NONE, 1, report_nan, progress, msg)
        self._default_state = self._state.copy()

    def run(self, duration, log=None, log_interval=1.0, report_nan=True,
            progress=None, msg='Running SimulationOpenCL'):
        """
        Runs for ``duration`` time units and returns a :class:`myokit.DataLog`
        with keys ``"x.comp.var"`` (1d) or ``"x.y.comp.var"`` (2d) for
        per-cell variables and plain qnames for time and pace. A log entry is
        made every time at least ``log_interval`` has passed; the final time
        point is not logged.
        """
        r = self._run(duration, log, log_interval, report_nan, progress, msg)
        self._time += duration
        return r

    def _diffusion_mode(self):
        if not self._diffusion_enabled:
            return _exp.DIFF_NONE
        if self._connections is not None:
            return _exp.DIFF_CONN
        if self._gx_field is not None:
            return _exp.DIFF_HETERO
        return _exp.DIFF_GRID

    def _tuned_choice(self):
        """A cached autotuner result for this configuration, or None."""
        from . import autotune
        key = (self._model_version, self._precision, self._accumulate,
               self._fp32_math, self._native_math, self._diffusion_mode(),
               tuple(v.qname() for v in self._fields))
        if self._tune_sig != key:
            self._tune_sig = key
            self._tune_hit = autotune.lookup(self)
        return self._tune_hit

    def _sync_mode(self):
        """How steps are separated: 'barrier' or 'neighbors'."""
        if self._sync is not None:
            return self._sync
        if self._block is None:
            hit = self._tuned_choice()
            if hit is not None:
                return hit.get('sync', 'barrier')
        return 'barrier'

    def _split_mode(self):
        """Warps that share each warp tile's work (1, 2, 4, 8 or 16)."""
        if self._split is not None:
            return int(self._split)
        if self._block is None:
            hit = self._tuned_choice()
            if hit is not None:
                return int(hit.get('split', 1))
        return 1

    def _lazy_staging(self):
        """Staged tiles prefetched into registers (0), or read where used
        from one (1) or two (2) shared-memory buffers per warp."""
        if self._stage_lazy is not None:
            return int(self._stage_lazy)
        if self._block is None:
            hit = self._tuned_choice()
            if hit is not None:
                return int(hit.get('stage_lazy', 0))
        return 0

    def _block_shape(self, two_d):
        """CTA shape (threads, 1); threads is a multiple of the warp size."""
        b = self._block
        if b is None:
            hit = self._tuned_choice()
            if hit is not None:
                b = tuple(hit['block'])
            elif self._precision == myokit.DOUBLE_PRECISION:
                b = 128
            else:
                b = 256
        if not isinstance(b, int):
            b = int(np.prod([int(x) for x in b]))
        b = max(32, (int(b) + 31) // 32 * 32)
        return (min(b, 1024), 1)

    def _default_min_blocks(self, block):
        """Minimum resident CTAs per SM asked of the compiler, which caps
        the registers per thread at 64K / (threads * min_blocks)."""
        if self._min_blocks is not None:
            return int(self._min_blocks)
        if self._block is None:
            hit = self._tuned_choice()
            if hit is not None:
                return int(hit['min_blocks'])
        if self._precision == myokit.DOUBLE_PRECISION:
            return 1
        # 128 registers per thread: 64K registers / 512 threads
        return max(1, 512 // (block[0] * block[1]))

    def _launch_steps(self):
        """Steps per launch: explicit, cached by the autotuner, or 0."""
        if self._steps_per_launch:
            return self._steps_per_launch
        if self._block is None:
            hit = self._tuned_choice()
            if hit is not None:
                return int(hit.get('steps_per_launch', 0))
        return 0

    def autotune(self, duration=None, verbose=False):
        """
        Times candidate launch shapes on this simulation (state and time
        are restored afterwards), keeps the fastest and caches it for
        simulations with the same configuration. Returns the choice.
        """
        from . import autotune
        best, results = autotune.autotune(self, duration, verbose=verbose)
        self._tune_sig = None
        return best

    def accumulated_states(self):
        """The states accumulated in FP64 or with a compensated update."""
        if self._accumulate is None:
            return []
        if self._acc_names is not None:
            return [self._model.get(n) for n in self._acc_names]
        conc = myokit.parse_unit('mM').exponents()
        out = []
        for st in self._model.states():
            u = st.unit()
            if st is self._vm:
                out.append(st)
            elif u is not None and u.exponents() == conc:
                out.append(st)
            elif st not in self._rl_states and abs(st.initial_value(True)) >= 1:
                out.append(st)
        return out

    def _kernel(self, inter_log):
        """The generated kernel for the current configuration (cached)."""
        mode = self._diffusion_mode()
        two_d = len(self._dims) == 2 and mode in (
            _exp.DIFF_GRID, _exp.DIFF_HETERO)
        block = self._block_shape(two_d)
        minb = self._default_min_blocks(block)
        acc = self.accumulated_states()
        # Tile staging with TMA for grids of at least 256 cells; rows that
        # are not a multiple of 4 cells need the padded copy width
        stage = self._stage_tiles and self._ntotal >= 256
        row_pad = two_d and self._nx % 4 != 0
        lazy = stage and self._lazy_staging()
        key = (
            self._model_version, self._precision, self._native_math, mode,
            two_d, block, minb, self._fp32_math, self._accumulate,
            stage, row_pad, lazy, self._sync_mode(), self._split_mode(),
            tuple(v.qname() for v in acc),
            tuple(v.qname() for v in self._fields.keys()),
            tuple(v.qname() for v in inter_log))
        k = self._kernels.get(key)
        if k is None:
            k = _exp.TissueKernel(
                self._model, self._precision, self._native_math,
                self._bound_variables, inter_log, mode, two_d,
                list(self._fields.keys()), self._rl_states, block,
                min_blocks=minb, math=self._fp32_math,
                accumulate=self._accumulate, accumulate_states=acc,
                stage=stage, row_pad=row_pad, stage_lazy=lazy,
                sync=self._sync_mode(), split=self._split_mode())
            if len(self._kernels) > 16:
                self._kernels.clear()
            self._kernels[key] = k
        return k

    def _get_backend(self, kernel):
        """A host-library handle for this kernel, reused between runs."""
        cfg = _lib.MkgConfig()
        cfg.nx = self._nx
        cfg.ny = self._ny
        cfg.real_bytes = 4 if self._precision == myokit.SINGLE_PRECISION \
            else 8
        cfg.n_state = self._nstate
        cfg.n_inter = len(kernel.inter_log)
        cfg.n_field = len(kernel.fields)
        cfg.i_vm = kernel.i_vm
        cfg.diffusion = kernel.diffusion
        cfg.block_x, cfg.block_y = kernel.block
        cfg.device = self._device
        cfg.two_d = 1 if kernel.two_d else 0
        cfg.hi_mode = {None: 0, 'double': 1, 'kahan': 2}[kernel.accumulate] \
            if kernel.hi_states else 0
        cfg.n_hi = len(kernel.hi_states)
        cfg.stage = kernel.stage_buffers if kernel.layout else 0
        cfg.v_double = 1 if kernel.v_double else 0
        cfg.split = kernel.split
        key = (kernel.key(), bytes(cfg))
        if self._backend is not None and self._backend[0] == key:
            return self._backend[1]
        if self._backend is not None:
            self._backend[1].close()
            self._backend = None
        be = _Backend(kernel, cfg)
        if cfg.n_hi:
            hs = np.ascontiguousarray(kernel.hi_states, dtype=np.int32)
            be.check(be.lib.mkg_set_hi_states(be.h, _lib.i32ptr(hs), len(hs)))
        self._backend = (key, be)
        return be

    def _log_columns(self, log, kernel):
        """
        Maps every log key to a column source: ``('time',)``, ``('pace',)``
        or a per-cell ``(item, cell)`` pair (openclsim.c:916-1001).
        """
        tvar = self._model.binding('time')
        pvar = self._model.binding('pace')
        tname = None if tvar is None else tvar.qname()
        pname = None if pvar is None else pvar.qname()
        ivar = self._model.binding('diffusion_current') \
            if self._diffusion_enabled else None
        inter_index = {v.qname(): k for k, v in enumerate(kernel.inter_log)}
        state_index = {v.qname(): v.index() for v in self._model.states()}
        ndims = len(self._dims)
        sources = []
        for key in log.keys():
            if key == tname:
                sources.append(('time',))
                continue
            if key == pname:
                sources.append(('pace',))
                continue
            pre, name = myokit.split_key(key)
            parts = pre.split('.')[:-1] if pre else []
            ok = len(parts) == ndims
            cell = -1
            if ok:
                try:
                    idx = [int(p) for p in parts]
                except ValueError:
                    ok = False
            if ok:
                if idx[0] < 0 or idx[0] >= self._nx:
                    ok = False
                elif ndims == 2 and (idx[1] < 0 or idx[1] >= self._ny):
                    ok = False
                else:
                    cell = idx[0] + (idx[1] * self._nx if ndims == 2 else 0)
            item = None
            if ok:
                if name in state_index:
                    item = state_index[name]
                elif ivar is not None and name == ivar.qname():
                    item = self._nstate
                elif name in inter_index:
                    item = self._nstate + 1 + inter_index[name]
            if item is None:
                raise Exception(
                    'Unknown variables found in logging dictionary.')
            sources.append((item, cell))
        return sources

    def _prepare_log(self, log, global_vars):
        """
        ``myokit.prepare_log`` with the simulation's arguments
        (openclsim.py:1033-1042). For a flag or a list of names, the empty
        log it builds is remembered as a template (per model version), so a
        repeated run does not re-validate every key against every cell.
        """
        key = None
        if isinstance(log, int) and not isinstance(log, bool):
            key = ('flag', log)
        elif isinstance(log, (list, tuple)) and all(
                isinstance(x, str) for x in log):
            key = ('names', tuple(log))
        elif log is None:
            key = ('none',)
        if key is not None:
            key = key + (self._model_version, tuple(global_vars))
            tpl = self._log_templates.get(key)
            if tpl is not None:
                out = myokit.DataLog(tpl)
                tc = 'd' if self._precision == myokit.DOUBLE_PRECISION \
                    else 'f'
                for k in tpl.keys():
                    OrderedDict.__setitem__(out, k, array.array(tc))
                return out
        out = myokit.prepare_log(
            log,
            self._model,
            dims=self._dims,
            global_vars=global_vars,
            if_empty=myokit.LOG_STATE + myokit.LOG_BOUND,
            allowed_classes=myokit.LOG_STATE + myokit.LOG_INTER
            + myokit.LOG_BOUND,
            precision=self._precision)
        if key is not None:
            if len(self._log_templates) > 32:
                self._log_templates.clear()
            self._log_templates[key] = myokit.DataLog(out)
        return out

    def _run(self, duration, log, log_interval, report_nan, progress, msg):
        # Times (openclsim.py:1018-1024)
        if duration < 0:
            raise ValueError('Simulation time can\'t be negative.')
        tmin = self._time
        tmax = tmin + duration

        g = []
        for label in self._global:
            v = self._model.binding(label)
            if v is not None:
                g.append(v.qname())
        log = self._prepare_log(log, g)

        # Logged intermediary variables (openclsim.py:1044-1053)
        inter_log = []
        checked = set()
        for key in log.keys():
            name = myokit.split_key(key)[1]
            if name in checked:
                continue
            checked.add(name)
            var = self._model.get(name)
            if var.is_intermediary() and not var.is_bound():
                inter_log.append(var)

        log_interval = 1e-9 if log_interval is None else float(log_interval)
        if log_interval <= 0:
            log_interval = 1e-9

        if progress is None:
            progress = myokit._simulation_progress
        if progress:
            if not isinstance(progress, myokit.ProgressReporter):
                raise ValueError(
                    'The argument "progress" must be either a subclass of'
                    ' myokit.ProgressReporter or None.')

        arithmetic_error = False
        if duration > 0:
            kernel = self._kernel(inter_log)
            self._last_kernel = kernel
            sources = self._log_columns(log, kernel)
            be = self._get_backend(kernel)
            arithmetic_error = self._execute(
                be, kernel, log, sources, tmin, tmax, log_interval, progress,
                msg, duration)

        if report_nan and (arithmetic_error or log.has_nan()):
            self._report_nan(log)
        return log

    def _host_buffer(self, use, n):
        """
        A page-locked float64 host array of ``n`` values, one per ``use``
        ('state', 'fields'), reused between runs: copies from and to it are
        DMA transfers without a pageable staging copy. ``self._state`` is
        the 'state' buffer after a run, so code that keeps the state across
        a run keeps a copy.
        """
        buf = self._pinned.get(use)
        if buf is None or buf[1].size != n:
            import torch
            t = torch.empty(n, dtype=torch.float64, pin_memory=True)
            buf = (t, t.numpy())
            self._pinned[use] = buf
        return buf[1]

    def _upload(self, be):
        """Copies state, fields, conductances, pacing and protocol."""
        lib, h = be.lib, be.h
        st = np.ascontiguousarray(self._state, dtype=np.float64)
        be.check(lib.mkg_set_state(h, _lib.dptr(st), st.size))
        if self._fields:
            if self._field_block is None:
                fd = self._host_buffer('fields',
                                       len(self._fields) * self._ntotal)
                fd.reshape(self._ntotal, -1)[:] = np.stack(
                    [np.asarray(v, dtype=float)
                     for v in self._fields.values()], axis=1)
                self._field_block = fd
            fd = self._field_block
            be.check(lib.mkg_set_fields(h, _lib.dptr(fd), fd.size))
        mode = self._diffusion_mode()
        if mode == _exp.DIFF_GRID:
            be.check(lib.mkg_set_conductance(
                h, self._gx or 0.0, self._gy or 0.0))
        elif mode == _exp.DIFF_HETERO:
            # Converted once per set_conductance_field (the fields are
            # lists, as the reference keeps them)
            key = (id(self._gx_field), id(self._gy_field))
            if self._g_arrays is None or self._g_arrays[0] != key:
                self._g_arrays = (key, np.ascontiguousarray(
                    self._gx_field, dtype=float), np.ascontiguousarray(
                    self._gy_field if self._gy_field is not None else [],
                    dtype=float))
            gx, gy = self._g_arrays[1:]
            be.check(lib.mkg_set_conductance_field(
                h, _lib.dptr(gx), gx.size, _lib.dptr(gy), gy.size))
        elif mode == _exp.DIFF_CONN:
            c = np.array(self._connections, dtype=float).reshape(-1, 3)
            c1 = np.ascontiguousarray(c[:, 0].astype(np.int64))
            c2 = np.ascontiguousarray(c[:, 1].astype(np.int64))
            gg = np.ascontiguousarray(c[:, 2])
            be.check(lib.mkg_set_connections(
                h, _lib.i64ptr(c1), _lib.i64ptr(c2), _lib.dptr(gg), len(gg)))
        if not self._diffusion_enabled:
            be.check(lib.mkg_set_pacing_mode(h, _lib.PACE_ALL))
        elif type(self._paced_cells) == tuple:
            nx, ny, x, y = self._paced_cells
            be.check(lib.mkg_set_paced_rect(h, nx, ny, x, y))
        elif self._paced_cells:
            cells = np.ascontiguousarray(self._paced_cells, dtype=np.int64)
            be.check(lib.mkg_set_paced_list(h, _lib.i64ptr(cells), len(cells)))
        else:
            be.check(lib.mkg_set_pacing_mode(h, _lib.PACE_NONE))
        ev = []
        if self._protocol is not None:
            for e in self._protocol.events():
                ev.append([e.level(), e.start(), e.duration(), e.period(),
                           e.multiplier()])
        ev = np.ascontiguousarray(np.array(ev, dtype=float).reshape(-1, 5))
        be.check(lib.mkg_set_protocol(h, _lib.dptr(ev), len(ev)))

    def _chunk_steps(self):
        """Steps per host round trip: enough to amortise the launch."""
        per = 2e9 if self._precision == myokit.SINGLE_PRECISION else 2e8
        return int(max(100, min(100000, per / self._ntotal)))

    def _execute(self, be, kernel, log, sources, tmin, tmax, log_interval,
                 progress, msg, duration):
        lib, h = be.lib, be.h
        n0 = _lib.ctypes.c_int64()
        lib.mkg_launch_count(h, _lib.ctypes.byref(n0))
        self._upload(be)
        cols = [(s[0], s[1]) for s in sources if len(s) == 2]
        items = np.ascontiguousarray([c[0] for c in cols], dtype=np.int32)
        cells = np.ascontiguousarray([c[1] for c in cols], dtype=np.int64)
        logging_states = any(c[0] < self._nstate for c in cols)
        be.log_sig = None
        be.check(lib.mkg_set_log(
            h, _lib.i32ptr(items), _lib.i64ptr(cells), len(cols),
            1 if logging_states else 0))
        be.check(lib.mkg_set_tuning(h, self._launch_steps(),
                                    self._blocks_per_sm, self._graphs))
        be.check(lib.mkg_run_begin(h, tmin, tmax, self._step_size,
                                   log_interval))

        keys = list(log.keys())
        col_of_key = []
        j = 0
        for s in sources:
            if len(s) == 2:
                col_of_key.append(j)
                j += 1
            else:
                col_of_key.append(s[0])
        ncol = len(cols)

        chunks_t, chunks_p, chunks_v = [], [], []
        t = tmin
        status = _lib.MKG_OK
        max_steps = self._chunk_steps()
        ms_total = 0.0
        launches = 0
        cell_steps = 0
        t_out = _lib.ctypes.c_double()
        rows = _lib.ctypes.c_int64()
        kms = _lib.ctypes.c_double()
        nl = _lib.ctypes.c_int64()
        ncs = _lib.ctypes.c_int64()
        rdur = 1.0 / duration if duration != 0 else 1

        def one_chunk():
            code = be.check(lib.mkg_run_chunk(
                h, max_steps, _lib.ctypes.byref(t_out),
                _lib.ctypes.byref(rows)))
            n = rows.value
            if n > 0:
                tt = np.empty(n)
                pp = np.empty(n)
                vv = np.empty((n, ncol))
                be.check(lib.mkg_read_log(
                    h, _lib.dptr(tt), _lib.dptr(pp),
                    _lib.dptr(vv) if ncol else None, n))
                chunks_t.append(tt)
                chunks_p.append(pp)
                chunks_v.append(vv)
            lib.mkg_last_stats(h, _lib.ctypes.byref(kms), _lib.ctypes.byref(nl),
                               _lib.ctypes.byref(ncs))
            return code

        if progress:
            with progress.job(msg):
                while status == _lib.MKG_OK:
                    status = one_chunk()
                    ms_total += kms.value
                    launches += nl.value
                    cell_steps += ncs.value
                    t = t_out.value
                    if not progress.update(min((t - tmin) * rdur, 1)):
                        raise myokit.SimulationCancelledError()
        else:
            while status == _lib.MKG_OK:
                status = one_chunk()
                ms_total += kms.value
                launches += nl.value
                cell_steps += ncs.value

        # Final state (openclsim.c:1185-1190); on an exception above the
        # state is left unchanged, as in the reference.
        st = self._host_buffer('state', self._nstate * self._ntotal)
        be.check(lib.mkg_get_state(h, _lib.dptr(st), st.size))
        self._state = st

        n1 = _lib.ctypes.c_int64()
        lib.mkg_launch_count(h, _lib.ctypes.byref(n1))
        self._last_stats = {
            'kernel_ms': ms_total, 'launches': launches,
            'cell_steps': cell_steps, 'all_launches': n1.value - n0.value,
        }

        # Append to the log
        if chunks_t:
            tt = np.concatenate(chunks_t)
            pp = np.concatenate(chunks_p)
            vv = np.concatenate(chunks_v) if ncol else None
            for key, src, c in zip(keys, sources, col_of_key):
                if src[0] == 'time':
                    data = tt
                elif src[0] == 'pace':
                    data = pp
                else:
                    data = vv[:, c]
                _extend(log[key], data)
        return status == _lib.MKG_HALT_NAN

    def run_frames(self, duration, interval=5.0, variable=None):
        """
        Runs for ``duration`` time units and records ``variable`` (a state;
        by default the membrane potential) of every cell every ``interval``
        time units into a CUDA tensor that never leaves the device. Returns
        ``(times, frames)``: a numpy array of the frame times and a torch
        tensor shaped ``(n_frames, ny, nx)`` (``(n_frames, nx)`` in 1d) in
        the simulation precision. Time and state advance as in :meth:`run`;
        the NaN check of logged runs does not apply.
        """
        import torch
        if duration < 0:
            raise ValueError('Simulation time can\'t be negative.')
        interval = float(interval)
        if interval <= 0:
            raise ValueError('The frame interval must be positive.')
        var = self._vm if variable is None else self._model.get(
            variable.qname() if isinstance(variable, myokit.Variable)
            else variable)
        if var is None or not var.is_state():
            raise ValueError('Frames record a state variable.')
        cap = int(np.ceil(duration / interval)) + 1
        dtype = torch.float32 if self._precision == myokit.SINGLE_PRECISION \
            else torch.float64
        frames = torch.empty((cap, self._ntotal), dtype=dtype,
                             device='cuda:%d' % self._device)
        kernel = self._kernel([])
        self._last_kernel = kernel
        be = self._get_backend(kernel)
        lib, h = be.lib, be.h
        tmin = self._time
        times = []
        if duration > 0:
            n0 = _lib.ctypes.c_int64()
            lib.mkg_launch_count(h, _lib.ctypes.byref(n0))
            self._upload(be)
            sig = ('frames', var.index())
            if be.log_sig != sig:
                items = np.full(self._ntotal, var.index(), dtype=np.int32)
                cells = np.arange(self._ntotal, dtype=np.int64)
                be.log_sig = None
                be.check(lib.mkg_set_log(h, _lib.i32ptr(items),
                                         _lib.i64ptr(cells), len(cells), 0))
                be.log_sig = sig
            be.check(lib.mkg_set_tuning(h, self._launch_steps(),
                                        self._blocks_per_sm, self._graphs))
            torch.cuda.synchronize(self._device)
            be.check(lib.mkg_set_frame_buffer(
                h, _lib.ctypes.c_void_p(frames.data_ptr()), cap))
            try:
                be.check(lib.mkg_run_begin(h, tmin, tmin + duration,
                                           self._step_size, interval))
                t_out = _lib.ctypes.c_double()
                rows = _lib.ctypes.c_int64()
                status = _lib.MKG_OK
                ms = 0.0
                cs = 0
                nlaunch = 0
                while status == _lib.MKG_OK:
                    status = be.check(lib.mkg_run_chunk(
                        h, self._chunk_steps(), _lib.ctypes.byref(t_out),
                        _lib.ctypes.byref(rows)))
                    if rows.value:
                        tt = np.empty(rows.value)
                        be.check(lib.mkg_read_log(h, _lib.dptr(tt), None,
                                                  None, rows.value))
                        times.append(tt)
                    kms = _lib.ctypes.c_double()
                    nl = _lib.ctypes.c_int64()
                    ncs = _lib.ctypes.c_int64()
                    lib.mkg_last_stats(h, _lib.ctypes.byref(kms),
                                       _lib.ctypes.byref(nl),
                                       _lib.ctypes.byref(ncs))
                    ms += kms.value
                    cs += ncs.value
                    nlaunch += nl.value
            finally:
                lib.mkg_set_frame_buffer(h, None, 0)
            st = self._host_buffer('state', self._nstate * self._ntotal)
            be.check(lib.mkg_get_state(h, _lib.dptr(st), st.size))
            self._state = st
            n1 = _lib.ctypes.c_int64()
            lib.mkg_launch_count(h, _lib.ctypes.byref(n1))
            self._last_stats = {'kernel_ms': ms, 'cell_steps': cs,
                                'launches': nlaunch,
                                'all_launches': n1.value - n0.value}
        self._time += duration
        t = np.concatenate(times) if times else np.zeros(0)
        shape = (len(t), self._ny, self._nx) if len(self._dims) == 2 else (
            len(t), self._nx)
        return t, frames[:len(t)].reshape(shape)

    def cuda_stream(self):
        """
        The CUDA stream (an integer handle) the last run was queued on, or
        ``None`` before the first run.
        """
        if self._backend is None:
            return None
        ptr = _lib.ctypes.c_void_p()
        be = self._backend[1]
        be.check(be.lib.mkg_stream(be.h, _lib.ctypes.byref(ptr)))
        return ptr.value

    def last_run_stats(self):
        """
        Device statistics of the last run: kernel milliseconds, kernel
        launches and cell-steps computed.
        """
        return dict(self._last_stats) if self._last_stats else None

    # ------------------------------------------------------------------
    # NaN diagnosis (openclsim.py:395-702, 1152-1281)
    # ------------------------------------------------------------------

    def find_nan(self, log, watch_var=None, safe_range=None,
                 return_log=False):
        """
        Locates the first ``NaN``/``inf`` (or, with ``watch_var`` and
        ``safe_range``, the first out-of-range value of a state) in a log of
        this simulation by re-running with successively finer log intervals.

        Returns ``(time, icell, variable, value, states, bounds)`` and, with
        ``return_log=True``, a log of all variables around the error.
        """
        from ._nan import find_nan
        return find_nan(self, log, watch_var, safe_range, return_log)

    def _report_nan(self, log):
        from ._nan import report_nan
        report_nan(self, log)


def _extend(target, values):
    """Appends numpy values to a log list or array."""
    if isinstance(target, array.array):
        dt = np.float32 if target.typecode == 'f' else np.float64
        target.frombytes(np.ascontiguousarray(values, dtype=dt).tobytes())
    else:
        target.extend(np.asarray(values, dtype=float).tolist())
