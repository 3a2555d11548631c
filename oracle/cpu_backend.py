"""
CPU stand-in for the compiled module of ``myokit.SimulationOpenCL``.

TEST INFRASTRUCTURE (the oracle). Only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py`` use it; the product never does.

``SimulationOpenCL`` renders its OpenCL kernel (``myokit/_sim/openclsim.cl``)
and hands it to a generated CPython module with the methods ``sim_init``,
``sim_step`` and ``sim_clean`` (``myokit/_sim/openclsim.c:1216-1221``).
:class:`CpuBackend` implements those three methods with the same arguments
and effects, but compiles the rendered kernel as C (with
``oracle/oracle_shim.h``) and runs it with ``oracle/cl_runner.c``, a C
restatement of the reference step loop. The reference Python layer
(argument checks, kernel rendering, logging, ``find_nan``) runs unmodified.

Build products go to ``oracle/_ref/`` (one shared library per kernel text).
"""
import ctypes
import hashlib
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, '_ref')
_LOCK = threading.Lock()
_LOADED = {}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def _threads():
    n = os.environ.get('MKG_ORACLE_THREADS')
    if n:
        return max(1, int(n))
    return 1


def build_runner(kernel_source, diff_mode):
    """Compiles ``cl_runner.c`` around a rendered kernel; returns a CDLL."""
    h = hashlib.sha256()
    h.update(kernel_source.encode())
    h.update(str(diff_mode).encode())
    for name in ('cl_runner.c', 'oracle_shim.h'):
        with open(os.path.join(_HERE, name), 'rb') as f:
            h.update(f.read())
    key = h.hexdigest()[:24]
    with _LOCK:
        if key in _LOADED:
            return _LOADED[key]
        os.makedirs(REF_DIR, exist_ok=True)
        cl = os.path.join(REF_DIR, key + '.cl')
        so = os.path.join(REF_DIR, key + '.so')
        if not os.path.exists(so):
            with open(cl, 'w') as f:
                f.write(kernel_source)
            tmp = so + '.%d' % os.getpid()
            cmd = [
                'gcc', '-O2', '-std=gnu99', '-fPIC', '-shared', '-fopenmp',
                '-ffp-contract=off', '-w',
                '-I' + _HERE,
                '-DORC_KERNEL="' + cl + '"', '-DORC_DIFF=%d' % diff_mode,
                os.path.join(_HERE, 'cl_runner.c'), '-o', tmp, '-lm',
            ]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError('Oracle build failed:\n' + r.stderr)
            os.replace(tmp, so)
        lib = ctypes.CDLL(so)
        lib.orc_init.restype = ctypes.c_int
        lib.orc_init.argtypes = [
            ctypes.c_long, ctypes.c_long, ctypes.c_double, ctypes.c_double,
            _dp, ctypes.c_long, _dp, ctypes.c_long,
            _lp, _lp, _dp, ctypes.c_long,
            ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, _dp, _dp, ctypes.c_long, _dp, ctypes.c_long,
            _ip, _lp, ctypes.c_long, ctypes.c_int]
        lib.orc_step.restype = ctypes.c_int
        lib.orc_step.argtypes = [ctypes.c_long, _dp]
        lib.orc_rows.restype = ctypes.c_long
        lib.orc_take_rows.argtypes = [_dp]
        lib.orc_get_state.argtypes = [_dp]
        for f in ('orc_n_state', 'orc_n_inter', 'orc_n_field',
                  'orc_real_bytes'):
            getattr(lib, f).restype = ctypes.c_int
        _LOADED[key] = lib
        return lib


def _arr(x, dtype):
    return np.ascontiguousarray(np.asarray(x, dtype=dtype).reshape(-1))


class CpuBackend(object):
    """
    Implements ``sim_init``/``sim_step``/``sim_clean`` of the generated
    module (``openclsim.c``) on the CPU.
    """
    def __init__(self, model, precision, dims):
        self._model = model
        self._precision = precision
        self._dims = dims
        self._lib = None
        self._running = False
        self.threads = _threads()
        # Time steps per sim_step call (None: the default below); the
        # benchmark's CPU timing sets it between calls
        self.chunk_steps = None

    # --- helpers ---------------------------------------------------------

    def _log_columns(self, log, nx, ny, n_state, inter_names, diffusion):
        """Key -> (kind, index) as log_add binds them (openclsim.c:935-1001)."""
        import myokit
        m = self._model
        tvar = m.binding('time')
        pvar = m.binding('pace')
        ivar = m.binding('diffusion_current') if diffusion else None
        states = {v.qname(): v.index() for v in m.states()}
        inters = {n: k for k, n in enumerate(inter_names)}
        kinds, idx = [], []
        for key in log.keys():
            if tvar is not None and key == tvar.qname():
                kinds.append(0)
                idx.append(0)
                continue
            if pvar is not None and key == pvar.qname():
                kinds.append(1)
                idx.append(0)
                continue
            pre, name = myokit.split_key(key)
            parts = pre.split('.')[:-1] if pre else []
            if len(parts) != self._dims:
                raise Exception(
                    'Unknown variables found in logging dictionary.')
            try:
                ix = int(parts[0])
                iy = int(parts[1]) if self._dims == 2 else 0
            except ValueError:
                raise Exception(
                    'Unknown variables found in logging dictionary.')
            if not (0 <= ix < nx and 0 <= iy < ny):
                raise Exception(
                    'Unknown variables found in logging dictionary.')
            cell = ix + iy * nx
            if ivar is not None and name == ivar.qname():
                kinds.append(2)
                idx.append(cell)
            elif name in states:
                kinds.append(3)
                idx.append(cell * n_state + states[name])
            elif name in inters:
                kinds.append(4)
                idx.append(cell * len(inter_names) + inters[name])
            else:
                raise Exception(
                    'Unknown variables found in logging dictionary.')
        return kinds, idx

    # --- reference module interface -----------------------------------

    def sim_init(self, platform, device, kernel, nx, ny, diffusion, gx, gy,
                 gx_field, gy_field, connections, tmin, tmax, dt, state_in,
                 state_out, protocol, log, log_interval, inter_log,
                 field_data):
        import myokit
        if self._running:
            raise Exception('Simulation already initialized.')
        if connections is not None and gx_field is not None:
            raise Exception('Connections and conductance fields cannot be'
                            ' used together.')
        if connections is not None:
            mode = 3
        elif gx_field is not None:
            mode = 2
        elif diffusion:
            mode = 1
        else:
            mode = 0
        lib = build_runner(kernel, mode)
        n_state = lib.orc_n_state()
        if len(state_in) != nx * ny * n_state:
            raise Exception("'state_in' must have size nx * ny * n_states.")
        inter_names = [x.decode('ascii') for x in inter_log]
        kinds, idx = self._log_columns(
            log, nx, ny, n_state, inter_names, diffusion)
        st = _arr(state_in, np.float64)
        fd = _arr(field_data, np.float64)
        gxa = _arr(gx_field if gx_field is not None else [], np.float64)
        gya = _arr(gy_field if gy_field is not None else [], np.float64)
        if connections:
            c = np.array(connections, dtype=float).reshape(-1, 3)
        else:
            c = np.zeros((0, 3))
        c1 = _arr(c[:, 0], np.int64)
        c2 = _arr(c[:, 1], np.int64)
        cg = _arr(c[:, 2], np.float64)
        ev = []
        if protocol is not None:
            for e in protocol.events():
                ev.append([e.level(), e.start(), e.duration(), e.period(),
                           e.multiplier()])
        ev = _arr(ev, np.float64)
        ki = _arr(kinds, np.int32)
        li = _arr(idx, np.int64)
        self._keep = (st, fd, gxa, gya, c1, c2, cg, ev, ki, li)
        code = lib.orc_init(
            nx, ny, gx, gy,
            gxa.ctypes.data_as(_dp), len(gxa),
            gya.ctypes.data_as(_dp), len(gya),
            c1.ctypes.data_as(_lp), c2.ctypes.data_as(_lp),
            cg.ctypes.data_as(_dp), len(cg),
            tmin, tmax, dt, log_interval,
            st.ctypes.data_as(_dp), fd.ctypes.data_as(_dp), len(fd),
            ev.ctypes.data_as(_dp), len(ev) // 5,
            ki.ctypes.data_as(_ip), li.ctypes.data_as(_lp), len(ki),
            self.threads)
        if code == -50:
            lib.orc_clean()
            raise myokit.SimultaneousProtocolEventError(
                'E-Pacing error: Event scheduled or re-occuring at the same'
                ' time as another event.')
        if code != 0:
            lib.orc_clean()
            raise Exception('E-Pacing error: Unlisted error %d' % code)
        self._lib = lib
        self._log = log
        self._keys = list(log.keys())
        self._state_out = state_out
        self._ncell = nx * ny
        self._n_state = n_state
        self._steps = max(1000, 500 + 200000 // (nx * ny))
        self._running = True

    def _flush_log(self):
        lib = self._lib
        n = lib.orc_rows()
        if n <= 0:
            return
        k = len(self._keys)
        buf = np.empty(n * max(k, 1))
        lib.orc_take_rows(buf.ctypes.data_as(_dp))
        buf = buf[:n * k].reshape(n, k)
        for j, key in enumerate(self._keys):
            self._log[key].extend(buf[:, j].tolist())

    def sim_step(self):
        import myokit
        if not self._running:
            raise Exception('Simulation not initialized.')
        t = ctypes.c_double()
        code = self._lib.orc_step(self.chunk_steps or self._steps,
                                  ctypes.byref(t))
        self._flush_log()
        if code == 0:
            return t.value
        if code < 0:
            self.sim_clean()
            if code == -50:
                raise myokit.SimultaneousProtocolEventError(
                    'E-Pacing error: Event scheduled or re-occuring at the'
                    ' same time as another event.')
            raise Exception('E-Pacing error: Unlisted error %d' % code)
        out = np.empty(self._ncell * self._n_state)
        self._lib.orc_get_state(out.ctypes.data_as(_dp))
        self._state_out[:] = out.tolist()
        self.sim_clean()
        if code == 2:
            raise ArithmeticError('Encountered nan in simulation.')
        return t.value

    def sim_clean(self):
        if self._lib is not None:
            self._lib.orc_clean()
        self._running = False
        self._keep = None
