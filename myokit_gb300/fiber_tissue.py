"""
The fiber-tissue simulation on the GPU.

:class:`FiberTissueSimulationCUDA` is the reference's
``myokit.FiberTissueSimulation`` (``myokit/_sim/fiber_tissue.py``) with its
compiled OpenCL module replaced: the reference class keeps its argument
checks, state handling, log preparation, ``find_nan`` and NaN report, and
calls ``sim_init`` / ``sim_step`` / ``sim_clean`` (``fiber_tissue.c``) on a
backend that runs one fused sm_103a kernel per chunk of steps over both
domains through the C ABI (``mkg_set_partner``). The reference renders two
OpenCL programs per run and launches five kernels per time step
(``fiber_tissue.c:1003-1130``); here there is one cooperative launch per
chunk with a bounded grid barrier between steps.
"""
import numpy as np

from ._deps import myokit
from . import _lib
from . import exporter as _exp
from .simulation import compile_kernel


class _FiberTissueBackend(object):
    """sim_init / sim_step / sim_clean over the C ABI, for one simulation."""

    def __init__(self, owner):
        self._owner = owner
        self._lib = _lib.load()
        self._handles = None       # (key, fiber handle, tissue handle)
        self._run = None

    # -- helpers ---------------------------------------------------------

    def _check(self, code, h):
        return _lib.check(code, h)

    def _kernel(self, inter_f, inter_t):
        o = self._owner
        single = o._precision == myokit.SINGLE_PRECISION
        block = (256, 1) if single else (128, 1)
        minb = 2 if single else 1
        kf = _exp.TissueKernel(
            o._modelf, o._precision, o._native_math, o._bound_variablesf,
            inter_f, _exp.DIFF_GRID, True, [], {}, block, min_blocks=minb,
            math='fast')
        kt = _exp.TissueKernel(
            o._modelt, o._precision, o._native_math, o._bound_variablest,
            inter_t, _exp.DIFF_GRID, True, [], {}, block, min_blocks=minb,
            math='fast')
        return _exp.FiberTissueKernel(kf, kt)

    def _config(self, kernel, nx, ny, n_state, n_inter, i_vm):
        cfg = _lib.MkgConfig()
        cfg.nx, cfg.ny = nx, ny
        cfg.real_bytes = 4 if kernel.single else 8
        cfg.n_state, cfg.n_inter, cfg.n_field = n_state, n_inter, 0
        cfg.i_vm = i_vm
        cfg.diffusion = _exp.DIFF_GRID
        cfg.block_x, cfg.block_y = kernel.block
        cfg.device = self._owner._device
        cfg.two_d = 1
        return cfg

    def _handles_for(self, kernel, cfgf, cfgt):
        key = (kernel.key(), bytes(cfgf), bytes(cfgt))
        if self._handles is not None and self._handles[0] == key:
            return self._handles[1], self._handles[2]
        self._close()
        cubin = compile_kernel(kernel)
        hf, ht = _lib.ctypes.c_void_p(), _lib.ctypes.c_void_p()
        _lib.check(self._lib.mkg_create(_lib.ctypes.byref(cfgf), cubin,
                                        len(cubin), _lib.ctypes.byref(hf)))
        try:
            _lib.check(self._lib.mkg_create(
                _lib.ctypes.byref(cfgt), cubin, len(cubin),
                _lib.ctypes.byref(ht)))
        except Exception:
            self._lib.mkg_destroy(hf)
            raise
        self._handles = (key, hf, ht)
        return hf, ht

    def _close(self):
        if self._handles is not None:
            for h in self._handles[1:]:
                if h is not None and h.value:
                    self._lib.mkg_destroy(h)
        self._handles = None

    def __del__(self):
        try:
            self._close()
        except Exception:   # pragma: no cover
            pass

    @staticmethod
    def _columns(log, model, nx, inter, glob):
        """
        Log keys of one domain as (item, cell) columns plus the global keys
        (the key forms of fiber_tissue.c:840-960): item = state index,
        n_state for the diffusion current, n_state + 1 + k for logged
        intermediary k.
        """
        n_state = model.count_states()
        inter_index = {v.qname(): k for k, v in enumerate(inter)}
        items, cells, cols, globals_ = [], [], [], []
        for key in log.keys():
            idx, name = myokit.split_key(key)
            if not idx:
                if name not in glob:
                    raise Exception(
                        'Unknown variables found in logging dictionary.')
                globals_.append((key, glob[name]))
                continue
            x, y = [int(v) for v in idx.split('.')[:2]]
            var = model.get(name)
            if var.is_state():
                item = var.index()
            elif var.binding() == 'diffusion_current':
                item = n_state
            elif name in inter_index:
                item = n_state + 1 + inter_index[name]
            else:
                raise Exception(
                    'Unknown variables found in logging dictionary.')
            items.append(item)
            cells.append(x + y * nx)
            cols.append(key)
        return (np.ascontiguousarray(items, dtype=np.int32),
                np.ascontiguousarray(cells, dtype=np.int64), cols, globals_)

    # -- the reference module interface ----------------------------------

    def sim_init(self, platform, device, kernelf, kernelt, nfx, nfy, ntx, nty,
                 ivf, ivt, gfx, gfy, gtx, gty, gft, cfx, ctx, cty, tmin, tmax,
                 dt, state_inf, state_int, state_outf, state_outt, protocol,
                 logf, logt, log_interval, inter_logf, inter_logt):
        o = self._owner
        lib = self._lib
        inter_f = [o._modelf.get(x.decode()) for x in inter_logf]
        inter_t = [o._modelt.get(x.decode()) for x in inter_logt]
        kernel = self._kernel(inter_f, inter_t)
        nsf, nst = o._modelf.count_states(), o._modelt.count_states()
        cfgf = self._config(kernel, nfx, nfy, nsf, len(inter_f), ivf)
        cfgt = self._config(kernel, ntx, nty, nst, len(inter_t), ivt)
        hf, ht = self._handles_for(kernel, cfgf, cfgt)

        # States, conductances, pacing (the fiber's first columns), protocol
        for h, st in ((hf, state_inf), (ht, state_int)):
            a = np.ascontiguousarray(st, dtype=np.float64)
            self._check(lib.mkg_set_state(h, _lib.dptr(a), a.size), h)
        self._check(lib.mkg_set_conductance(hf, gfx, gfy), hf)
        self._check(lib.mkg_set_conductance(ht, gtx, gty), ht)
        npaced = len(o._paced_cells) // max(nfy, 1)
        if npaced > 0:
            self._check(lib.mkg_set_paced_rect(hf, npaced, nfy, 0, 0), hf)
        else:
            self._check(lib.mkg_set_pacing_mode(hf, _lib.PACE_NONE), hf)
        self._check(lib.mkg_set_pacing_mode(ht, _lib.PACE_NONE), ht)
        ev = []
        if protocol is not None:
            for e in protocol.events():
                ev.append([e.level(), e.start(), e.duration(), e.period(),
                           e.multiplier()])
        ev = np.ascontiguousarray(np.array(ev, dtype=float).reshape(-1, 5))
        self._check(lib.mkg_set_protocol(hf, _lib.dptr(ev), len(ev)), hf)

        # Logs: time and pace are logged from the fiber
        globf = {o._modelf.time().qname(): 'time'}
        if o._modelf.binding('pace') is not None:
            globf[o._modelf.binding('pace').qname()] = 'pace'
        globt = {o._modelt.time().qname(): 'time'}
        if o._modelt.binding('pace') is not None:
            globt[o._modelt.binding('pace').qname()] = 'pace'
        colsf = self._columns(logf, o._modelf, nfx, inter_f, globf)
        colst = self._columns(logt, o._modelt, ntx, inter_t, globt)
        for h, (items, cells, _, _), n_state in (
                (hf, colsf, nsf), (ht, colst, nst)):
            nan = 1 if np.any(items < n_state) else 0
            self._check(lib.mkg_set_log(
                h, _lib.i32ptr(items), _lib.i64ptr(cells), len(items),
                nan), h)
        self._check(lib.mkg_set_partner(hf, ht, gft, cty), hf)
        self._check(lib.mkg_set_tuning(hf, 0, 0, 0), hf)
        self._check(lib.mkg_run_begin(hf, tmin, tmax, dt, log_interval), hf)
        self._run = dict(
            hf=hf, ht=ht, tmin=tmin, logf=logf, logt=logt, colsf=colsf,
            colst=colst, outf=state_outf, outt=state_outt,
            nf=nfx * nfy * nsf, nt=ntx * nty * nst,
            chunk=int(max(40, min(100000, 2e9 / (nfx * nfy + ntx * nty)))))

    def _append(self, log, cols, values, time, pace):
        items, cells, keys, globs = cols
        for j, key in enumerate(keys):
            log[key].extend(values[:, j].tolist())
        for key, what in globs:
            log[key].extend((time if what == 'time' else pace).tolist())

    def sim_step(self):
        r = self._run
        lib = self._lib
        hf, ht = r['hf'], r['ht']
        t = _lib.ctypes.c_double()
        rows = _lib.ctypes.c_int64()
        status = self._check(lib.mkg_run_chunk(
            hf, r['chunk'], _lib.ctypes.byref(t), _lib.ctypes.byref(rows)),
            hf)
        n = rows.value
        if n:
            time, pace = np.empty(n), np.empty(n)
            vf = np.empty((n, len(r['colsf'][2])))
            vt = np.empty((n, len(r['colst'][2])))
            self._check(lib.mkg_read_log(
                hf, _lib.dptr(time), _lib.dptr(pace),
                _lib.dptr(vf) if vf.size else None, n), hf)
            self._check(lib.mkg_read_log(
                ht, None, None, _lib.dptr(vt) if vt.size else None, n), ht)
            self._append(r['logf'], r['colsf'], vf, time, pace)
            self._append(r['logt'], r['colst'], vt, time, pace)
        if status == _lib.MKG_OK:
            return t.value
        # Final states (also after a NaN halt, fiber_tissue.c:1160-1172)
        for h, out, size in ((hf, r['outf'], r['nf']),
                             (ht, r['outt'], r['nt'])):
            a = np.empty(size)
            self._check(lib.mkg_get_state(h, _lib.dptr(a), size), h)
            out[:] = a.tolist()
        if status == _lib.MKG_HALT_NAN:
            return r['tmin'] - 1
        return t.value

    def sim_clean(self):
        # Device buffers and the compiled kernel stay for the next run
        if self._run is not None:
            self._lib.mkg_set_partner(self._run['hf'], None, 0.0, 0)
        self._run = None


class FiberTissueSimulationCUDA(myokit.FiberTissueSimulation):
    """
    ``myokit.FiberTissueSimulation`` (same arguments, methods and results)
    running on one GB300: a fiber of ``ncells_fiber`` cells leading into a
    rectangular tissue of ``ncells_tissue`` cells, each with its own model,
    advanced by one fused CUDA kernel per chunk of steps.

    The extra keyword argument ``device`` selects the CUDA device.
    """
    def __init__(self, *args, device=0, **kwargs):
        self._device = int(device)
        super().__init__(*args, **kwargs)

    def _create_backend(self):
        self._sim = _FiberTissueBackend(self)

    def _export(self, template, variables, target=None,
                continue_in_debug_mode=False):
        # The OpenCL kernels the reference renders per run are not used:
        # the CUDA kernel is generated from the models themselves
        return ''
