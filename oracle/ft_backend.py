"""
CPU stand-in for the compiled module of ``myokit.FiberTissueSimulation``.

TEST INFRASTRUCTURE (the oracle). Only ``tests/`` use it; the product never
does.

``FiberTissueSimulation`` renders two OpenCL programs per run (fiber and
tissue) and hands them to a generated CPython module with the methods
``sim_init``, ``sim_step`` and ``sim_clean`` (``myokit/_sim/fiber_tissue.c``).
:class:`FiberTissueCpuBackend` implements those methods with the same
arguments and effects: each rendered program is compiled as C
(``oracle/ft_kernel.c`` with ``oracle/oracle_shim.h``), and the step loop of
``fiber_tissue.c:1003-1185`` is restated here, with the reference's own
``myokit.PacingSystem`` for the event pacing. The reference Python layer
(argument checks, rendering, logging, ``find_nan``) runs unmodified in
:class:`ReferenceFiberTissueCpu`.
"""
import ctypes
import hashlib
import os
import subprocess
import threading

import numpy as np

from myokit_gb300._deps import myokit

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, '_ref')
_LOCK = threading.Lock()
_LOADED = {}


def build_kernel(source, junction):
    """Compiles ``ft_kernel.c`` around one rendered program; returns a CDLL."""
    h = hashlib.sha256()
    h.update(source.encode())
    h.update(b'junction' if junction else b'-')
    for name in ('ft_kernel.c', 'oracle_shim.h'):
        with open(os.path.join(_HERE, name), 'rb') as f:
            h.update(f.read())
    key = 'ft_' + h.hexdigest()[:24]
    with _LOCK:
        if key in _LOADED:
            return _LOADED[key]
        os.makedirs(REF_DIR, exist_ok=True)
        cl = os.path.join(REF_DIR, key + '.cl')
        so = os.path.join(REF_DIR, key + '.so')
        if not os.path.exists(so):
            with open(cl, 'w') as f:
                f.write(source)
            tmp = so + '.%d' % os.getpid()
            cmd = ['gcc', '-O2', '-std=gnu99', '-fPIC', '-shared',
                   '-ffp-contract=off', '-w', '-I' + _HERE,
                   '-DORC_KERNEL="' + cl + '"']
            if junction:
                cmd.append('-DFTK_JUNCTION')
            cmd += [os.path.join(_HERE, 'ft_kernel.c'), '-o', tmp, '-lm']
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError('Oracle build failed:\n' + r.stderr)
            os.replace(tmp, so)
        lib = ctypes.CDLL(so)
        vp, L, D = ctypes.c_void_p, ctypes.c_long, ctypes.c_double
        lib.ftk_real_bytes.restype = ctypes.c_int
        lib.ftk_diff.argtypes = [L, L, D, D, vp, vp]
        lib.ftk_cell.argtypes = [L, L, D, D, D, vp, vp, vp, vp]
        if junction:
            lib.ftk_junction.argtypes = [L, L, L, L, L, L, L, ctypes.c_int,
                                         ctypes.c_int, D, vp, vp, vp, vp]
        _LOADED[key] = lib
        return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _Domain(object):
    """Buffers and log sources of the fiber or the tissue."""

    def __init__(self, lib, model, nx, ny, state, inter_names, log, glob,
                 real):
        self.lib, self.nx, self.ny = lib, nx, ny
        self.n_state = model.count_states()
        self.state = np.array(state, dtype=real)
        self.idiff = np.zeros(nx * ny, dtype=real)
        n_inter = len(inter_names)
        self.n_inter = n_inter
        self.inter = np.zeros(max(1, nx * ny * n_inter), dtype=real)
        self.field = np.zeros(1, dtype=real)
        inter_index = {n: k for k, n in enumerate(inter_names)}
        self.log = log
        # Log sources (fiber_tissue.c:840-960): ('g', 'time' | 'pace'),
        # ('s', state index), ('d', cell), ('i', inter index)
        self.sources = []
        self.logging_states = False
        for key in log.keys():
            idx, name = myokit.split_key(key)
            if not idx:
                if name not in glob:
                    raise Exception(
                        'Unknown variables found in logging dictionary.')
                self.sources.append((key, 'g', glob[name]))
                continue
            x, y = [int(v) for v in idx.split('.')[:2]]
            cell = x + y * nx
            var = model.get(name)
            if var.is_state():
                self.sources.append(
                    (key, 's', cell * self.n_state + var.index()))
                self.logging_states = True
            elif var.binding() == 'diffusion_current':
                self.sources.append((key, 'd', cell))
            elif name in inter_index:
                self.sources.append(
                    (key, 'i', cell * n_inter + inter_index[name]))
            else:
                raise Exception(
                    'Unknown variables found in logging dictionary.')
        self.snap = {}

    def diff(self, gx, gy):
        self.lib.ftk_diff(self.nx, self.ny, gx, gy, _ptr(self.state),
                          _ptr(self.idiff))

    def cell(self, t, dt, pace):
        self.lib.ftk_cell(self.nx, self.ny, t, dt, pace, _ptr(self.state),
                          _ptr(self.idiff), _ptr(self.inter),
                          _ptr(self.field))

    def snapshot(self):
        # States at t, read before the cell kernel (fiber_tissue.c:1036)
        self.snap = {key: float(self.state[i])
                     for key, kind, i in self.sources if kind == 's'}

    def write(self, arg_time, arg_pace):
        for key, kind, i in self.sources:
            if kind == 'g':
                v = arg_time if i == 'time' else arg_pace
            elif kind == 's':
                v = self.snap[key]
            elif kind == 'd':
                v = self.idiff[i]
            else:
                v = self.inter[i]
            self.log[key].append(float(v))


class FiberTissueCpuBackend(object):
    """sim_init / sim_step / sim_clean of fiber_tissue.c, on the CPU."""

    def __init__(self, owner):
        self._owner = owner

    def sim_init(self, platform, device, kernelf, kernelt, nfx, nfy, ntx, nty,
                 ivf, ivt, gfx, gfy, gtx, gty, gft, cfx, ctx, cty, tmin, tmax,
                 dt, state_inf, state_int, state_outf, state_outt, protocol,
                 logf, logt, log_interval, inter_logf, inter_logt):
        o = self._owner
        libf = build_kernel(kernelf, True)
        libt = build_kernel(kernelt, False)
        real = np.float32 if libf.ftk_real_bytes() == 4 else np.float64
        self.R = real
        globf = {o._modelf.time().qname(): 'time'}
        if o._modelf.binding('pace') is not None:
            globf[o._modelf.binding('pace').qname()] = 'pace'
        globt = {o._modelt.time().qname(): 'time'}
        if o._modelt.binding('pace') is not None:
            globt[o._modelt.binding('pace').qname()] = 'pace'
        self.f = _Domain(libf, o._modelf, nfx, nfy, state_inf,
                         [x.decode() for x in inter_logf], logf, globf, real)
        self.t = _Domain(libt, o._modelt, ntx, nty, state_int,
                         [x.decode() for x in inter_logt], logt, globt, real)
        self.g = (gfx, gfy, gtx, gty, gft)
        self.junction = (nfx, nfy, ntx, ctx, cty, self.f.n_state,
                         self.t.n_state, ivf, ivt)
        self.tmin, self.tmax, self.default_dt = tmin, tmax, dt
        self.log_interval = log_interval
        self.pacing = myokit.PacingSystem(
            protocol if protocol is not None else myokit.Protocol(), tmin)
        self.tnext_pace = self.pacing.next_time()
        self.engine_pace = self.pacing.pace()
        self.arg_pace = float(real(self.engine_pace))
        self.engine_time = tmin
        self.arg_time = float(real(tmin))
        self.istep = 1
        self.inext_log = 0
        self.tnext_log = tmin
        self.halt = False
        self.outf, self.outt = state_outf, state_outt
        self.steps_per_call = max(40, int(6e6 / (nfx * nfy + ntx * nty)))

    def sim_step(self):
        f, t = self.f, self.t
        gfx, gfy, gtx, gty, gft = self.g
        R = self.R
        left = self.steps_per_call
        while True:
            logging = self.engine_time >= self.tnext_log
            intermediary = False
            dt = (self.tmin + self.istep * self.default_dt
                  - self.engine_time)
            for tn in (self.tmax, self.tnext_pace, self.tnext_log):
                d = tn - self.engine_time
                if d > 0 and d < dt:
                    dt = d
                    intermediary = True
            if not intermediary:
                self.istep += 1
            arg_dt = float(R(dt))

            # Diffusion current at t (fiber, tissue, junction)
            f.diff(gfx, gfy)
            t.diff(gtx, gty)
            f.lib.ftk_junction(*self.junction, gft, _ptr(f.state),
                               _ptr(t.state), _ptr(f.idiff), _ptr(t.idiff))

            # States at t for the log; the NaN check on the first entry
            if logging:
                for d in (f, t):
                    if d.logging_states:
                        d.snapshot()
                        if np.isnan(d.state[0]):
                            self.halt = True

            # Intermediaries at t, states to t + dt
            f.cell(self.arg_time, arg_dt, self.arg_pace)
            t.cell(self.arg_time, arg_dt, self.arg_pace)

            if logging:
                f.write(self.arg_time, self.arg_pace)
                t.write(self.arg_time, self.arg_pace)
                self.inext_log += 1
                self.tnext_log = self.tmin + self.inext_log * self.log_interval

            self.engine_time += dt
            self.arg_time = float(R(self.engine_time))
            self.pacing.advance(self.engine_time)
            self.tnext_pace = self.pacing.next_time()
            self.engine_pace = self.pacing.pace()
            self.arg_pace = float(R(self.engine_pace))

            if self.engine_time >= self.tmax or self.halt:
                break
            left -= 1
            if left == 0:
                return self.engine_time

        self.outf[:] = [float(x) for x in f.state]
        self.outt[:] = [float(x) for x in t.state]
        return self.tmin - 1 if self.halt else self.engine_time

    def sim_clean(self):
        pass


class ReferenceFiberTissueCpu(myokit.FiberTissueSimulation):
    """The reference FiberTissueSimulation, unmodified apart from its
    compiled module, which is :class:`FiberTissueCpuBackend`."""

    def _create_backend(self):
        self._sim = FiberTissueCpuBackend(self)
