#!/usr/bin/env python3
"""
Headline benchmark: cell-steps/s of the fused tissue step on one GB300.

Workload (a 2D sheet as in the reference's SimulationOpenCL use):
  512 x 512 cells, Rush-Larsen on, dt = 0.005 ms, the 4 left columns paced
  by a 1 Hz protocol (2 ms pulses, level 1), per-cell GKr and GNa scale
  fields lognormal(0, 0.2) from a seed, V logged every 1 ms at 256 seeded
  random probe cells. The O'Hara-Rudy 2011 model file is not available, so
  the 48-state Decker 2009 canine model shipped with myokit stands in.

One bench step = ``run(step_ms)`` of that sheet (2000 time steps at the
default 10 ms). ``value`` is cell-steps per second of device time with the
state resident in HBM (CUDA events on the simulation's stream around the
kernel launches); ``e2e`` is the same metric through the public
``SimulationCUDA.run`` call, state upload, log and final state download
included. Single precision is the headline; double precision is timed on
the same sheet and the largest |dV| between the two at the probes is
reported.

--impl reference times the reference's own kernel (the OpenCL C that
myokit's SimulationOpenCL renders for this model, compiled for the host
CPU and driven by the oracle's restatement of the reference step loop) on
all host cores, with the same metric and configuration.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'cell-steps/s on 1 GB300 (FP32 vs FP64 at stated max|dV|)'

# Single precision variants: FP64 or compensated accumulation of V and the
# concentrations, and the fast FP32 arithmetic option
VARIANTS = [
    ('fp32+double', {'accumulate': 'double'}),
    ('fp32+kahan', {'accumulate': 'kahan'}),
    ('fp32-ieee-div', {'fp32_math': 'ieee'}),
]
UNIT = 'cell-steps/s'


def parse():
    p = argparse.ArgumentParser(description=__doc__.split('\n')[1])
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=10)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    p.add_argument('--size', type=int, default=512)
    p.add_argument('--step-ms', type=float, default=10.0)
    p.add_argument('--fp64-steps', type=int, default=2,
                   help='timed double precision bench steps (0 = skip)')
    p.add_argument('--variant-steps', type=int, default=3,
                   help='timed steps of the FP64/Kahan accumulation variants')
    p.add_argument('--accuracy-ms', type=float, default=400.0,
                   help='simulated time of the precision comparison runs'
                        ' (0 = skip)')
    p.add_argument('--adjoint-ms', type=float, default=300.0,
                   help='simulated time of the adjoint measurement (the'
                        ' 256 x 256 adjoint configuration runs 300 ms;'
                        ' 0 = skip)')
    p.add_argument('--configs', default='c1,c3,c5',
                   help='other configurations to time: comma list of c1'
                        ' (200-cell FP64 cable), c3 (512 batched cables), c5'
                        ' (2048x2048 S1-S2 sheet), or none')
    p.add_argument('--c5-full', action='store_true',
                   help='run the whole 1000 ms S1-S2 protocol of the'
                        ' 2048x2048 sheet instead of a 20 ms window')
    p.add_argument('--full', action='store_true',
                   help='run every configuration at its full length: the'
                        ' batched cables for 2000 ms, the adjoint over'
                        ' 300 ms, the 2048x2048 S1-S2 protocol for 1000 ms')
    p.add_argument('--profile', action='store_true',
                   help='run one small sheet case for a profiler and exit')
    p.add_argument('--tune', action='store_true',
                   help='autotune the launch shape of every benchmark'
                        ' configuration, print the timings and the table'
                        ' (the format of myokit_gb300/tuned.json), exit')
    p.add_argument('--profile-steps', type=int, default=40)
    p.add_argument('--no-fields', action='store_true',
                   help='with --profile: a sheet without scalar fields (the'
                        ' 2048x2048 S1-S2 configuration)')
    p.add_argument('--profile-adjoint', action='store_true',
                   help='with --profile: run the discrete adjoint (loss on'
                        ' 64 probes, checkpoints every 200 steps) instead')
    p.add_argument('--adj-min-blocks', type=int, default=1,
                   help='resident CTAs per SM asked for the reverse kernel')
    p.add_argument('--adj-threads', type=int, default=0,
                   help='CTA size of the reverse kernel (0: the forward\'s)')
    p.add_argument('--adj-guards', action='store_true',
                   help='reverse sweep with a zero-adjoint branch per'
                        ' equation (default: straight-line)')
    p.add_argument('--no-stage', action='store_true',
                   help='profile the kernel that reads tiles from global'
                        ' memory instead of staging them with TMA')
    p.add_argument('--precision', choices=['single', 'double'],
                   default='single')
    p.add_argument('--accumulate', choices=['none', 'kahan', 'double'],
                   default='none')
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--clocks-csv', default=None,
                   help='also write the raw nvidia-smi clock samples of the'
                        ' timed region to this CSV file')
    p.add_argument('--cpu-seconds', type=float, default=12.0,
                   help='target CPU work for the cpu_baseline sample')
    return p.parse_args()


def load_model():
    from myokit_gb300._deps import myokit
    path = os.path.join(os.path.dirname(myokit.__file__), 'tests', 'data',
                        'decker-2009.mmt')
    return myokit.load_model(path)


def make_sheet(cls, precision, size, seed=0, fields=True, **kw):
    """The benchmark sheet; returns (simulation, log variable list)."""
    from myokit_gb300._deps import myokit
    m = load_model()
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = cls(m, p, ncells=(size, size), precision=precision, rl=True, **kw)
    s.set_step_size(0.005)
    s.set_paced_cells(nx=4, ny=size, x=0, y=0)
    rng = np.random.default_rng(seed)
    gkr = m.get('ikr.Gbar').eval()
    gna = m.get('ina.Gbar').eval()
    if fields:
        s.set_field('ikr.Gbar', gkr * rng.lognormal(0, 0.2, (size, size)))
        s.set_field('ina.Gbar', gna * rng.lognormal(0, 0.2, (size, size)))
    cells = rng.choice(size * size, 256, replace=False)
    log = ['engine.time'] + [
        '%d.%d.membrane.V' % (c % size, c // size) for c in sorted(cells)]
    return s, log


def config(args, workload):
    return {
        'workload': workload,
        'model': 'decker-2009 (48 states; stands in for O\'Hara-Rudy 2011'
                 ' endo, whose model file is unavailable)',
        'grid': [args.size, args.size],
        'rl': True, 'dt_ms': 0.005, 'step_ms': args.step_ms,
        'paced': 'left 4 columns, 1 Hz, 2 ms, level 1',
        'fields': 'GKr, GNa x lognormal(0, 0.2), seed 0',
        'log': 'V at 256 probes every 1 ms',
        'l2': 'flushed between timed steps (256 MiB write)',
    }


class ClockSampler(object):
    """Samples nvidia-smi clocks and throttle reasons in the background."""
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,'
              'clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, out=None):
        self.proc = None
        self.out = out

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        self.lines = []
        if self.proc is not None:
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:   # pragma: no cover
            self.proc.kill()
        self.th.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(name)
        if self.out:
            with open(self.out, 'w') as f:
                f.write('\n'.join(self.lines) + '\n')
        if not sm:
            return None
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': max(mx),
                'samples': len(sm), 'reasons': sorted(reasons)}


def read_peaks():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def read_traffic():
    """Per-cell-step DRAM bytes of the tissue kernel from the committed ncu
    summary, or None."""
    path = os.path.join(ROOT, 'profiles', 'tissue_step_traffic.json')
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def cpu_baseline(args, precision, seconds):
    """Times the reference kernel on the host cores for a bounded sample."""
    from oracle.refsim import ReferenceCpuSimulation
    cores = os.cpu_count() or 1
    s, _ = make_sheet(ReferenceCpuSimulation, precision, args.size)
    s.set_threads(cores)
    ncell = args.size * args.size
    # Calibrate on a short run, then size the sample
    t0 = time.perf_counter()
    s.run(0.05, log=['engine.time'], log_interval=1)   # 10 steps
    dt = time.perf_counter() - t0
    rate0 = ncell * 10 / max(dt, 1e-9)
    nsteps = int(max(20, min(20000, rate0 * seconds / ncell)))
    t0 = time.perf_counter()
    s.run(nsteps * 0.005, log=['engine.time'], log_interval=1)
    dt = time.perf_counter() - t0
    return {
        'value': ncell * nsteps / dt, 'unit': UNIT, 'cores': cores,
        'kind': 'reference',
        'sample': '%d time steps (%.3g ms) of the %dx%d sheet, %s; the'
                  ' reference-rendered OpenCL kernel compiled as C (gcc -O2,'
                  ' OpenMP) with the oracle host loop' % (
                      nsteps, nsteps * 0.005, args.size, args.size,
                      'single precision' if precision == 32 else
                      'double precision'),
        'seconds': dt,
    }


def accuracy_runs(args, device):
    """
    Precision comparison over a full action potential: max |dV|, activation
    time and APD90 errors at probe cells of (a) a 128x128 sheet against its
    FP64 run on the GPU and (b) a 24x24 sheet against the FP64 CPU oracle
    (the reference's kernel), both with the bench sheet's configuration.
    """
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    from myokit_gb300 import metrics
    from oracle.refsim import ReferenceCpuSimulation
    modes = [('fp32', {})] + list(VARIANTS)
    out = {}

    def probes(n, k, seed):
        rng = np.random.default_rng(seed)
        cells = sorted(rng.choice(n * n, k, replace=False))
        return ['%d.%d.membrane.V' % (c % n, c // n) for c in cells]

    def traces(d, keys):
        return {k: np.asarray(d[k], dtype=float) for k in keys}

    # (a) 128 x 128 against FP64 on the GPU
    n = 128
    keys = probes(n, 64, 1)
    log = ['engine.time'] + keys
    s, _ = make_sheet(mg.SimulationCUDA, myokit.DOUBLE_PRECISION, n,
                      device=device)
    ref = s.run(args.accuracy_ms, log=log, log_interval=0.5)
    t = np.asarray(ref['engine.time'])
    res = {}
    for name, kw in modes:
        s, _ = make_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION, n,
                          device=device, **kw)
        d = s.run(args.accuracy_ms, log=log, log_interval=0.5)
        res[name] = metrics.compare(t, traces(d, keys), traces(ref, keys))
    out['sheet128_vs_fp64_gpu'] = dict(res, window_ms=args.accuracy_ms,
                                       probes=len(keys))

    # (b) 24 x 24 against the FP64 CPU oracle
    n = 24
    keys = probes(n, 32, 2)
    log = ['engine.time'] + keys
    so, _ = make_sheet(ReferenceCpuSimulation, myokit.DOUBLE_PRECISION, n)
    so.set_threads(os.cpu_count() or 1)
    ref = so.run(args.accuracy_ms, log=log, log_interval=0.5)
    t = np.asarray(ref['engine.time'])
    res = {}
    for name, kw in [('fp64', {'precision': myokit.DOUBLE_PRECISION})] + [
            (m, dict(k, precision=myokit.SINGLE_PRECISION))
            for m, k in modes]:
        kw = dict(kw)
        prec = kw.pop('precision')
        s, _ = make_sheet(mg.SimulationCUDA, prec, n, device=device, **kw)
        d = s.run(args.accuracy_ms, log=log, log_interval=0.5)
        res[name] = metrics.compare(t, traces(d, keys), traces(ref, keys))
    out['sheet24_vs_fp64_oracle'] = dict(res, window_ms=args.accuracy_ms,
                                         probes=len(keys))
    return out


def adjoint_runs(args, device):
    """
    The discrete adjoint on a 256 x 256 sheet of the bench configuration
    (single precision forward with V and concentrations in FP64): loss =
    sum of squared V errors at 64 probes every 1 ms against a target made
    with seed-perturbed GKr/GNa fields; gradient with respect to both
    fields and gx, gy; checkpoints every 200 steps.
    Reports adjoint time / forward time, and a central finite-difference
    check (relative step 1e-4, double precision, 64 x 64 sheet, 20 random
    entries).
    """
    import torch
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    from myokit_gb300 import adjoint as ad
    out = {}
    n = 256
    dur = 300.0 if args.full else args.adjoint_ms
    rng = np.random.default_rng(5)
    cells = rng.choice(n * n, 64, replace=False)
    probes = [(int(c % n), int(c // n)) for c in cells]
    keys = ['%d.%d.membrane.V' % p for p in probes]
    s, _ = make_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION, n,
                      seed=1, device=device, accumulate='double')
    adj = ad.TissueAdjoint(s, probes, segment_steps=200)
    target = adj.forward(dur, 1.0)
    s, _ = make_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION, n,
                      seed=0, device=device, accumulate='double')
    adj = ad.TissueAdjoint(s, probes, segment_steps=200)
    adj.loss_and_gradient(min(dur, 5.0), target[:int(min(dur, 5.0))], 1.0)
    s.run(min(dur, 5.0), log=['engine.time'] + keys, log_interval=1)
    s.reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.run(dur, log=['engine.time'] + keys, log_interval=1)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    s.reset()
    t0 = time.perf_counter()
    v = adj.forward(dur, 1.0)
    t1 = time.perf_counter()
    grads = adj.backward(2 * (v - target))
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    out['sheet256_fp32'] = {
        'precision': 'fp32 with FP64 V and concentrations',
        'accumulated_states': [x.qname() for x in s.accumulated_states()],
        'window_ms': dur, 'probes': len(probes), 'segment_steps': 200,
        'forward_s': t_fwd, 'adjoint_forward_s': t1 - t0,
        'adjoint_backward_s': t2 - t1,
        'adjoint_over_forward': (t2 - t0) / t_fwd,
        'loss': float(np.sum((v - target) ** 2)),
        'grad_norm_gkr': float(np.linalg.norm(grads['ikr.Gbar'])),
        'grad_gx': grads['gx'], 'grad_gy': grads['gy'],
    }

    # Finite-difference check in double precision on a 64 x 64 sheet
    n = 64
    fd_ms = min(dur, 50.0)
    cells = rng.choice(n * n, 16, replace=False)
    probes = [(int(c % n), int(c // n)) for c in cells]
    s, _ = make_sheet(mg.SimulationCUDA, myokit.DOUBLE_PRECISION, n,
                      seed=1, device=device)
    adj = ad.TissueAdjoint(s, probes, segment_steps=200)
    target = adj.forward(fd_ms, 1.0)
    s, _ = make_sheet(mg.SimulationCUDA, myokit.DOUBLE_PRECISION, n,
                      seed=0, device=device)
    adj = ad.TissueAdjoint(s, probes, segment_steps=200)
    L, grads = adj.loss_and_gradient(fd_ms, target, 1.0)
    base = {k: np.array(s._fields[s._model.get(k)]).reshape(n, n)
            for k in ('ikr.Gbar', 'ina.Gbar')}

    def loss():
        v = adj.forward(fd_ms, 1.0)
        return float(np.sum((v - target) ** 2))
    worst = 0.0
    entries = []
    for i in range(20):
        name = ('ikr.Gbar', 'ina.Gbar')[i % 2]
        iy, ix = int(rng.integers(0, n)), int(rng.integers(0, n))
        f = base[name].copy()
        h = 1e-4 * f[iy, ix]
        vals = []
        for sg in (1, -1):
            g = f.copy()
            g[iy, ix] += sg * h
            s.set_field(name, g)
            vals.append(loss())
        s.set_field(name, f)
        fd = (vals[0] - vals[1]) / (2 * h)
        a = grads[name][iy, ix]
        rel = abs(a - fd) / max(abs(fd), 1e-12 * abs(L))
        worst = max(worst, rel)
        entries.append({'field': name, 'cell': [ix, iy], 'adjoint': a,
                        'fd': fd, 'rel_err': rel})
    out['fd_check_sheet64_fp64'] = {
        'window_ms': fd_ms, 'entries': len(entries),
        'max_rel_err': worst, 'loss': L, 'sample': entries[:4]}
    return out


def config_c1(args, device):
    """
    Plain method, FP64: a 200-cell Beeler-Reuter 1977 cable, forward Euler,
    dt 0.005 ms, g = 9, the first 5 cells paced at 1 Hz (2 ms pulses), V of
    every cell logged every 1 ms, 1000 ms. Timed on the GPU in double
    precision and single precision with Kahan accumulation; compared with
    the reference's own Simulation1d (C, one host core) on a 100 ms window.
    """
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    path = os.path.join(os.path.dirname(myokit.__file__), 'tests', 'data',
                        'beeler-1977-model.mmt')
    m = myokit.load_model(path)
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    out = {'cells': 200, 'steps': 200000}

    def setup(cls, **kw):
        s = cls(m, p, ncells=200, **kw)
        s.set_step_size(0.005)
        s.set_conductance(9)
        s.set_paced_cells(5)
        return s
    log = ['engine.time', 'membrane.V']
    logs = {}
    for name, kw in (('fp64', {'precision': myokit.DOUBLE_PRECISION}),
                     ('fp32+kahan', {'precision': myokit.SINGLE_PRECISION,
                                     'accumulate': 'kahan'})):
        s = setup(mg.SimulationCUDA, device=device, **kw)
        s.run(5, log=log, log_interval=1)
        s.reset()
        t0 = time.perf_counter()
        d = s.run(1000, log=log, log_interval=1)
        wall = time.perf_counter() - t0
        st = s.last_run_stats()
        logs[name] = d
        out[name] = {'value': 200 * 200000 / (st['kernel_ms'] / 1000),
                     'e2e': 200 * 200000 / wall, 'unit': UNIT,
                     'wall_s': wall}
    try:
        sa = setup(myokit.Simulation1d)
        t0 = time.perf_counter()
        da = sa.run(100, log=log, log_interval=1)
        wall = time.perf_counter() - t0
    except Exception as e:  # the reference compiles C at run time
        out['simulation1d_cpu'] = {'unavailable': str(e).splitlines()[0]}
        return out
    out['simulation1d_cpu'] = {'value': 200 * 20000 / wall, 'unit': UNIT,
                               'cores': 1, 'window_ms': 100}
    dv = {}
    for name, d in logs.items():
        dv[name] = max(float(np.max(np.abs(
            np.asarray(da['membrane.V', c]) -
            np.asarray(d['membrane.V', c])[:100]))) for c in range(200))
    out['max_abs_dV_vs_simulation1d_mV'] = dv
    return out


def config_c3(args, device):
    """
    Batched: 512 independent cables of lengths uniform 50-2000 cells in one
    1D simulation (zero conductance between cables), 6 conductances per
    cable scaled lognormal(0, 0.3), dt 0.01 ms, the first 5 cells of each
    cable paced at 1 Hz; single precision with Kahan-compensated V and
    concentrations; launches of 100 steps replayed from CUDA graphs. The
    Decker 2009 model stands in for ten Tusscher 2006. Timed over 20 ms.
    """
    from myokit_gb300._deps import myokit
    m = load_model()
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    out = {}
    for spl in (100, 0):
        s, batch = _cables(m, p, steps_per_launch=spl, device=device)
        out['cables'] = len(batch.lengths)
        out['cells'] = batch.ncells
        window = 2000 if (args.full and spl == 100) else 20
        s.run(2, log=['engine.time'], log_interval=1)
        t0 = time.perf_counter()
        d = s.run(window, log=['engine.time'] + batch.cable_log_keys(
            len(batch.lengths) - 1)[-1:], log_interval=1)
        wall = time.perf_counter() - t0
        st = s.last_run_stats()
        out['steps_per_launch_%d' % spl] = {
            'value': st['cell_steps'] / (st['kernel_ms'] / 1000),
            'e2e': st['cell_steps'] / wall,
            'unit': UNIT, 'launches': st['launches'], 'window_ms': window}
        if window == 2000:
            # The last cable's far end fires once per paced beat
            v = np.asarray(d[batch.cable_log_keys(
                len(batch.lengths) - 1)[-1]])
            out['last_cable_end_max_v_mV'] = float(v.max())
    return out


CABLE_FIELDS = ['ina.Gbar', 'inal.Gbar', 'ik1.Gbar', 'ikr.Gbar', 'ito.Gbar',
                'ikur.Gbar']


def _cables(m, p, **kw):
    """The 512 batched cables: lengths uniform 50-2000 (seed 3), six
    conductances x lognormal(0, 0.3) per cable, first 5 cells paced,
    g = 10 inside a cable, dt 0.01 ms, FP32 + Kahan."""
    from myokit_gb300.batch import CableBatch
    rng = np.random.default_rng(3)
    lengths = rng.integers(50, 2001, 512)
    fields = {name: m.get(name).eval() * rng.lognormal(0, 0.3, 512)
              for name in CABLE_FIELDS}
    batch = CableBatch(m, lengths, p, conductance=10.0, paced_cells=5,
                       fields=fields, rl=True, accumulate='kahan', **kw)
    batch.sim.set_step_size(0.01)
    return batch.sim, batch


def config_c5(args, device):
    """
    Large: a 2048 x 2048 sheet, single precision with Kahan-compensated V
    and concentrations, dt 0.005 ms; S1 on the left edge at t = 0, then S2
    on the lower-left quadrant at t = 320 ms; the full V frame every 5 ms
    recorded in a device buffer (run_frames). Timed over a 20 ms window,
    or the whole 1000 ms with --c5-full.
    """
    import torch
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    n = 2048
    m = load_model()
    s1 = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = mg.SimulationCUDA(m, s1, ncells=(n, n), rl=True, accumulate='kahan',
                          device=device)
    s.set_step_size(0.005)
    s.set_paced_cells(nx=4, ny=n, x=0, y=0)
    s.run_frames(1, 5)
    s.reset()
    out = {'grid': [n, n]}
    torch.cuda.synchronize()
    if args.c5_full or args.full:
        t0 = time.perf_counter()
        t1_, f1 = s.run_frames(320, 5)
        ms = s.last_run_stats()['kernel_ms']
        s.set_paced_cells(nx=n // 2, ny=n // 2, x=0, y=0)
        p2 = myokit.Protocol()
        p2.schedule(level=1, start=320, duration=2)
        s.set_protocol(p2)
        t2_, f2 = s.run_frames(680, 5)
        ms += s.last_run_stats()['kernel_ms']
        wall = time.perf_counter() - t0
        frames = torch.cat([f1, f2])
        steps = 200000
        out.update({'window_ms': 1000, 'frames': int(frames.shape[0]),
                    'frame_bytes': int(frames[0].numel() *
                                       frames.element_size()),
                    'final_v_range_mV': [float(frames[-1].min()),
                                         float(frames[-1].max())],
                    'activated_fraction_final': float(
                        (frames[-1] > -40).float().mean())})
    else:
        t0 = time.perf_counter()
        tt, frames = s.run_frames(20, 5)
        wall = time.perf_counter() - t0
        ms = s.last_run_stats()['kernel_ms']
        steps = 4000
        out.update({'window_ms': 20, 'frames': int(frames.shape[0])})
    out['value'] = n * n * steps / (ms / 1000)
    out['e2e'] = n * n * steps / wall
    out['unit'] = UNIT
    k = s._last_kernel
    peak, kind = read_peaks()
    bpcs = k.bytes_per_cell_step()
    out['roofline'] = {'bound': 'hbm', 'bytes_per_cell_step': bpcs,
                       'achieved': out['value'] * bpcs / 1e9, 'peak': peak,
                       'unit': 'GB/s', 'peak_source': kind,
                       'frac': out['value'] * bpcs / 1e9 / peak}
    del s, frames
    torch.cuda.empty_cache()

    # The plain FP64 path on the same sheet, over 1 ms (200 steps)
    s64 = mg.SimulationCUDA(m, s1, ncells=(n, n), rl=True, device=device,
                            precision=myokit.DOUBLE_PRECISION)
    s64.set_step_size(0.005)
    s64.set_paced_cells(nx=4, ny=n, x=0, y=0)
    s64.run(0.05, log=['engine.time'], log_interval=1)
    s64.run(1, log=['engine.time'], log_interval=1)
    st = s64.last_run_stats()
    v64 = st['cell_steps'] / (st['kernel_ms'] / 1000)
    out['fp64'] = {'value': v64, 'unit': UNIT, 'window_ms': 1}
    out['speedup_over_fp64'] = out['value'] / v64
    return out


def tune_configs(args):
    """
    Runs the autotuner on each benchmark configuration: the 512 x 512 sheet
    in every precision mode, the 2048 x 2048 sheet (FP32 and Kahan), the
    512 batched cables and the 200-cell cable. Results go to the user cache
    (MYOKIT_GB300_CACHE or ~/.cache/myokit_gb300); the table is printed.
    """
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    from myokit_gb300 import autotune as at
    SP, DP = myokit.SINGLE_PRECISION, myokit.DOUBLE_PRECISION

    def tune(name, s):
        t0 = time.time()
        best, res = at.autotune(s)
        print(json.dumps({'config': name, 'best': str(best), 'seconds':
                          round(time.time() - t0, 1), 'rates': {
                              str(k): round(v / 1e9, 3)
                              for k, v in res.items()}}), flush=True)

    for label, prec, kw in [('fp32', SP, {}),
                            ('kahan', SP, {'accumulate': 'kahan'}),
                            ('double', SP, {'accumulate': 'double'}),
                            ('ieee', SP, {'fp32_math': 'ieee'}),
                            ('fp64', DP, {})]:
        s, _ = make_sheet(mg.SimulationCUDA, prec, 512, **kw)
        tune('sheet512-' + label, s)
    m = load_model()
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    for label, kw in (('kahan', {'accumulate': 'kahan'}), ('fp32', {})):
        s = mg.SimulationCUDA(m, p, ncells=(2048, 2048), rl=True, **kw)
        s.set_step_size(0.005)
        s.set_paced_cells(nx=4, ny=2048, x=0, y=0)
        tune('sheet2048-' + label, s)
    s, _ = _cables(m, p)
    tune('cables512-kahan', s)
    br = myokit.load_model(os.path.join(
        os.path.dirname(myokit.__file__), 'tests', 'data',
        'beeler-1977-model.mmt'))
    for label, prec, kw in (('fp64', DP, {}),
                            ('kahan', SP, {'accumulate': 'kahan'})):
        s = mg.SimulationCUDA(br, p, ncells=200, precision=prec, **kw)
        s.set_step_size(0.005)
        s.set_conductance(9)
        s.set_paced_cells(5)
        tune('cable200-' + label, s)
    with open(at._cache_path()) as f:
        print(f.read())
    return 0


def profile_case(args):
    """
    Runs the benchmark sheet (--size, --precision, --accumulate) for
    --profile-steps time steps after a short warm-up, for profilers; prints
    one line of launch statistics.
    """
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    prec = myokit.DOUBLE_PRECISION if args.precision == 'double' \
        else myokit.SINGLE_PRECISION
    acc = None if args.accumulate == 'none' else args.accumulate
    if args.profile_adjoint:
        from myokit_gb300 import adjoint as ad
        s, _ = make_sheet(mg.SimulationCUDA, prec, args.size,
                          stage_tiles=not args.no_stage)
        rng = np.random.default_rng(5)
        cells = rng.choice(args.size ** 2, 64, replace=False)
        probes = [(int(c % args.size), int(c // args.size)) for c in cells]
        adj = ad.TissueAdjoint(s, probes, segment_steps=200,
                               min_blocks=args.adj_min_blocks,
                               threads=args.adj_threads or None,
                               guards=args.adj_guards)
        ms = args.profile_steps * 0.005
        out = {}
        for _ in range(2):
            t0 = time.perf_counter()
            v = adj.forward(ms, 0.05)
            t1 = time.perf_counter()
            adj.backward(2 * (v + 80))
            t2 = time.perf_counter()
            s.run(ms, log=['engine.time'], log_interval=0.05)
            t3 = time.perf_counter()
            out = {'adjoint_forward_s': t1 - t0, 'adjoint_backward_s': t2 - t1,
                   'forward_s': t3 - t2,
                   'ratio': (t2 - t0) / (t3 - t2)}
        print(json.dumps(dict(out, size=args.size, steps=args.profile_steps,
                              adj_min_blocks=args.adj_min_blocks,
                              adj_threads=args.adj_threads,
                              guards=args.adj_guards,
                              staged=s._last_kernel.layout is not None)))
        return 0
    s, log = make_sheet(mg.SimulationCUDA, prec, args.size,
                        fields=not args.no_fields,
                        steps_per_launch=args.profile_steps, accumulate=acc,
                        stage_tiles=not args.no_stage)
    ms = args.profile_steps * 0.005
    for _ in range(2):
        s.run(ms, log=log, log_interval=1)
    st = s.last_run_stats()
    k = s._last_kernel
    print(json.dumps({'size': args.size, 'precision': args.precision,
                      'accumulate': args.accumulate,
                      'staged': k.layout is not None,
                      'lazy': bool(k.layout) and k.stage_lazy,
                      'block': k.block[0], 'min_blocks': k.min_blocks,
                      'bytes_per_cell_step': k.bytes_per_cell_step(),
                      'steps': st['cell_steps']
                      // (args.size * args.size), 'launches': st['launches'],
                      'kernel_ms': st['kernel_ms']}))
    return 0


def run_reference(args):
    """--impl reference: the reference kernel on the host cores."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    from myokit_gb300._deps import myokit
    from oracle.refsim import ReferenceCpuSimulation
    cores = os.cpu_count() or 1
    s, log = make_sheet(ReferenceCpuSimulation, myokit.SINGLE_PRECISION,
                        args.size)
    s.set_threads(cores)
    ncell = args.size * args.size
    # Bench step: a bounded sample sized to ~2 s of CPU time (calibrated
    # after a first run, which also builds the reference kernel)
    s.run(0.05, log=log, log_interval=1)
    t0 = time.perf_counter()
    s.run(0.05, log=log, log_interval=1)
    rate0 = ncell * 10 / max(time.perf_counter() - t0, 1e-9)
    nsteps = int(max(10, min(2000, rate0 * 2.0 / ncell)))
    dur = nsteps * 0.005
    for _ in range(args.warmup):
        s.run(dur, log=log, log_interval=1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.run(dur, log=log, log_interval=1)
    dt = time.perf_counter() - t0
    value = ncell * nsteps * args.steps / dt
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT,
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': dt * 1000 / args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic (seeded fields and probes)',
        'config': config(args, 'reference kernel on host CPU, %d time steps'
                         ' per step' % nsteps),
        'cpu_baseline': {
            'value': value, 'unit': UNIT, 'cores': cores,
            'kind': 'reference',
            'sample': '%d time steps of the %dx%d sheet per step' % (
                nsteps, args.size, args.size)},
        'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg

    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')

    def barrier():
        if dist is not None:
            dist.barrier(device_ids=[local])
        torch.cuda.synchronize()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device='cuda')
    ncell = args.size * args.size
    nsteps_per = int(round(args.step_ms / 0.005))

    # --- single precision (headline) -------------------------------------
    s, log = make_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION,
                        args.size, seed=rank, device=local)
    logs32 = []
    for _ in range(args.warmup):
        logs32.append(s.run(args.step_ms, log=log, log_interval=1))
    kernel = s._last_kernel
    sampler = ClockSampler(args.clocks_csv)
    sampler.start()
    barrier()
    dev_ms = 0.0
    wall = 0.0
    launches = 0
    step_launches = 0
    cell_steps = 0
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        logs32.append(s.run(args.step_ms, log=log, log_interval=1))
        wall += time.perf_counter() - t0
        st = s.last_run_stats()
        dev_ms += st['kernel_ms']
        launches += st['all_launches']
        step_launches += st['launches']
        cell_steps += st['cell_steps']
    barrier()
    clocks = sampler.stop()
    # Replicas: the slowest rank's times, every rank's cell-steps
    from myokit_gb300.replicas import combine
    dev_ms, wall, total_cell_steps = combine(
        dev_ms, wall, cell_steps, world, dist, 'cuda')
    value = total_cell_steps / (dev_ms / 1000.0)
    e2e_value = total_cell_steps / wall

    # Bytes crossing the host boundary per bench step (public run() call)
    nstate = s._nstate
    h2d = ncell * nstate * 8 + ncell * 2 * 8 + nsteps_per * 32
    d2h = ncell * nstate * 8 + (len(log) - 1) * int(args.step_ms) * 8

    # Roofline of the tissue kernel (algorithmic bytes per launch)
    bpcs = kernel.bytes_per_cell_step()
    avg_launch_s = (dev_ms / 1000.0) / max(step_launches, 1)
    per_launch_cs = cell_steps / max(step_launches, 1)
    achieved = bpcs * per_launch_cs / avg_launch_s / 1e9
    peak, peak_kind = read_peaks()
    traffic = read_traffic()
    traffic_per_launch = None
    if traffic and traffic.get('bytes_per_cell_step'):
        traffic_per_launch = traffic['bytes_per_cell_step'] * per_launch_cs
    # Compute roofline: FP32 lanes x 2 flops x SM clock under load
    sm_mhz = clocks['sm_mhz'] if clocks else 1900.0
    # Instruction-issue roofline (what binds the L2-resident sheet): warp
    # instructions per cell-step from the committed ncu capture, against
    # 4 warp schedulers x 152 SMs issuing one instruction per clock
    issue = None
    if traffic and traffic.get('warp_instructions_per_cell_step'):
        ach = traffic['warp_instructions_per_cell_step'] * value / world
        peak_i = 4 * 152 * sm_mhz * 1e6
        issue = {'unit': 'warp instructions/s', 'achieved': ach,
                 'peak': peak_i, 'frac': ach / peak_i,
                 'warp_instructions_per_cell_step':
                     traffic['warp_instructions_per_cell_step'],
                 'source': traffic.get('source')}
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    flops = kernel.flops_per_cell_step() * value / world / 1e12

    # --- double precision, same sheet --------------------------------------
    fp64 = None
    dv = None
    if args.fp64_steps > 0 and rank == 0:
        s64, _ = make_sheet(mg.SimulationCUDA, myokit.DOUBLE_PRECISION,
                            args.size, seed=rank, device=local)
        logs64 = []
        d64 = 0.0
        n64 = 0
        nrun = args.warmup + args.fp64_steps
        for i in range(nrun):
            logs64.append(s64.run(args.step_ms, log=log, log_interval=1))
            if i >= args.warmup:
                st = s64.last_run_stats()
                d64 += st['kernel_ms']
                n64 += st['cell_steps']
        fp64 = {'value': n64 / (d64 / 1000.0), 'unit': UNIT,
                'steps': args.fp64_steps, 'warmup': args.warmup}
        worst = 0.0
        for a, b in zip(logs32[:nrun], logs64):
            for k in a.keys():
                if k == 'engine.time':
                    continue
                worst = max(worst, float(np.max(np.abs(
                    np.asarray(a[k], dtype=float) -
                    np.asarray(b[k], dtype=float)))))
        dv = {'max_abs_dV_mV': worst,
              'window_ms': nrun * args.step_ms,
              'against': 'this sheet in double precision on the GPU'}
        fp64['speedup_fp32_over_fp64'] = value / world / fp64['value']

    # --- single precision with FP64 / Kahan accumulation --------------------
    variants = {}
    if args.variant_steps > 0 and rank == 0:
        for vname, kw in VARIANTS:
            sv, _ = make_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION,
                               args.size, seed=rank, device=local, **kw)
            dms = 0.0
            ncs = 0
            for i in range(args.warmup + args.variant_steps):
                flush.fill_(1)
                torch.cuda.synchronize()
                sv.run(args.step_ms, log=log, log_interval=1)
                if i >= args.warmup:
                    st = sv.last_run_stats()
                    dms += st['kernel_ms']
                    ncs += st['cell_steps']
            v = ncs / (dms / 1000.0)
            variants[vname] = {
                'value': v, 'unit': UNIT,
                'accumulated_states': [x.qname()
                                       for x in sv.accumulated_states()],
                'bytes_per_cell_step': sv._last_kernel.bytes_per_cell_step(),
                'speedup_over_fp64': (v / fp64['value']) if fp64 else None,
            }

    accuracy = {'fp32_vs_fp64_bench_sheet': dv}
    if args.accuracy_ms > 0 and rank == 0:
        accuracy.update(accuracy_runs(args, local))

    adj = None
    if args.adjoint_ms > 0 and rank == 0:
        adj = adjoint_runs(args, local)

    others = {}
    wanted = [c for c in args.configs.split(',') if c and c != 'none']
    if rank == 0:
        for c in wanted:
            others[c] = {'c1': config_c1, 'c3': config_c3,
                         'c5': config_c5}[c](args, local)

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        cpu = cpu_baseline(args, myokit.SINGLE_PRECISION, args.cpu_seconds)

    if rank != 0:
        return 0
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': dev_ms / args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic (seeded fields and probes)',
        'config': config(args, 'sheet %dx%d, %d time steps per step' % (
            args.size, args.size, nsteps_per)),
        'e2e': {'value': e2e_value, 'unit': UNIT, 'h2d_bytes_per_step': h2d,
                'd2h_bytes_per_step': d2h},
        'gpu_launches': launches,
        'roofline': {
            'bound': 'hbm', 'achieved': achieved, 'peak': peak,
            'unit': 'GB/s', 'frac': achieved / peak,
            'traffic': traffic_per_launch,
            'peak_source': peak_kind,
            'bytes_per_cell_step': bpcs,
            'compute': {
                'unit': 'TFLOP/s', 'achieved': flops, 'peak': fp32_peak,
                'frac': flops / fp32_peak,
                'flops_per_cell_step': kernel.flops_per_cell_step(),
                'transcendentals_per_cell_step': kernel.census.trans,
                'peak_source': 'FP32 lanes x 2 x median SM clock'},
            'issue': issue,
        },
        'fp64': fp64,
        'variants': variants,
        'accuracy': accuracy,
        'adjoint': adj,
        'other_configs': others,
        'clocks': clocks,
        'cpu_baseline': cpu,
    }
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    if args.profile:
        return profile_case(args)
    if args.tune:
        return tune_configs(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
