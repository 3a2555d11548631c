#!/usr/bin/env python3
"""
Headline benchmark: cell-steps/s of the fused tissue step on one GB300.

Headline workload (the large-sheet configuration):
  a 2048 x 2048 sheet of the 48-state Decker 2009 canine model (standing in
  for O'Hara-Rudy 2011 endo, whose model file is not available), Rush-Larsen
  on, dt = 0.005 ms, single precision with Kahan-compensated V and
  concentrations; S1 on the 4 left columns at t = 0 (2 ms, level 1), S2 on
  the lower-left quadrant at t = 320 ms; the full V frame every 5 ms
  recorded in a device buffer.

One bench step = ``run_frames(step_ms, 5)`` of that sheet (2000 time steps
at the default 10 ms). ``value`` is cell-steps per second of device time
with the state resident in HBM (CUDA events on the library's stream around
the kernel launches); ``e2e`` is the same metric through the public call,
with the host state uploaded, and the frames and the final state read back
to the host, every step. The state (805 MB, plus 134 MB of compensation
planes) is far larger than L2, so no flush is needed between steps.

Also reported: the plain FP64 path on the same sheet; max|dV|, activation
and APD90 errors of the headline precision against FP64 at full size (the
S1 phase, and a window after S2); the 512 x 512 sheet (the medium
configuration, L2-resident, bound by instruction issue) in every precision
mode; the adjoint; the 200-cell FP64 cable; the 512 batched cables; and the
reference's CPU rate on the host cores.

--impl reference times the reference's own kernel (the OpenCL C that
myokit's SimulationOpenCL renders for this model, compiled for the host CPU
and driven through the reference's unmodified Python layer by the oracle's
restatement of its step loop) on all host cores, on the same configuration.
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
UNIT = 'cell-steps/s'
FRAME_MS = 5.0      # the headline sheet's frame interval
S2_AT = 320.0       # S2 time of the headline protocol

# Single precision variants of the 512 x 512 sheet: FP64 or compensated
# accumulation of V and the concentrations, and IEEE division
VARIANTS = [
    ('fp32+double', {'accumulate': 'double'}),
    ('fp32+kahan', {'accumulate': 'kahan'}),
    ('fp32-ieee-div', {'fp32_math': 'ieee'}),
]


def parse():
    p = argparse.ArgumentParser(description=__doc__.split('\n')[1])
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=10)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    p.add_argument('--size', type=int, default=2048,
                   help='edge of the headline sheet')
    p.add_argument('--step-ms', type=float, default=10.0,
                   help='simulated time per bench step')
    p.add_argument('--fp64-ms', type=float, default=1.0,
                   help='simulated time of the timed FP64 run of the'
                        ' headline sheet (0 = skip)')
    p.add_argument('--s1-ms', type=float, default=S2_AT,
                   help='window of the full-size precision comparison before'
                        ' S2 (0 = skip the comparison)')
    p.add_argument('--s2-ms', type=float, default=10.0,
                   help='window of the full-size precision comparison after'
                        ' S2 (FP64 on the whole sheet; 0 = skip)')
    p.add_argument('--sheet512-steps', type=int, default=5,
                   help='timed steps of the 512 x 512 sheet (0 = skip it)')
    p.add_argument('--fp64-steps', type=int, default=2,
                   help='timed double precision steps of the 512 x 512'
                        ' sheet (0 = skip)')
    p.add_argument('--variant-steps', type=int, default=3,
                   help='timed steps of the 512 x 512 accumulation variants')
    p.add_argument('--accuracy-ms', type=float, default=400.0,
                   help='simulated time of the 128 x 128 and 24 x 24'
                        ' precision comparisons (0 = skip)')
    p.add_argument('--adjoint-ms', type=float, default=300.0,
                   help='simulated time of the adjoint measurement (the'
                        ' 256 x 256 adjoint configuration runs 300 ms;'
                        ' 0 = skip)')
    p.add_argument('--configs', default='c1,c3',
                   help='other configurations to time: comma list of c1'
                        ' (200-cell FP64 cable), c3 (512 batched cables), or'
                        ' none')
    p.add_argument('--full', action='store_true',
                   help='also run every configuration at its full length:'
                        ' the batched cables for 2000 ms, the adjoint over'
                        ' 300 ms, the 2048x2048 S1-S2 protocol for 1000 ms')
    p.add_argument('--profile', action='store_true',
                   help='run one small sheet case for a profiler and exit')
    p.add_argument('--tune-only', default='',
                   help='with --tune: a comma list of the configurations'
                        ' to tune (sheet512-fp32, cable200-fp64, ...)')
    p.add_argument('--tune', action='store_true',
                   help='autotune the launch shape of every benchmark'
                        ' configuration, print the timings and the table'
                        ' (the format of myokit_gb300/tuned.json), exit')
    p.add_argument('--profile-steps', type=int, default=40)
    p.add_argument('--no-fields', action='store_true',
                   help='with --profile: a sheet without scalar fields (the'
                        ' 2048x2048 S1-S2 configuration)')
    p.add_argument('--profile-cable', action='store_true',
                   help='with --profile: the 200-cell Beeler-Reuter cable'
                        ' (--precision, tuned launch shape) instead')
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
                   help='target CPU time of the cpu_baseline sample')
    p.add_argument('--ref-seconds', type=float, default=5.0,
                   help='target CPU time of one --impl reference step')
    return p.parse_args()


def load_model():
    from myokit_gb300._deps import myokit
    path = os.path.join(os.path.dirname(myokit.__file__), 'tests', 'data',
                        'decker-2009.mmt')
    return myokit.load_model(path)


def make_sheet(cls, precision, size, seed=0, fields=True, **kw):
    """The 512 x 512 benchmark sheet (medium configuration, any size);
    returns (simulation, log variable list)."""
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


def make_s1_sheet(cls, precision, n, **kw):
    """The headline sheet before S2: n x n, no fields, S1 on the 4 left
    columns at t = 0 (a 1 Hz block train of 2 ms pulses, level 1)."""
    from myokit_gb300._deps import myokit
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = cls(load_model(), p, ncells=(n, n), precision=precision, rl=True,
            **kw)
    s.set_step_size(0.005)
    s.set_paced_cells(nx=4, ny=n, x=0, y=0)
    return s


def make_s1_cable(cls, precision, n, **kw):
    """One row of the S1 sheet as a 1D cable (gx = 10, the sheet's default;
    the first 4 cells paced). Every row of the S1 sheet equals it."""
    from myokit_gb300._deps import myokit
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = cls(load_model(), p, ncells=n, precision=precision, rl=True, **kw)
    s.set_step_size(0.005)
    s.set_conductance(10)
    s.set_paced_cells(4)
    return s


def apply_s2(s, n):
    """Switches a sheet at t = 320 ms to the S2 stimulus: the lower-left
    quadrant paced once, at 320 ms (2 ms, level 1)."""
    from myokit_gb300._deps import myokit
    s.set_paced_cells(nx=n // 2, ny=n // 2, x=0, y=0)
    p2 = myokit.Protocol()
    p2.schedule(level=1, start=S2_AT, duration=2)
    s.set_protocol(p2)


def config(args):
    """The headline configuration (identical for both arms)."""
    n = args.size
    return {
        'workload': 'sheet %dx%d, S1-S2 protocol, full V frame every 5 ms'
                    ' to a device buffer, %d time steps per step' % (
                        n, n, int(round(args.step_ms / 0.005))),
        'model': 'decker-2009 (48 states; stands in for O\'Hara-Rudy 2011'
                 ' endo, whose model file is unavailable)',
        'grid': [n, n], 'rl': True, 'dt_ms': 0.005,
        'step_ms': args.step_ms,
        'paced': 'left 4 columns, S1 at 0 ms (2 ms, level 1); lower-left'
                 ' quadrant, S2 at 320 ms',
        'fields': 'none',
        'fp32_math': 'fast (single precision divisions within the 2.5 ulp'
                     ' that OpenCL allows; exp, log and pow accurate)',
        'log': 'full V frame every 5 ms (device buffer)',
        'l2': ('inputs larger than L2 (state %.0f MB), no flush' if
               n * n * 48 * 4 > 129e6 else
               'state of %.1f MB, smaller than L2, not flushed') % (
                   n * n * 48 * 4 / 1e6),
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


def read_traffic(workload):
    """Per-cell-step DRAM bytes and warp instructions of the tissue kernel
    on one workload, from the committed ncu summaries, or None."""
    path = os.path.join(ROOT, 'profiles', 'tissue_step_traffic.json')
    try:
        with open(path) as f:
            return json.load(f).get(workload)
    except (OSError, ValueError):
        return None


def sm_count(device):
    import torch
    return torch.cuda.get_device_properties(device).multi_processor_count


def issue_roofline(traffic, value, sm_mhz, n_sm):
    """Instruction-issue roofline: warp instructions per cell-step (from an
    ncu capture) against 4 schedulers per SM issuing one per clock."""
    if not traffic or not traffic.get('warp_instructions_per_cell_step'):
        return None
    ach = traffic['warp_instructions_per_cell_step'] * value
    peak = 4 * n_sm * sm_mhz * 1e6
    return {'unit': 'warp instructions/s', 'achieved': ach, 'peak': peak,
            'frac': ach / peak,
            'warp_instructions_per_cell_step':
                traffic['warp_instructions_per_cell_step'],
            'source': traffic.get('source')}


class _ChunkClock(object):
    """
    Progress reporter for the reference's run(): the reference calls
    update() after every sim_step, so the times between calls are the
    times of its step-loop chunks. After a calibration chunk it sets the
    chunk length for about ``seconds`` of CPU time, and it cancels the run
    after ``n_warm + n_timed`` further chunks.
    """
    def __init__(self, backend, ncell, seconds, n_warm, n_timed):
        self.be = backend
        self.ncell = ncell
        self.seconds = seconds
        self.n_warm = n_warm
        self.n_timed = n_timed
        self.marks = []
        self.steps = None

    def enter(self, msg=None):
        self.marks = [time.perf_counter()]

    def exit(self):
        pass

    def update(self, progress):
        self.marks.append(time.perf_counter())
        if len(self.marks) == 2:
            dt = self.marks[1] - self.marks[0]
            rate = self.ncell * self.be.chunk_steps / max(dt, 1e-9)
            self.steps = int(max(1, min(20000, round(
                rate * self.seconds / self.ncell))))
            self.be.chunk_steps = self.steps
            return True
        return len(self.marks) < 2 + self.n_warm + self.n_timed


def reference_rate(n, precision, seconds, n_warm, n_timed, cores=None):
    """
    Times the reference's kernel on the host cores on the headline sheet
    through the reference's own run() (myokit.SimulationOpenCL with the
    oracle's CPU backend). The chunks of its step loop are timed after its
    per-run set-up (kernel rendering, Python-list marshalling of the state),
    which is left out, to the reference's advantage. Returns (cell-steps/s,
    time steps per chunk, chunk seconds, threads).
    """
    from myokit_gb300._deps import myokit
    from oracle.refsim import ReferenceCpuSimulation
    cores = cores or os.cpu_count() or 1
    s = make_s1_sheet(ReferenceCpuSimulation, precision, n)
    s.set_threads(cores)
    be = s._sim
    be.chunk_steps = 2          # the calibration chunk

    class Clock(_ChunkClock, myokit.ProgressReporter):
        pass
    clock = Clock(be, n * n, seconds, n_warm, n_timed)
    try:
        s.run(1000, log=['engine.time'], log_interval=FRAME_MS,
              progress=clock)
    except myokit.SimulationCancelledError:
        pass
    be.chunk_steps = None
    times = np.diff(clock.marks)[1 + n_warm:1 + n_warm + n_timed]
    rate = n * n * clock.steps * len(times) / float(np.sum(times))
    return rate, clock.steps, [float(x) for x in times], cores


def cpu_baseline(args):
    """The reference's CPU rate on a bounded sample of the headline sheet."""
    from myokit_gb300._deps import myokit
    rate, steps, times, cores = reference_rate(
        args.size, myokit.SINGLE_PRECISION, args.cpu_seconds, 0, 1)
    return {
        'value': rate, 'unit': UNIT, 'cores': cores, 'kind': 'reference',
        'sample': '%d time steps (%.3g ms) of the %dx%d sheet in single'
                  ' precision (the reference has no compensated mode),'
                  ' timed inside one run() of the reference after its'
                  ' per-run set-up; the reference-rendered OpenCL kernel'
                  ' compiled as C (gcc -O2, OpenMP, %d threads) with the'
                  ' oracle host loop' % (steps, steps * 0.005, args.size,
                                         args.size, cores),
        'seconds': sum(times),
    }


def run_reference(args):
    """--impl reference: the reference kernel on the host cores."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    from myokit_gb300._deps import myokit
    rate, steps, times, cores = reference_rate(
        args.size, myokit.SINGLE_PRECISION, args.ref_seconds, args.warmup,
        args.steps)
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': rate, 'unit': UNIT,
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1000 * float(np.mean(times)),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32', 'data': 'synthetic (seeded probes)',
        'precision': 'FP32 (the reference has no compensated mode)',
        'config': config(args),
        'cpu_baseline': {
            'value': rate, 'unit': UNIT, 'cores': cores,
            'kind': 'reference',
            'sample': 'each step: %d time steps (%.3g ms) of the %dx%d'
                      ' sheet, one chunk of the reference step loop inside'
                      ' one run() of the reference (its per-run kernel'
                      ' rendering and state marshalling are outside the'
                      ' timed chunks; no frames are logged)' % (
                          steps, steps * 0.005, args.size, args.size)},
        'e2e': {'value': rate, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))
    return 0


def c5_accuracy(args, device):
    """
    Max |dV|, activation-time and APD90 errors of the headline precision
    (FP32 + Kahan) against FP64, on the full 2048 x 2048 sheet.

    - S1 phase (0 to 320 ms): the sheet paced along its whole left edge has
      identical rows, so its FP64 solution is a 2048-cell FP64 cable (the
      FP64 sheet's rows equal the cable bit for bit; checked by the fp64
      block). 256 probe traces every 0.1 ms against the cable's traces at
      their x, and the whole V plane at 320 ms against the cable's V.
    - After S2 (320 ms on): the FP64 sheet itself, started from the FP64
      cable state broadcast to every row, against the FP32 + Kahan sheet
      continuing from its own state; probe traces and the whole V plane at
      the end of the window.
    """
    import torch
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    from myokit_gb300 import metrics
    SP, DP = myokit.SINGLE_PRECISION, myokit.DOUBLE_PRECISION
    n = args.size
    rng = np.random.default_rng(7)
    cells = sorted(rng.choice(n * n, 256, replace=False))
    xy = [(int(c % n), int(c // n)) for c in cells]
    keys = ['%d.%d.membrane.V' % p for p in xy]
    log = ['engine.time'] + keys
    out = {}

    # S1 phase
    t1 = args.s1_ms
    s32 = make_s1_sheet(mg.SimulationCUDA, SP, n, accumulate='kahan',
                        device=device)
    d32 = s32.run(t1, log=log, log_interval=0.1)
    c64 = make_s1_cable(mg.SimulationCUDA, DP, n, device=device)
    xs = sorted(set(x for x, _ in xy))
    dc = c64.run(t1, log=['engine.time'] + ['%d.membrane.V' % x
                                            for x in xs], log_interval=0.1)
    t = np.asarray(dc['engine.time'])
    # the single precision log holds the float32 rounding of the times
    assert np.array_equal(np.asarray(d32['engine.time']),
                          t.astype(np.float32))
    got = {k: np.asarray(d32[k]) for k in keys}
    ref = {k: np.asarray(dc['%d.membrane.V' % x]) for k, (x, _) in
           zip(keys, xy)}
    res = metrics.compare(t, got, ref)
    i_vm = s32._vm.index()
    ns = s32._nstate
    v32 = s32.state_array().reshape(n, n, ns)[:, :, i_vm]
    st64 = c64.state_array().reshape(n, ns)
    res['full_sheet_max_abs_dV_mV_at_end'] = float(
        np.max(np.abs(v32 - st64[None, :, i_vm])))
    res['activated_traces'] = int(sum(
        np.isfinite(metrics.activation_time(t, ref[k])) for k in keys))
    out['s1_phase'] = dict(
        res, window_ms=[0.0, t1], probes=len(keys), log_interval_ms=0.1,
        reference='FP64 %d-cell cable on the GPU (every row of the S1'
                  ' sheet equals it)' % n)
    del v32

    # After S2
    if args.s2_ms > 0 and abs(t1 - S2_AT) < 1e-9:
        s64 = make_s1_sheet(mg.SimulationCUDA, DP, n, device=device)
        s64.set_state(np.tile(st64.reshape(-1), n))
        s64.set_time(t1)
        for s in (s32, s64):
            apply_s2(s, n)
        d32 = s32.run(args.s2_ms, log=log, log_interval=0.1)
        d64 = s64.run(args.s2_ms, log=log, log_interval=0.1)
        t = np.asarray(d64['engine.time'])
        res = metrics.compare(t, {k: np.asarray(d32[k]) for k in keys},
                              {k: np.asarray(d64[k]) for k in keys})
        v32 = s32.state_array().reshape(n, n, ns)[:, :, i_vm]
        v64 = s64.state_array().reshape(n, n, ns)[:, :, i_vm]
        res['full_sheet_max_abs_dV_mV_at_end'] = float(
            np.max(np.abs(v32 - v64)))
        res['s2_activated_fraction_at_end'] = float(np.mean(
            (v64[:n // 2, :n // 2] > -40)))
        out['after_s2'] = dict(
            res, window_ms=[t1, t1 + args.s2_ms], probes=len(keys),
            log_interval_ms=0.1,
            reference='FP64 %dx%d sheet on the GPU, started from the FP64'
                      ' cable state at %g ms' % (n, n, t1))
        del s64, v64, v32
    del s32, c64
    torch.cuda.empty_cache()
    return out


def c5_fp64(args, device, value):
    """
    The plain FP64 path on the headline sheet, timed over args.fp64_ms;
    its rows are checked against the FP64 cable bit for bit.
    """
    import torch
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    DP = myokit.DOUBLE_PRECISION
    n = args.size
    s64 = make_s1_sheet(mg.SimulationCUDA, DP, n, device=device)
    s64.run(0.05, log=['engine.time'], log_interval=1)
    s64.run(args.fp64_ms, log=['engine.time'], log_interval=1)
    st = s64.last_run_stats()
    v64 = st['cell_steps'] / (st['kernel_ms'] / 1000)
    x = s64.state_array().reshape(n, n, -1)
    del s64
    c = make_s1_cable(mg.SimulationCUDA, DP, n, device=device)
    c.run(0.05, log=['engine.time'], log_interval=1)
    c.run(args.fp64_ms, log=['engine.time'], log_interval=1)
    rows = bool(np.array_equal(x, np.broadcast_to(
        c.state_array().reshape(1, n, -1), x.shape)))
    del x
    torch.cuda.empty_cache()
    return {'value': v64, 'unit': UNIT, 'window_ms': args.fp64_ms,
            'speedup_fp32_kahan_over_fp64': value / v64,
            'rows_equal_fp64_cable': rows}


def c5_full(args, device):
    """The whole 1000 ms S1-S2 protocol of the headline sheet (--full)."""
    import torch
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    n = args.size
    s = make_s1_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION, n,
                      accumulate='kahan', device=device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, f1 = s.run_frames(S2_AT, FRAME_MS)
    ms = s.last_run_stats()['kernel_ms']
    apply_s2(s, n)
    _, f2 = s.run_frames(1000 - S2_AT, FRAME_MS)
    ms += s.last_run_stats()['kernel_ms']
    wall = time.perf_counter() - t0
    frames = torch.cat([f1, f2])
    steps = 200000
    out = {'window_ms': 1000, 'frames': int(frames.shape[0]),
           'frame_bytes': int(frames[0].numel() * frames.element_size()),
           'value': n * n * steps / (ms / 1000),
           'e2e_frames_on_device': n * n * steps / wall, 'unit': UNIT,
           'final_v_range_mV': [float(frames[-1].min()),
                                float(frames[-1].max())],
           'activated_fraction_final': float(
               (frames[-1] > -40).float().mean())}
    del s, frames, f1, f2
    torch.cuda.empty_cache()
    return out


def sheet512_runs(args, device, n_sm):
    """
    The 512 x 512 sheet (medium configuration: GKr/GNa lognormal fields,
    V at 256 probes every 1 ms): FP32 device and end-to-end rates with L2
    flushed between steps, its instruction-issue roofline (the state is
    L2-resident, so issue binds), FP64 on the same sheet, and the FP32
    accumulation and division variants.
    """
    import torch
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    SP, DP = myokit.SINGLE_PRECISION, myokit.DOUBLE_PRECISION
    size = 512
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    out = {'grid': [size, size], 'step_ms': args.step_ms,
           'fields': 'GKr, GNa x lognormal(0, 0.2), seed 0',
           'log': 'V at 256 probes every 1 ms',
           'l2': 'flushed between timed steps (256 MiB write)'}

    def timed(s, log, steps, warm):
        dms, wall, ncs, logs = 0.0, 0.0, 0, []
        for i in range(warm + steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            logs.append(s.run(args.step_ms, log=log, log_interval=1))
            if i >= warm:
                wall += time.perf_counter() - t0
                st = s.last_run_stats()
                dms += st['kernel_ms']
                ncs += st['cell_steps']
        return ncs / (dms / 1000), ncs / wall, logs

    s, log = make_sheet(mg.SimulationCUDA, SP, size, device=device)
    value, e2e, logs32 = timed(s, log, args.sheet512_steps, 3)
    k = s._last_kernel
    peak, kind = read_peaks()
    bpcs = k.bytes_per_cell_step()
    traffic = read_traffic('sheet512_fp32')
    out.update({'precision': 'fp32', 'fp32_math': s._fp32_math,
                'value': value, 'e2e': e2e, 'unit': UNIT})
    out['roofline'] = {
        'bound': 'issue',
        'issue': None, 'hbm_equivalent': {
            'bytes_per_cell_step': bpcs, 'achieved': value * bpcs / 1e9,
            'peak': peak, 'unit': 'GB/s', 'peak_source': kind,
            'frac': value * bpcs / 1e9 / peak,
            'dram_bytes_per_cell_step':
                traffic and traffic.get('bytes_per_cell_step')}}
    out['_issue_inputs'] = (traffic, value)
    del s
    if args.fp64_steps > 0:
        s64, _ = make_sheet(mg.SimulationCUDA, DP, size, device=device)
        v64, _, logs64 = timed(s64, log, args.fp64_steps, 3)
        worst = 0.0
        for a, b in zip(logs32, logs64):
            for key in a.keys():
                if key == 'engine.time':
                    continue
                worst = max(worst, float(np.max(np.abs(
                    np.asarray(a[key], dtype=float) -
                    np.asarray(b[key], dtype=float)))))
        out['fp64'] = {'value': v64, 'unit': UNIT,
                       'speedup_fp32_over_fp64': value / v64,
                       'max_abs_dV_fp32_vs_fp64_mV': worst,
                       'dV_window_ms': len(logs64) * args.step_ms}
        del s64
    variants = {}
    if args.variant_steps > 0:
        for vname, kw in VARIANTS:
            sv, _ = make_sheet(mg.SimulationCUDA, SP, size, device=device,
                               **kw)
            v, _, _ = timed(sv, log, args.variant_steps, 3)
            variants[vname] = {
                'value': v, 'unit': UNIT,
                'accumulated_states': [x.qname()
                                       for x in sv.accumulated_states()],
                'bytes_per_cell_step': sv._last_kernel.bytes_per_cell_step()}
            del sv
    out['variants'] = variants
    del flush
    torch.cuda.empty_cache()
    return out


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
        'max_rel_err': worst, 'loss': L, 'sample': entries[:4],
        'precision': 'fp64 forward and adjoint (the precision that meets'
                     ' the 1e-4 bar)'}

    # The adjoint configuration's precision (FP32 with FP64 V and
    # concentrations) against the same FP64 finite differences
    s, _ = make_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION, n,
                      seed=0, device=device, accumulate='double')
    adj = ad.TissueAdjoint(s, probes, segment_steps=200)
    L32, g32 = adj.loss_and_gradient(fd_ms, target, 1.0)
    errs = []
    for e in entries:
        ix, iy = e['cell']
        a = g32[e['field']][iy, ix]
        errs.append(abs(a - e['fd']) / max(abs(e['fd']), 1e-12 * abs(L)))
    out['fd_check_sheet64_fp32_double'] = {
        'window_ms': fd_ms, 'entries': len(errs),
        'max_rel_err': float(max(errs)),
        'median_rel_err': float(np.median(errs)), 'loss': L32,
        'precision': 'fp32 forward and adjoint with FP64 V and'
                     ' concentrations, against central differences of the'
                     ' FP64 forward'}
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
        k = s._last_kernel
        out[name] = {'value': 200 * 200000 / (st['kernel_ms'] / 1000),
                     'e2e': 200 * 200000 / wall, 'unit': UNIT,
                     'wall_s': wall, 'block': list(k.block),
                     'warps_per_tile': k.split,
                     'ctas_per_cluster': k.split_cl}
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
        log = ['engine.time'] + batch.cable_log_keys(
            len(batch.lengths) - 1)[-1:]
        # Warm-up with the same log list: the first run with a new list
        # prepares its log template (myokit's prepare_log, 0.3 s here)
        s.run(2, log=log, log_interval=1)
        t0 = time.perf_counter()
        d = s.run(window, log=log, log_interval=1)
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


def tune_configs(args):
    """
    Runs the autotuner on each benchmark configuration (or those
    --tune-only names): the 512 x 512 sheet in every precision mode, the
    2048 x 2048 sheet (FP32 and Kahan), the 512 batched cables, the 200-cell
    cable and the 2048-cell FP64 cable. Results go to the user cache
    (MYOKIT_GB300_CACHE or ~/.cache/myokit_gb300); the table is printed.
    """
    from myokit_gb300._deps import myokit
    import myokit_gb300 as mg
    from myokit_gb300 import autotune as at
    SP, DP = myokit.SINGLE_PRECISION, myokit.DOUBLE_PRECISION

    only = set(filter(None, (args.tune_only or '').split(',')))

    def tune(name, s):
        if only and name not in only:
            return
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
                            ('kahan', SP, {'accumulate': 'kahan'}),
                            ('fp32', SP, {})):
        s = mg.SimulationCUDA(br, p, ncells=200, precision=prec, **kw)
        s.set_step_size(0.005)
        s.set_conductance(9)
        s.set_paced_cells(5)
        tune('cable200-' + label, s)
    # The FP64 reference of the S1 phase: a row of the 2048 x 2048 sheet
    tune('cable2048-fp64', make_s1_cable(mg.SimulationCUDA, DP, 2048))
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
    if args.profile_cable:
        path = os.path.join(os.path.dirname(myokit.__file__), 'tests',
                            'data', 'beeler-1977-model.mmt')
        p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
        s = mg.SimulationCUDA(myokit.load_model(path), p, ncells=200,
                              precision=prec, accumulate=acc)
        s.set_step_size(0.005)
        s.set_conductance(9)
        s.set_paced_cells(5)
        s._steps_per_launch = args.profile_steps
        ms = args.profile_steps * 0.005
        for _ in range(2):
            s.run(ms, log=['engine.time'], log_interval=1)
        st = s.last_run_stats()
        k = s._last_kernel
        print(json.dumps({'cable': 200, 'precision': args.precision,
                          'block': k.block[0], 'split': k.split,
                          'launches': st['launches'],
                          'kernel_ms': st['kernel_ms'],
                          'cell_steps_per_s': st['cell_steps'] /
                          (st['kernel_ms'] / 1000)}))
        return 0
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


def guarded(fn, *a):
    """fn(*a), or {'error': ...} (traceback on stderr) if it raises."""
    import traceback
    try:
        return fn(*a)
    except Exception as e:
        traceback.print_exc()
        return {'error': '%s: %s' % (type(e).__name__, e)}


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

    n = args.size
    ncell = n * n
    n_sm = sm_count(local)
    nsteps_per = int(round(args.step_ms / 0.005))

    # --- headline: FP32 + Kahan sheet, frames on the device ---------------
    s = make_s1_sheet(mg.SimulationCUDA, myokit.SINGLE_PRECISION, n,
                      accumulate='kahan', device=local)
    s2_applied = [None]

    def step():
        # S2 switches on at the first step boundary at or after 320 ms
        if s2_applied[0] is None and s.time() >= S2_AT - 1e-9:
            apply_s2(s, n)
            s2_applied[0] = s.time()
        return s.run_frames(args.step_ms, FRAME_MS)

    for _ in range(args.warmup):
        step()
    kernel = s._last_kernel
    sampler = ClockSampler(args.clocks_csv)
    sampler.start()
    barrier()
    dev_ms = 0.0
    wall = 0.0
    launches = 0
    step_launches = 0
    cell_steps = 0
    frame_bytes = 0
    n_frames = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        tt, frames = step()
        host = frames.cpu()         # the step's result, read back
        wall += time.perf_counter() - t0
        st = s.last_run_stats()
        dev_ms += st['kernel_ms']
        launches += st['all_launches']
        step_launches += st['launches']
        cell_steps += st['cell_steps']
        frame_bytes += host.numel() * host.element_size() + 8 * len(tt)
        n_frames += len(tt)
        del host, frames
    barrier()
    clocks = sampler.stop()
    t_end = s.time()
    del s
    torch.cuda.empty_cache()
    # Replicas: the slowest rank's times, every rank's cell-steps
    from myokit_gb300.replicas import combine
    dev_ms, wall, total_cell_steps = combine(
        dev_ms, wall, cell_steps, world, dist, 'cuda')
    value = total_cell_steps / (dev_ms / 1000.0)
    e2e_value = total_cell_steps / wall

    # Bytes crossing the host boundary per bench step: the state up (the
    # public call keeps the state on the host between calls, as the
    # reference does) and the step schedule; the state and frames down
    nstate = 48
    h2d = ncell * nstate * 8 + nsteps_per * 40
    d2h = ncell * nstate * 8 + frame_bytes // max(args.steps, 1)

    # Roofline of the tissue kernel (algorithmic bytes per launch)
    bpcs = kernel.bytes_per_cell_step()
    avg_launch_s = (dev_ms / 1000.0) / max(step_launches, 1)
    per_launch_cs = cell_steps / max(step_launches, 1)
    achieved = bpcs * per_launch_cs / avg_launch_s / 1e9
    peak, peak_kind = read_peaks()
    traffic = read_traffic('sheet2048_kahan')
    traffic_per_launch = None
    if traffic and traffic.get('bytes_per_cell_step'):
        traffic_per_launch = traffic['bytes_per_cell_step'] * per_launch_cs
    sm_mhz = clocks['sm_mhz'] if clocks else 1900.0
    issue = issue_roofline(traffic, value / world, sm_mhz, n_sm)
    fp32_peak = n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12
    flops = kernel.flops_per_cell_step() * value / world / 1e12

    def sheet512():
        sh = sheet512_runs(args, local, n_sm)
        tr, v = sh.pop('_issue_inputs')
        sh['roofline']['issue'] = issue_roofline(tr, v, sm_mhz, n_sm)
        if sh['roofline']['issue']:
            sh['roofline']['frac'] = sh['roofline']['issue']['frac']
        return sh

    extra = {}
    if rank == 0:
        # Each further measurement reports its own failure instead of
        # losing the headline line
        if args.fp64_ms > 0:
            extra['fp64'] = guarded(c5_fp64, args, local, value / world)
        if args.s1_ms > 0:
            extra['accuracy'] = guarded(c5_accuracy, args, local)
        if args.sheet512_steps > 0:
            extra['sheet512'] = guarded(sheet512)
        if args.accuracy_ms > 0:
            extra['sheet512_accuracy'] = guarded(accuracy_runs, args, local)
        if args.adjoint_ms > 0:
            extra['adjoint'] = guarded(adjoint_runs, args, local)
        others = {}
        for c in [c for c in args.configs.split(',') if c and c != 'none']:
            others[c] = guarded({'c1': config_c1, 'c3': config_c3}[c], args,
                                local)
        if args.full:
            others['c5_full'] = guarded(c5_full, args, local)
        extra['other_configs'] = others
        if not args.no_cpu_baseline:
            extra['cpu_baseline'] = guarded(cpu_baseline, args)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': dev_ms / args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic (seeded probes)',
        'precision': 'FP32 with Kahan-compensated V and concentrations'
                     ' (%s)' % ', '.join(kernel.states[i].qname()
                                         for i in kernel.hi_states),
        'fp32_math': kernel.math,
        'config': config(args),
        'timed_window_ms': [t_end - args.steps * args.step_ms, t_end],
        's2_applied_at_ms': s2_applied[0],
        'e2e': {'value': e2e_value, 'unit': UNIT, 'h2d_bytes_per_step': h2d,
                'd2h_bytes_per_step': d2h},
        'gpu_launches': launches,
        'frames_per_step': n_frames / max(args.steps, 1),
        'roofline': {
            'bound': 'hbm', 'achieved': achieved, 'peak': peak,
            'unit': 'GB/s', 'frac': achieved / peak,
            'traffic': traffic_per_launch,
            'peak_source': peak_kind,
            'bytes_per_cell_step': bpcs,
            'cell_steps_per_launch': per_launch_cs,
            'traffic_source': traffic and traffic.get('source'),
            'compute': {
                'unit': 'TFLOP/s', 'achieved': flops, 'peak': fp32_peak,
                'frac': flops / fp32_peak,
                'flops_per_cell_step': kernel.flops_per_cell_step(),
                'transcendentals_per_cell_step': kernel.census.trans,
                'peak_source': 'FP32 lanes x 2 x median SM clock'},
            'issue': issue,
        },
        'clocks': clocks,
    }
    line.update(extra)
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
