"""
Launch-shape autotuner for :class:`SimulationCUDA`.

The fused kernel's speed depends on the CTA size, on the register cap that
the minimum number of resident CTAs per SM implies, and on how steps are
grouped into launches (one cooperative launch per chunk with a grid barrier
between steps, or one plain launch per step replayed from a CUDA graph).
:func:`autotune` times candidates on the simulation itself -- same model,
grid, fields and precision -- and keeps the fastest. Results are cached per
configuration signature in ``<cache dir>/tune.json``; a simulation created
with ``block=None`` uses a cached result when one matches.
"""
import json
import os
import time

import numpy as np

from ._deps import myokit

# Candidate (threads per CTA, min CTAs per SM, steps per launch, tile
# staging, step synchronisation). The register cap is 64K / (threads * min
# CTAs), and a warp scheduler holds 16K registers. 576 and 640 threads trade
# registers for the 18 or 20 warps per SM that even out the warp tiles of
# mid-size sheets. Staging 0 prefetches each tile into registers; 1 and 2
# read it from shared memory where used (lazy), which keeps those kernels
# from spilling, with one or two buffers per warp (2: the copies of the
# tile after the next overlap a tile's computation). Steps are separated by
# a grid barrier or by waits on the neighbouring warps only.
_B, _N = 'barrier', 'neighbors'
_CANDIDATES = [
    ((256, 1), 2, 0, False, _B), ((128, 1), 4, 0, False, _B),
    ((512, 1), 1, 0, False, _B), ((192, 1), 3, 0, False, _B),
    ((384, 1), 1, 0, False, _B), ((640, 1), 1, 0, False, _B),
    ((128, 1), 1, 0, False, _B), ((256, 1), 2, 1, False, _B),
    ((512, 1), 1, 0, True, _B), ((576, 1), 1, 0, True, _B),
    ((640, 1), 1, 0, True, _B), ((256, 1), 2, 0, True, _B),
    ((384, 1), 1, 0, True, _B),
    ((512, 1), 1, 0, False, _N), ((384, 1), 1, 0, False, _N),
    ((256, 1), 2, 0, False, _N), ((640, 1), 1, 0, True, _N),
    ((256, 1), 2, 0, True, _N),
    ((256, 1), 2, 0, 2, _B), ((384, 1), 1, 0, 2, _N),
]
_CANDIDATES_FP64 = [((128, 1), 1, 0, False, _B), ((256, 1), 1, 0, False, _B),
                    ((64, 1), 1, 0, False, _B), ((32, 1), 1, 0, False, _B),
                    ((256, 1), 1, 0, True, _B), ((256, 1), 1, 0, False, _N)]
# Grids with fewer warp tiles than SMs: teams of 2 to 16 warps share each
# tile's work (a sixth entry: warps per tile): one team per CTA or two, or
# one team per cluster of 2 or 4 CTAs
_CANDIDATES_SPLIT = [((64, 1), 1, 0, False, _B, 2),
                     ((128, 1), 1, 0, False, _B, 4),
                     ((128, 1), 1, 0, False, _B, 2),
                     ((256, 1), 1, 0, False, _B, 4),
                     ((128, 1), 1, 0, False, _B, 8),
                     ((128, 1), 1, 0, False, _B, 16)]


def _cache_path():
    from .simulation import _cache_dir
    return os.path.join(_cache_dir(), 'tune.json')


def _shipped_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)),
                        'tuned.json')


def signature(sim):
    """A string identifying what the best launch shape depends on."""
    import hashlib
    code = hashlib.sha1(sim._model.code().encode()).hexdigest()[:16]
    return '|'.join(str(x) for x in (
        sim._model.name(), code, sim._nx, sim._ny, len(sim._dims),
        sim._precision, sim._accumulate, sim._diffusion_mode(),
        ','.join(v.qname() for v in sim._fields), len(sim._rl_states),
        sim._fp32_math, sim._native_math,
        'staged' if sim._stage_tiles else 'direct'))


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(sim):
    """The cached choice for this simulation's signature, or None."""
    sig = signature(sim)
    for path in (_cache_path(), _shipped_path()):
        d = _load(path)
        if sig in d:
            return d[sig]
    return None


def _apply(sim, block, min_blocks, spl, lazy=False, sync='barrier',
           split=1):
    sim._block = tuple(block)
    sim._min_blocks = int(min_blocks)
    sim._steps_per_launch = int(spl)
    sim._stage_lazy = int(lazy)
    sim._sync = sync
    sim._split = int(split)
    sim._graphs = 1


def _sm_count(device):
    """SMs of a CUDA device (152 on a GB300, taken when it cannot be
    read)."""
    try:
        import torch
        if torch.cuda.is_available():
            return int(torch.cuda.get_device_properties(
                device).multi_processor_count)
    except Exception:   # pragma: no cover
        pass
    return 152


def _few_tiles(sim):
    """True when the grid has fewer warp tiles than the device has SMs."""
    tiles = -(-sim._nx // 32) * sim._ny
    return tiles < _sm_count(sim._device)


def _candidates(sim):
    """The launch configurations the tuner times on ``sim``."""
    double = sim._precision == myokit.DOUBLE_PRECISION
    # FP64 kernels spill when registers are capped
    out = list(_CANDIDATES_FP64 if double else _CANDIDATES)
    if _few_tiles(sim) and sim._accumulate is None:
        # Cluster teams (more warps per tile than the CTA holds) pay where
        # a tile's double precision instructions bind; a single precision
        # small grid is bound by the step's latency, and its cluster
        # barrier only costs (200-cell cable: 0.074 and 0.065 against
        # 0.098e9 cell-steps/s)
        out += [c for c in _CANDIDATES_SPLIT
                if double or c[5] <= c[0][0] // 32]
    return out


def autotune(sim, duration=None, candidates=None, store=True,
             verbose=False):
    """
    Times each candidate launch configuration on ``sim`` for ``duration``
    time units (default: about 4e8 cell-steps) without logging, restores the
    simulation's state and time, applies the fastest configuration and
    returns ``(best, results)``. ``results`` maps each candidate to its
    cell-steps per second of device time.
    """
    if candidates is None:
        candidates = _candidates(sim)
    if duration is None:
        steps = max(20, int(4e8 / sim._ntotal))
        if sim._precision == myokit.DOUBLE_PRECISION:
            steps = max(4, steps // 20)
        duration = steps * sim.step_size()
    saved = (sim._state.copy(), sim._time, sim._block, sim._min_blocks,
             sim._steps_per_launch, sim._graphs, sim._stage_lazy, sim._sync,
             sim._split)
    results = {}
    try:
        for cand in candidates:
            _apply(sim, *cand)
            block, mb, spl = cand[:3]
            sim._state = saved[0].copy()
            sim._time = saved[1]
            try:
                sim._run(duration / 4, myokit.LOG_NONE, 1, False, None, '')
                sim._state = saved[0].copy()
                sim._run(duration, myokit.LOG_NONE, 1, False, None, '')
            except Exception as e:   # pragma: no cover
                if verbose:
                    print('autotune: %s failed: %s' % (cand, e))
                continue
            st = sim.last_run_stats()
            rate = st['cell_steps'] / (st['kernel_ms'] / 1000.0)
            results[cand] = rate
            if verbose:
                print('autotune: block=%s min_blocks=%d steps/launch=%d'
                      ' -> %.4g cell-steps/s' % (block, mb, spl, rate))
    finally:
        sim._state, sim._time = saved[0], saved[1]
        sim._block, sim._min_blocks = saved[2], saved[3]
        sim._steps_per_launch, sim._graphs = saved[4], saved[5]
        sim._stage_lazy, sim._sync = saved[6], saved[7]
        sim._split = saved[8]
    if not results:
        return None, results
    best = max(results, key=results.get)
    _apply(sim, *best)
    sim._tuned = True
    if store:
        path = _cache_path()
        d = _load(path)
        d[signature(sim)] = {
            'block': list(best[0]), 'min_blocks': best[1],
            'steps_per_launch': best[2],
            'stage_lazy': int(best[3]) if len(best) > 3 else 0,
            'sync': best[4] if len(best) > 4 else 'barrier',
            'split': best[5] if len(best) > 5 else 1,
            'rate': results[best],
            'when': time.strftime('%Y-%m-%dT%H:%M:%S')}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            tmp = path + '.%d' % os.getpid()
            with open(tmp, 'w') as f:
                json.dump(d, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:   # pragma: no cover
            pass
    return best, results
