"""
Accuracy metrics between two voltage traces of the same simulation run in
different precisions: the largest |dV|, the activation-time error and the
APD90 error, per probe cell.

Activation time: first upward crossing of ``threshold`` (default -30 mV),
linearly interpolated between log points. APD90: from activation until V
first falls below ``V_rest + 0.1 * (V_peak - V_rest)`` after the peak, with
V_rest the value at the first log point.
"""
import numpy as np


def activation_time(t, v, threshold=-30.0):
    """First upward crossing of ``threshold``, or NaN."""
    t = np.asarray(t, dtype=float)
    v = np.asarray(v, dtype=float)
    above = v >= threshold
    idx = np.nonzero(above[1:] & ~above[:-1])[0]
    if len(idx) == 0:
        return float('nan')
    i = idx[0]
    f = (threshold - v[i]) / (v[i + 1] - v[i])
    return float(t[i] + f * (t[i + 1] - t[i]))


def apd90(t, v, threshold=-30.0):
    """Action potential duration at 90% repolarisation, or NaN."""
    t = np.asarray(t, dtype=float)
    v = np.asarray(v, dtype=float)
    ta = activation_time(t, v, threshold)
    if not np.isfinite(ta):
        return float('nan')
    i0 = int(np.searchsorted(t, ta))
    ip = i0 + int(np.argmax(v[i0:]))
    vrest = v[0]
    level = vrest + 0.1 * (v[ip] - vrest)
    below = np.nonzero(v[ip:] < level)[0]
    if len(below) == 0:
        return float('nan')
    j = ip + below[0]
    f = (level - v[j - 1]) / (v[j] - v[j - 1])
    tr = t[j - 1] + f * (t[j] - t[j - 1])
    return float(tr - ta)


def compare(t, traces, reference):
    """
    Compares a dict of V traces (name -> array) with reference traces of
    the same names. Returns max |dV|, max activation-time error and max
    APD90 error over the traces (errors where both are defined), plus how
    many traces had an APD90 in both.
    """
    dv = 0.0
    dta = 0.0
    dapd = 0.0
    n_apd = 0
    for k, v in traces.items():
        r = reference[k]
        v = np.asarray(v, dtype=float)
        r = np.asarray(r, dtype=float)
        dv = max(dv, float(np.max(np.abs(v - r))))
        a, b = activation_time(t, v), activation_time(t, r)
        if np.isfinite(a) and np.isfinite(b):
            dta = max(dta, abs(a - b))
        a, b = apd90(t, v), apd90(t, r)
        if np.isfinite(a) and np.isfinite(b):
            dapd = max(dapd, abs(a - b))
            n_apd += 1
    return {'max_abs_dV_mV': dv, 'max_activation_error_ms': dta,
            'max_apd90_error_ms': dapd, 'traces_with_apd90': n_apd}


def _frames64(frames):
    import torch
    f = frames if torch.is_tensor(frames) else torch.as_tensor(
        np.asarray(frames, dtype=float))
    return f.detach().to(torch.float64)


def _first(mask):
    """Index of the first True along dim 0, and whether there is one."""
    import torch
    has = mask.any(dim=0)
    return torch.argmax(mask.to(torch.int8), dim=0), has


def _at(x, idx):
    return x.gather(0, idx.unsqueeze(0)).squeeze(0)


def activation_map(times, frames, threshold=-30.0):
    """
    :func:`activation_time` of every cell of a frame set at once: ``frames``
    shaped ``(n, ...)`` (a torch tensor on any device, as returned by
    ``SimulationCUDA.run_frames``, or an array), ``times`` the ``n`` frame
    times. Returns a float64 tensor shaped like one frame, on the frames'
    device, NaN where V never crosses ``threshold`` upwards.
    """
    import torch
    v = _frames64(frames)
    t = torch.as_tensor(np.asarray(times, dtype=float), device=v.device)
    if v.shape[0] != t.shape[0] or v.shape[0] < 2:
        raise ValueError('One time per frame, and at least two frames.')
    above = v >= threshold
    i, has = _first(above[1:] & ~above[:-1])
    vi, vj = _at(v, i), _at(v, i + 1)
    ti, tj = t[i], t[i + 1]
    ta = ti + (threshold - vi) / (vj - vi) * (tj - ti)
    return torch.where(has, ta, torch.full_like(ta, float('nan')))


def apd90_map(times, frames, threshold=-30.0):
    """
    :func:`apd90` of every cell of a frame set at once (see
    :func:`activation_map`): from activation until V first falls below
    ``V_rest + 0.1 * (V_peak - V_rest)`` after the peak, V_rest the first
    frame's value. NaN where there is no activation or no repolarisation.
    """
    import torch
    v = _frames64(frames)
    t = torch.as_tensor(np.asarray(times, dtype=float), device=v.device)
    ta = activation_map(times, v, threshold)
    n = v.shape[0]
    k = torch.arange(n, device=v.device).reshape((n,) + (1,) * (v.dim() - 1))
    # First frame at or after the activation time, then the peak from there
    i0 = (t.reshape(k.shape) < ta.unsqueeze(0)).sum(dim=0)
    masked = torch.where(k >= i0.unsqueeze(0), v,
                         torch.full_like(v, float('-inf')))
    ip = torch.argmax(masked, dim=0)
    vrest = v[0]
    level = vrest + 0.1 * (_at(v, ip) - vrest)
    j, has = _first((v < level.unsqueeze(0)) & (k >= ip.unsqueeze(0)))
    jm = (j - 1).clamp(min=0)
    vj, vm = _at(v, j), _at(v, jm)
    tr = t[jm] + (level - vm) / (vj - vm) * (t[j] - t[jm])
    ok = has & torch.isfinite(ta)
    return torch.where(ok, tr - ta, torch.full_like(ta, float('nan')))


def compare_frames(times, frames, reference, threshold=-30.0):
    """
    :func:`compare` over every cell of two frame sets (for example the
    single- and double-precision ``run_frames`` of one simulation), computed
    on the frames' device: ``max_abs_dV_mV``, ``max_activation_error_ms``
    and ``max_apd90_error_ms`` (where both are defined), and
    ``cells_with_apd90``.
    """
    import torch
    a = _frames64(frames)
    b = _frames64(reference).to(a.device)
    if a.shape != b.shape:
        raise ValueError('The frame sets must have the same shape.')
    dv = float((a - b).abs().max())
    ta, tb = activation_map(times, a, threshold), activation_map(
        times, b, threshold)
    both = torch.isfinite(ta) & torch.isfinite(tb)
    dta = float((ta - tb).abs()[both].max()) if bool(both.any()) else 0.0
    pa, pb = apd90_map(times, a, threshold), apd90_map(times, b, threshold)
    both = torch.isfinite(pa) & torch.isfinite(pb)
    dp = float((pa - pb).abs()[both].max()) if bool(both.any()) else 0.0
    return {'max_abs_dV_mV': dv, 'max_activation_error_ms': dta,
            'max_apd90_error_ms': dp, 'cells_with_apd90': int(both.sum())}


def cable_cv(times, frames, threshold=-30, length=0.01, time_multiplier=1e-3,
             border=None):
    """
    Conduction velocity (cm/s) of a cable from frames shaped ``(n, nx)`` (a
    torch tensor on any device, or an array), as ``myokit.DataBlock1d.cv``
    computes it from a block (``myokit/_datablock.py:152-248``), with the
    same arguments and rules: per cell, the first frame after the first
    where V exceeds -30 mV while rising (the reference's fixed detection
    level), interpolated linearly to ``threshold``; cells from the first
    with a crossing to the last of the run that follows, ``border`` cells
    left out at each end (default a third, at most 50); a least-squares
    line through (time, position). Returns 0 without a crossing. The
    crossings are found on the frames' device; only one time per cell
    comes to the host.
    """
    import torch
    v = _frames64(frames)
    if v.dim() != 2:
        raise ValueError('Cable frames are shaped (n, nx).')
    n, nx = v.shape
    if border is None:
        border = min(50, nx // 3)
    else:
        border = int(border)
        if border < 0:
            raise ValueError('The argument `border` cannot be negative.')
        elif border >= nx // 2:
            raise ValueError(
                'The argument `border` must be less than half the number'
                ' of cells.')
    t = np.asarray(times, dtype=float)
    # Per cell: first frame k >= 1 with V_k > -30 and V_k > V_(k-1)
    rise = (v[1:] > -30) & (v[1:] - v[:-1] > 0)
    k, has = _first(rise)
    k = k + 1
    v1 = _at(v, k)
    v0 = _at(v, k - 1)
    k = k.cpu().numpy()
    has = has.cpu().numpy() & (k > 1)
    v0, v1 = v0.cpu().numpy(), v1.cpu().numpy()
    ts, i1, i2 = [], None, None
    for i in range(border, nx - border):
        if not has[i]:
            if i1 is not None:
                i2 = i - 1
                break
            continue
        if i1 is None:
            i1 = i
        else:
            i2 = i
        t0, t1 = t[k[i] - 1], t[k[i]]
        ts.append(t0 + (threshold - v0[i]) * (t1 - t0) / (v1[i] - v0[i]))
    if i1 is None:
        return 0
    ts = np.asarray(ts) * time_multiplier
    x = np.arange(i1, 1 + i2, dtype=float) * length
    a = np.vstack([ts, np.ones(len(ts))]).T
    return np.linalg.lstsq(a, x, rcond=None)[0][0]
