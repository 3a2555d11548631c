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
