"""
NaN diagnosis for :class:`SimulationCUDA`, with the behaviour of
``SimulationOpenCL.find_nan`` (``myokit/_sim/openclsim.py:395-702``) and of
the error report raised at the end of ``_run`` (``openclsim.py:1152-1281``).

The search re-runs the simulation from the last good logged state with
log intervals ten times finer each round, until every step is logged, then
reports the first bad cell and variable.
"""
import numpy as np

from ._deps import myokit


def _first_nonfinite(ar, lo, hi):
    """Index of the first non-finite entry in ar[lo:hi+1], given that ar[hi]
    is non-finite (bisection, openclsim.py:464-473)."""
    while True:
        if not np.isfinite(ar[lo]):
            return lo
        md = lo + int(np.ceil(0.5 * (hi - lo)))
        if md == hi:
            return hi
        if not np.isfinite(ar[md]):
            hi = md
        else:
            lo = md


def _nan_locator(sim):
    def locate(log):
        ifirst = None
        kfirst = None
        for key, ar in log.items():
            if ifirst is None:
                if not np.isfinite(ar[-1]):
                    kfirst = key
                    ifirst = _first_nonfinite(ar, 0, len(ar) - 1)
                    if ifirst == 0:
                        break
            elif not np.isfinite(ar[ifirst - 1]):   # pragma: no cover
                kfirst = key
                ifirst = _first_nonfinite(ar, 0, ifirst)
                if ifirst == 0:
                    break
        return ifirst, kfirst
    return locate


def _range_locator(sim, watch_var, safe_range):
    lower, upper = safe_range
    post = '.' + watch_var.qname()

    def locate(log):
        ifirst = None
        kfirst = None
        for dims in myokit._dimco(*sim._dims):
            key = '.'.join([str(x) for x in dims]) + post
            ar = np.asarray(log[key])
            bad = np.where(
                (ar < lower) | (ar > upper) | np.isnan(ar) | np.isinf(ar))[0]
            if len(bad) > 0:
                i = bad[0]
                if ifirst is None or i < ifirst:
                    kfirst = key
                    ifirst = i
                if i == 0:  # pragma: no cover
                    break
        return ifirst, kfirst
    return locate


def _cell_state(sim, log, index):
    state = []
    for dims in myokit._dimco(*sim._dims):
        pre = '.'.join([str(x) for x in dims]) + '.'
        for s in sim._model.states():
            state.append(log[pre + s.qname()][index])
    return state


def find_nan(sim, log, watch_var=None, safe_range=None, return_log=False):
    """See :meth:`SimulationCUDA.find_nan`."""
    # The log must hold all states and bound variables
    g = []
    for label in sim._global:
        var = sim._model.binding(label)
        if var is not None:
            g.append(var.qname())
    need = myokit.prepare_log(
        myokit.LOG_STATE + myokit.LOG_BOUND, sim._model, dims=sim._dims,
        global_vars=g)
    for key in need:
        if key not in log:
            raise myokit.FindNanError(
                'Method requires a simulation log containing all states'
                ' and bound variables. Missing variable <' + key + '>.')

    if watch_var is None:
        locate = _nan_locator(sim)
    else:
        try:
            watch_var = sim._model.get(watch_var)
        except KeyError:
            raise myokit.FindNanError(
                'Variable <' + str(watch_var) + '> not found.')
        if not watch_var.is_state():
            raise myokit.FindNanError('The watched variable must be a state.')
        try:
            lo, hi = safe_range
        except Exception:
            raise myokit.FindNanError(
                'A safe range must be specified for the watched variable'
                ' as a tuple (lower, upper).')
        if lo >= hi:
            raise myokit.FindNanError(
                'The safe range must have a lower bound that is lower than'
                ' the upper bound.')
        locate = _range_locator(sim, watch_var, safe_range)

    time_var = sim._model.time().qname()

    def rerun(log, interval):
        ifirst, kfirst = locate(log)
        if kfirst is None:
            raise myokit.FindNanError('Error condition not found in log.')
        if ifirst == 0:
            raise myokit.FindNanError(
                'Unable to work with simulation logs where the error'
                ' condition is met in the very first data point.')
        istart = ifirst - 1
        state = _cell_state(sim, log, istart)
        t0 = log[time_var][istart]
        saved = (sim._state.copy(), sim._time)
        sim._state = np.array(state, dtype=float)
        sim._time = t0
        try:
            return sim.run(
                log[time_var][ifirst] - t0,
                log=myokit.LOG_BOUND + myokit.LOG_STATE,
                log_interval=interval, report_nan=False)
        finally:
            sim._state, sim._time = saved

    try:
        dt = log[time_var][1] - log[time_var][0]
    except IndexError:  # pragma: no cover
        dt = 5
    while dt > 0:
        dt *= 0.1
        if dt < 0.5:
            dt = 0
        log = rerun(log, dt)

    ifirst, kfirst = locate(log)
    if ifirst is None:
        ifirst = 0
        kfirst = next(iter(log.items()))[0]

    ndims = len(sim._dims)
    icell = [int(x) for x in kfirst.split('.')[0:ndims]]

    def cell_values(index):
        s = []
        b = {}
        for var in sim._model.states():
            s.append(log[var.qname(), icell][index])
        for var in sim._model.variables(bound=True):
            if var.binding() in sim._global:
                b[var.qname()] = log[var.qname()][index]
            else:
                b[var.qname()] = log[var.qname(), icell][index]
        return s, b

    times, states, bounds = [], [], []
    max_states = 3
    for k in range(ifirst, ifirst - max_states - 1, -1):
        if k < 0:
            break
        times.append(log[time_var][k])
        s, b = cell_values(k)
        states.append(s)
        bounds.append(b)

    var = sim._model.get('.'.join(kfirst.split('.')[ndims:]))
    if var.is_state():
        value = states[1 if ifirst > 0 else 0][var.index()]
    else:  # pragma: no cover
        value = bounds[1 if ifirst > 0 else 0][var.qname()]
    var = var.qname()
    time = log[time_var][ifirst]

    if return_log:
        istart = max(0, ifirst - max_states)
        state = _cell_state(sim, log, istart)
        saved = (sim._state.copy(), sim._time)
        sim._state = np.array(state, dtype=float)
        sim._time = times[-1]
        try:
            log = sim.run(
                len(times) * sim._step_size,
                log=myokit.LOG_BOUND + myokit.LOG_STATE + myokit.LOG_INTER,
                log_interval=0, report_nan=False)
        finally:
            sim._state, sim._time = saved
        return time, icell, var, value, states, bounds, log
    return time, icell, var, value, states, bounds


def report_nan(sim, log):
    """Raises a :class:`myokit.SimulationError` describing the first
    numerical error in ``log`` (openclsim.py:1152-1281)."""
    prec = sim._precision
    fs = myokit.float.str
    txt = ['Numerical error found in simulation logs.']
    try:
        time, icell, var, value, states, bounds, d = find_nan(
            sim, log, return_log=True)
        icell_str = '(' + ','.join([str(x) for x in icell]) + ')'
        txt.append(
            'Encountered numerical error at t=' + fs(time, precision=prec)
            + ' in cell ' + icell_str + ' when ' + var + '='
            + fs(value, precision=prec) + '.')
        is_paced = sim.is_paced(*icell)
        paced_str = (', cell ' + icell_str + ' '
                     + ('IS' if is_paced else 'is NOT') + ' paced')
        vtime = sim._model.time().qname()
        vpace = sim._model.binding('pace')
        vpace = None if vpace is None else vpace.qname()
        vdiff = None
        if sim._diffusion_enabled:
            vdiff = sim._model.binding('diffusion_current')
            vdiff = None if vdiff is None else vdiff.qname()
        neighbors = sim.neighbors(*icell)
        if len(sim._dims) == 2:
            neighbors_str = ', '.join(
                ('(' + ','.join([str(i) for i in j]) + ')') for j in neighbors)
        else:
            neighbors_str = ', '.join(str(j) for j in neighbors)

        def bound_lines(b):
            out = ['  Time: ' + fs(b[vtime], precision=prec)]
            if vpace is not None:
                out.append('  Pacing variable: ' + fs(b[vpace], precision=prec)
                           + paced_str)
            if vdiff is not None:
                out.append('  Diffusion current: '
                           + fs(b[vdiff], precision=prec))
            if neighbors:
                out.append('  Connected cells: ' + neighbors_str)
            return out

        txt.append('State during:')
        txt.append(sim._model.format_state(states[0], precision=prec))
        txt.append('Simulation variables during:')
        txt.extend(bound_lines(bounds[0]))

        n_states = len(states)
        txt.append('Obtained ' + str(n_states) + ' previous state(s).')
        if n_states > 1:
            state = states[1]
            bound = {'time': bounds[1][vtime], 'pace': 0,
                     'diffusion_current': 0}
            if is_paced and vpace is not None:
                bound['pace'] = bounds[1][vpace]
            if vdiff is not None:
                bound['diffusion_current'] = bounds[1][vdiff]
            eval_error = None
            try:
                derivs = sim._model.evaluate_derivatives(
                    state, bound, prec, ignore_errors=False)
            except myokit.NumericalError as ee:
                derivs = sim._model.evaluate_derivatives(
                    state, bound, prec, ignore_errors=True)
                eval_error = str(ee)
            txt.append('State before:')
            txt.append(sim._model.format_state_derivatives(
                state, derivs, prec))
            txt.append('Simulation variables before:')
            txt.extend(bound_lines(bounds[1]))
            txt.append('Logged all variables for points: ' + ', '.join(
                fs(t, precision=prec) for t in d.time()))
            txt.append('Non-finite valued variables at t='
                       + fs(d.time()[-2], precision=prec))
            for key, values in d.items():
                v = values[-2]
                if not np.isfinite(v):
                    txt.append('  ' + str(key) + ' = ' + fs(v, precision=prec))
            if eval_error is not None:
                txt.append('Error when evaluating derivatives:')
                txt.append(eval_error)
    except myokit.FindNanError as e:
        txt.append('Unable to pinpoint source of NaN, an error occurred:')
        txt.append(str(e))
    raise myokit.SimulationError('\n'.join(txt))
