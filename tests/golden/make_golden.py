"""
Generates the golden fixtures in this folder from the reference itself.

Run here, where the reference (myokit) and a C compiler are available:

    python tests/golden/make_golden.py

``br77_sim1d.npz``: myokit's ``Simulation1d`` (reference C code,
``myokit/_sim/cable.c``) on the setting of the reference's own cross-check
``myokit/tests/test_simulation_opencl_vs_sim1d.py:28-60``: Beeler-Reuter
1977, stimulus amplitude -80, 10 cells, 2 paced, blocktrain(1000, 2,
offset=3), dt 0.005, 15 ms, log every 0.5 ms. SimulationOpenCL must match it
to 1e-13 in double precision (same file, lines 123-136).

``br77_cable200_sim1d.npz``: ``Simulation1d`` on the 200-cell cable of the
plain FP64 benchmark configuration (BR77, g = 9, 5 paced cells, 1 Hz 2 ms
pulses, dt 0.005), shortened to 20 ms and logged every 1 ms.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from myokit_gb300._deps import myokit  # noqa: E402


def model():
    path = os.path.join(os.path.dirname(myokit.__file__), 'tests', 'data',
                        'beeler-1977-model.mmt')
    return myokit.load_model(path)


def make_small():
    m = model()
    m.get('membrane.i_stim.amplitude').set_rhs(-80)
    p = myokit.pacing.blocktrain(period=1000, duration=2, offset=3)
    s = myokit.Simulation1d(m, p, ncells=10)
    s.set_step_size(0.005)
    s.set_paced_cells(2)
    log = ['engine.time', 'membrane.V', 'engine.pace', 'isi.Isi',
           'membrane.i_diff']
    d = s.run(15, log=log, log_interval=0.5).npview()
    out = {k.replace('.', '_'): np.asarray(v) for k, v in d.items()}
    np.savez_compressed(os.path.join(HERE, 'br77_sim1d.npz'), **out)


def make_cable():
    m = model()
    p = myokit.pacing.blocktrain(period=1000, duration=2, level=1)
    s = myokit.Simulation1d(m, p, ncells=200)
    s.set_step_size(0.005)
    s.set_conductance(9)
    s.set_paced_cells(5)
    d = s.run(20, log=['engine.time', 'membrane.V'],
              log_interval=1).npview()
    out = {k.replace('.', '_'): np.asarray(v) for k, v in d.items()}
    np.savez_compressed(os.path.join(HERE, 'br77_cable200_sim1d.npz'), **out)


if __name__ == '__main__':
    make_small()
    make_cable()
    print('written to', HERE)
