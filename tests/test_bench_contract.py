"""
The bench's JSON contract on the CPU: the reference arm (the reference's
kernel on the host cores) at a tiny size prints one line with the fields
the measurement contract asks for.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run(
        [sys.executable, os.path.join(ROOT, 'bench.py'), '--impl',
         'reference', '--size', '24', '--steps', '2', '--warmup', '1'],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line['impl'] == 'reference'
    for key in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup',
                'ms_per_step', 'higher_is_better', 'scaling', 'dtype',
                'config', 'cpu_baseline', 'e2e'):
        assert key in line, key
    assert line['value'] > 0 and line['steps'] == 2
    assert line['cpu_baseline']['kind'] == 'reference'
    assert line['e2e']['h2d_bytes_per_step'] == 0
    assert line['config']['grid'] == [24, 24]


def test_help_lists_options():
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'),
                        '--help'], capture_output=True, text=True,
                       timeout=120, cwd=ROOT)
    assert r.returncode == 0
    for opt in ('--gpus', '--steps', '--warmup', '--impl', '--tune',
                '--profile', '--configs'):
        assert opt in r.stdout
