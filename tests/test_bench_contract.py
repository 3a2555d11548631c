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


def test_reference_arm_under_torchrun_two_ranks():
    # Launched like the multi-GPU runs: rank 0 alone runs and prints one
    # line, the other rank exits 0 without work
    r = subprocess.run(
        [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1',
         '--nproc-per-node', '2', '--master-addr', '127.0.0.1',
         '--master-port', '29533', os.path.join(ROOT, 'bench.py'),
         '--impl', 'reference', '--size', '16', '--steps', '1', '--warmup',
         '1', '--gpus', '2'],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith('{')]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line['impl'] == 'reference' and line['value'] > 0
