"""
Shared fixtures. Tests marked ``gpu`` need a CUDA device; everything else
runs on the CPU (the host library loads and NVRTC compiles without a GPU).
"""
import os
import sys
import warnings

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

warnings.filterwarnings('ignore', message='Using development version')

from myokit_gb300._deps import myokit  # noqa: E402

DATA = os.path.join(os.path.dirname(myokit.__file__), 'tests', 'data')
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def pytest_configure(config):
    config.addinivalue_line(
        'markers', 'gpu: needs a CUDA GPU (sm_103a); run with -m gpu')


def load(name):
    """Loads a model file shipped with myokit's test data."""
    if name == 'example':
        return myokit.load_model('example')
    return myokit.load_model(os.path.join(DATA, name))


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:   # pragma: no cover
        return False


@pytest.fixture(scope='session')
def br77():
    return load('beeler-1977-model.mmt')


@pytest.fixture(scope='session')
def decker():
    return load('decker-2009.mmt')
