"""
Builds the host library ``libmkg_tissue.so`` in-tree with nvcc.

The library holds the C ABI of ``include/mkg_tissue.h`` and the fixed CUDA
kernels (state layout conversion), compiled for sm_103a only. The per-model
tissue kernels are not built here: they are generated per simulation and
compiled at run time with NVRTC (``mkg_compile``), the way the reference
builds its OpenCL program per run.
"""
import os
import shutil
import subprocess
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(_HERE)
LIB_NAME = 'libmkg_tissue.so'
LIB_PATH = os.path.join(_HERE, LIB_NAME)
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def cuda_home():
    home = os.environ.get('CUDA_HOME') or os.environ.get('CUDA_PATH')
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which('nvcc')
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return '/usr/local/cuda'


def sources():
    csrc = os.path.join(_HERE, 'csrc')
    return [os.path.join(csrc, 'mkg_host.cu')]


def headers():
    csrc = os.path.join(_HERE, 'csrc')
    return [
        os.path.join(csrc, 'mkg_kernel_abi.h'),
        os.path.join(csrc, 'mkg_pacing.h'),
        os.path.join(ROOT, 'include', 'mkg_tissue.h'),
    ]


def needs_build():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in sources() + headers())


def build(force=False, verbose=False):
    """Compiles the library if it is missing or stale; returns its path."""
    if not force and not needs_build():
        return LIB_PATH
    home = cuda_home()
    nvcc = os.path.join(home, 'bin', 'nvcc')
    if not os.path.exists(nvcc):
        nvcc = 'nvcc'
    lib64 = os.path.join(home, 'lib64')
    tmp = LIB_PATH + '.tmp.%d' % os.getpid()
    cmd = [nvcc] + ARCH + [
        '-O3', '-lineinfo', '-std=c++17', '-shared',
        '-Xcompiler', '-fPIC', '-Xcompiler', '-Wall',
        '-cudart', 'static',
        '-o', tmp,
    ] + sources() + [
        '-L' + lib64, '-lnvrtc',
        '-Xlinker', '-rpath', '-Xlinker', lib64,
    ]
    if verbose:
        print(' '.join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(
            'Building ' + LIB_NAME + ' failed:\n' + r.stdout + r.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))
