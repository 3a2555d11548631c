"""
Locates the ``myokit`` package that this backend builds on.

``myokit_gb300`` is a backend for myokit: models, expressions, protocols and
data logs are myokit objects, exactly as for ``myokit.SimulationOpenCL``
(``myokit/_sim/openclsim.py``). This module imports the installed ``myokit``.
When none is installed it falls back to an unmodified myokit installed with
``pip install --target baseline/_ref`` at the repository root, so that a
checkout without a site-wide myokit still runs.
"""
import os
import sys
import warnings

_HERE = os.path.dirname(os.path.abspath(__file__))
_LOCAL_REF = os.path.join(os.path.dirname(_HERE), 'baseline', '_ref')


def import_myokit():
    """Returns the ``myokit`` module, or raises ``ImportError``."""
    try:
        import myokit  # noqa: F401
    except ImportError:
        if os.path.isdir(os.path.join(_LOCAL_REF, 'myokit')):
            sys.path.append(_LOCAL_REF)
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            try:
                import myokit  # noqa: F401,F811
            except ImportError as e:
                raise ImportError(
                    'myokit_gb300 requires myokit: install it, or install it'
                    ' into baseline/_ref at the repository root.') from e
    import myokit  # noqa: F811
    return myokit


myokit = import_myokit()
