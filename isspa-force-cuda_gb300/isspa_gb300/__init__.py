"""GB300-native IS-SPA implicit-solvent MD force engine (Python host bindings).

The compute path is libisspa_gb300.so (hand-written sm_103a kernels behind a
C ABI, include/isspa_gb300.h).  This package only binds it: there is no CPU
fallback, and loading fails loudly when the library has not been built.
"""
from .abi import IsspaError, lib  # noqa: F401
from .engine import Engine, host_array, measure_fp32_peak  # noqa: F401
from .system import System, read_run_config  # noqa: F401
from . import synth  # noqa: F401
