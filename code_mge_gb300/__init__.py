"""GB300-native multigrid Runge-Kutta residual cycle of code_mge.

The compute path is hand-written CUDA for sm_103a behind the C-ABI of
include/mge_gpu.h (libmge_gpu.so, built in-tree by ``build.build()``);
``runtime.Cycle`` drives it with the reference's routine names and
``cases`` builds synthetic cut-cell cases.  There is no CPU fallback: every
entry point fails loudly when the library is missing.
"""
from . import _abi, cases  # noqa: F401

__all__ = ["_abi", "cases"]
