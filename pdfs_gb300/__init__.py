"""GB300-native Fast Sweeping Method (|grad u| = 1) solver: a drop-in for the
FSM solve of GEM3D/PDFS.  The compute path is libpdfs.so (hand-written
sm_103a CUDA kernels behind the C ABI of include/pdfs.h); this package is its
Python front end."""
from . import _lib  # noqa: F401
from .api import Context, PdfsError, run_fsm, solve, sweep  # noqa: F401
