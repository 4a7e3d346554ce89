"""GB300 (sm_103a) split-operator propagation path behind the split_operator API.

The compute lives in ``_build/libsplit_operator_gb300.so`` (hand-written CUDA +
C++ host runtime, C ABI in ``include/split_operator.h``); this package is the
Python mirror of the Rust crate's API over that ABI.
"""
from .api import *  # noqa: F401,F403
from .api import (  # noqa: F401
    APPLY_NONE, FIRST_HALF, FULL, HALF, INVERSE_FIRST, NORMAL, PRECISION, SECOND_HALF,
    SplitOperatorError, launch_count,
)
