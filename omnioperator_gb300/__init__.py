"""GB300-native hash aggregation and hash join operators with OmniOperator's operator API.

The compute path is libomniop_gb300.so (hand-written CUDA for sm_103a behind a C ABI,
include/omniop_gb300.h); this package is its Python mirror.  There is no CPU fallback.
"""
from ._capi import OmgError, header_symbols, lib  # noqa: F401
from .api import *  # noqa: F401,F403
