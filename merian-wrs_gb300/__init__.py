"""GB300-native weighted random sampling (the merian-wrs WRS hot path).

The compute lives in libwrs_gb300.so (CUDA, sm_103a) behind the C ABI of
include/wrs.h; `wrs` mirrors the reference's host-side WRS / WRSBuffers API on top.
The directory name contains a hyphen, so load it with
    importlib.import_module("merian-wrs_gb300")
"""
from . import wrs  # noqa: F401
from .wrs import (AliasTableConfig, Batch, CutpointConfig, ITSConfig, WRS,  # noqa: F401
                  WRSBuffers, WRSConfig, WRSError)
from .build import build  # noqa: F401
