"""gundam_gb300: GB300-native replacement for GUNDAM's Cache::Manager reweighting path.

The compute path is libgw.so (C ABI: include/gw.h), hand-written CUDA for
sm_103a.  This package is its Python host side.
"""
from . import _native as native  # noqa: F401
from .cache_manager import CacheManager, Deferred  # noqa: F401
from .engine import Engine  # noqa: F401
from .workload import Workload  # noqa: F401

__all__ = ["CacheManager", "Deferred", "Engine", "Workload", "native"]
