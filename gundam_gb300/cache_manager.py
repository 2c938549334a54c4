"""Cache::Manager's static interface, as the reference's Propagator uses it.

Mirrors src/CacheManager/include/CacheManager.h:54-200: Build once, then per
likelihood evaluation Fill (a deferred result whose get() copies the bins
back, CacheManager.cpp:750-866), CopyHistogramContents / CopyEventWeights,
ValidateHistogramContents.  A generated Workload stands in for the
SampleSet + EventDialCache pair the reference's Build receives.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .engine import Engine


class Deferred:
    """std::future<bool> with std::launch::deferred semantics."""

    def __init__(self, fn=None):
        self._fn = fn
        self._done = False
        self._value = False

    def valid(self) -> bool:
        return self._fn is not None and not self._done

    def get(self) -> bool:
        if self._fn is None:
            raise RuntimeError("invalid future")
        if not self._done:
            self._value = bool(self._fn())
            self._done = True
        return self._value


class CacheManager:
    _singleton: "CacheManager | None" = None
    _enabled = True
    _hist_copy = True
    _weight_copy = False

    def __init__(self, engine: Engine, workload):
        self.engine = engine
        self.workload = workload
        self.sums = np.zeros(engine.n_bins)
        self.sums2 = np.zeros(engine.n_bins)
        self.llh = 0.0
        self.llh_stat = 0.0
        self.weights = None
        self.params = None

    # ---- static control (CacheManager.h:62-135) ----
    @staticmethod
    def HasCUDA() -> bool:
        """Cache::Manager::HasCUDA: whether the library was built with CUDA
        (CacheManager.cpp:190-192); False when libgw cannot be loaded."""
        try:
            lib = N.libgw()
        except (OSError, RuntimeError):
            return False
        v = C.c_int32()
        N.check(lib.gw_using_cuda(C.byref(v)))
        return bool(v.value)

    @staticmethod
    def HasGPU(dump: bool = False) -> bool:
        v = C.c_int32()
        N.check(N.libgw().gw_has_gpu(C.byref(v)))
        return bool(v.value)

    @classmethod
    def SetIsEnabled(cls, enable: bool) -> None:
        cls._enabled = bool(enable)

    @classmethod
    def IsCacheManagerEnabled(cls) -> bool:
        return cls._enabled

    @classmethod
    def SetIsHistContentCopyEnabled(cls, enable: bool) -> bool:
        old, cls._hist_copy = cls._hist_copy, bool(enable)
        return old

    @classmethod
    def SetIsEventWeightCopyEnabled(cls, enable: bool) -> bool:
        old, cls._weight_copy = cls._weight_copy, bool(enable)
        if cls._singleton is not None:
            cls._singleton.engine.set_event_weight_copy(cls._weight_copy)
        return old

    @classmethod
    def Get(cls) -> "CacheManager | None":
        return cls._singleton

    @classmethod
    def IsBuilt(cls) -> bool:
        return cls._singleton is not None

    # ---- build / fill (CacheManager.cpp:198-475, :750-810) ----
    @classmethod
    def Build(cls, workload, precision: str = "fp64", k_max: int = 1, llh_type=None, device: int = 0) -> bool:
        if not cls._enabled:
            return False
        if cls._singleton is not None:
            cls._singleton.engine.close()
        eng = Engine.from_workload(workload, precision=precision, k_max=k_max, llh_type=llh_type, device=device)
        cls._singleton = CacheManager(eng, workload)
        if cls._weight_copy:
            eng.set_event_weight_copy(True)
        return True

    @classmethod
    def Fill(cls, params) -> Deferred:
        cm = cls._singleton
        if cm is None:
            return Deferred()
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        sums, sums2, llh, stat = cm.engine.eval(p)
        cm.params = p

        def finish():
            cm.sums, cm.sums2 = sums[0], sums2[0]
            cm.llh, cm.llh_stat = float(llh[0]), float(stat[0])
            if cls._weight_copy:
                cm.CopyEventWeights()
            return True

        return Deferred(finish)

    @classmethod
    def PropagateParameters(cls, params) -> bool:
        fut = cls.Fill(params)
        if not fut.valid():
            return False
        return fut.get()

    # ---- results ----
    def CopyHistogramContents(self):
        """BinContent {sumWeights, sqrtSumSqWeights} per global bin (CacheSampleHistFiller.cpp:9-19)."""
        return self.sums.copy(), np.sqrt(self.sums2)

    def CopyEventWeights(self) -> np.ndarray:
        self.weights = self.engine.event_weights()
        return self.weights

    def ValidateHistogramContents(self, sum_weights, sqrt_sum_sq, rel: float = 1e-12) -> bool:
        """Compares with bins filled another way (CacheSampleHistFiller.cpp:21-50)."""
        s, e = self.CopyHistogramContents()
        ok_s = np.allclose(s, sum_weights, rtol=rel, atol=0.0)
        ok_e = np.allclose(e, sqrt_sum_sq, rtol=rel, atol=0.0)
        return bool(ok_s and ok_e)

    def GetResidentMemory(self) -> int:
        return self.engine.resident_memory()

    @classmethod
    def Reset(cls) -> None:
        if cls._singleton is not None:
            cls._singleton.engine.close()
        cls._singleton = None
