"""Cache::Manager's static interface (gundam_gb300/cache_manager.py) on the CPU:
the deferred result, the enable switches and the state before a Build
(CacheManager.h:54-135, CacheManager.cpp:198-201).  Build, Fill and the copies
run on the GPU (tests/test_gpu_engine.py)."""
import pytest

from gundam_gb300.cache_manager import CacheManager, Deferred


def test_deferred_runs_once_on_get():
    calls = []
    fut = Deferred(lambda: calls.append(1) or True)
    assert fut.valid() and not calls
    assert fut.get() is True and calls == [1]
    assert fut.get() is True and calls == [1]  # the result is kept, the work not redone
    assert not fut.valid()
    with pytest.raises(RuntimeError):
        Deferred().get()


def test_disabled_manager_builds_nothing():
    """Build returns false when the manager is disabled (CacheManager.cpp:200),
    before any device work; Fill then has no valid result."""
    CacheManager.Reset()
    CacheManager.SetIsEnabled(False)
    try:
        assert not CacheManager.IsCacheManagerEnabled()
        assert CacheManager.Build(workload=None) is False
        assert not CacheManager.IsBuilt() and CacheManager.Get() is None
        assert not CacheManager.Fill([0.0]).valid()
        assert CacheManager.PropagateParameters([0.0]) is False
    finally:
        CacheManager.SetIsEnabled(True)


def test_copy_switches_return_the_previous_setting():
    old = CacheManager.SetIsHistContentCopyEnabled(False)
    assert CacheManager.SetIsHistContentCopyEnabled(old) is False
    old_w = CacheManager.SetIsEventWeightCopyEnabled(True)
    assert CacheManager.SetIsEventWeightCopyEnabled(old_w) is True


def test_has_gpu_reports_the_host():
    import torch

    assert CacheManager.HasGPU() == torch.cuda.is_available()


def test_has_cuda_asks_the_library():
    """HasCUDA reports whether the kernels were compiled with CUDA
    (Cache::Parameters::UsingCUDA, CacheParameters.cpp:12-18): the library
    answers, no device is needed."""
    import ctypes as C

    from gundam_gb300 import _native as N

    v = C.c_int32(-1)
    assert N.libgw().gw_using_cuda(C.byref(v)) == N.GW_OK
    assert v.value == 1
    assert CacheManager.HasCUDA() is True
