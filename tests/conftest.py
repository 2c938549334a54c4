import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _sources_newer_than_outputs() -> bool:
    from gundam_gb300 import build as B

    outs = [B.LIBDIR / "libgw.so", B.LIBDIR / "libgw_workload.so", B.ORACLE / "_build" / "liboracle.so"]
    if not all(p.exists() for p in outs):
        return True
    srcs = list(B.CSRC.glob("*")) + list(B.INCLUDE.glob("*.h")) + [B.ORACLE / "oracle.cpp", B.ORACLE / "oracle.h"]
    return max(p.stat().st_mtime for p in srcs) > min(p.stat().st_mtime for p in outs)


@pytest.fixture(scope="session", autouse=True)
def native_build():
    if _sources_newer_than_outputs():
        from gundam_gb300 import build as B

        B.build()
    yield


def _have_gpu() -> bool:
    try:
        import ctypes

        from gundam_gb300 import _native as N

        if _sources_newer_than_outputs():
            from gundam_gb300 import build as B

            B.build()
        v = ctypes.c_int32()
        N.libgw().gw_has_gpu(ctypes.byref(v))
        return bool(v.value)
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    gpu_items = [it for it in items if "gpu" in it.keywords]
    if gpu_items and not _have_gpu():
        skip = pytest.mark.skip(reason="no CUDA device")
        for it in gpu_items:
            it.add_marker(skip)
