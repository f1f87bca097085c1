"""C ABI checks that need no GPU: libodegpu loads and exports every function
declared in include/*.h, the ODE-API demo compiles and links against it, and
the library refuses to run without a CUDA device (no CPU fallback)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b(d[A-Z]\w+|odegpu[A-Z]\w+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", os.path.dirname(LIB), "libodegpu.so"], check=True)
    return C.CDLL(LIB)


@pytest.mark.parametrize("header", ["odegpu.h", "ode_gpu.h"])
def test_exports_every_declared_symbol(lib, header):
    names = declared(header)
    assert len(names) > 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_demo_links_against_libodegpu():
    import c_api_util as U
    with tempfile.TemporaryDirectory() as d:
        U.build_gpu_demo(os.path.join(d, "demo"))


def test_no_device_fails_loudly():
    """Without a CUDA device, creating a batch returns ODEGPU_E_CUDA with a
    message; nothing silently runs on the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from odegpu import scene as S
    from odegpu._lib import OdeGpuError
    from odegpu.batch import Batch
    with pytest.raises(OdeGpuError, match="CUDA"):
        Batch(S.box_drop(seed=0))
