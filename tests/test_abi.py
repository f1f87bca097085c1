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
        U.build_gpu_demo(os.path.join(d, "player"), src=U.PLAYER)


def test_scene_player_is_the_reference_harness_sequence():
    """tests/c_api/scene_player.c, built against the reference ODE 0.12
    (dSINGLE) where it was built in this checkout, reproduces the reference
    harness bit for bit on the joint-type scene and the cylinder pile: the program the GPU test
    links against libodegpu is a faithful ODE program."""
    import c_api_util as U
    import numpy as np
    import oracle_lib as O
    from odegpu import scene as S
    if not (U.ref_demo_available() and O.ref_available("s")):
        pytest.skip("reference not built in this checkout")
    with tempfile.TemporaryDirectory() as d:
        exe = U.build_ref_demo(os.path.join(d, "player"), src=U.PLAYER)
        for sc in (S.mechanisms(n_worlds=2, steps=60), S.cylinder_pile(n_worlds=1)):
            for w in range(sc.n_worlds):
                inp = os.path.join(d, f"in{w}.txt")
                U.player_input(sc, w, 60, inp)
                st = U.run_demo(exe, inp).astype(np.float32).astype(np.float64)
                ref = O.run_world(O.ref("s").ref_run_world, sc, w, 60)["state"][-1]
                assert np.array_equal(st, ref), float(np.abs(st - ref).max())
        # and with dWorldStep
        sc = S.mechanisms(n_worlds=2, steps=60)
        with O.exact_stepper(O.ref("s")):
            for w in range(sc.n_worlds):
                inp = os.path.join(d, f"in{w}.txt")
                U.player_input(sc, w, 40, inp)
                st = U.run_demo(exe, inp, "exact").astype(np.float32).astype(np.float64)
                ref = O.run_world(O.ref("s").ref_run_world, sc, w, 40)["state"][-1]
                assert np.array_equal(st, ref), float(np.abs(st - ref).max())


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
