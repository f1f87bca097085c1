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


def test_rotation_utilities_match_reference_fp32():
    """dRFromAxisAndAngle, dRFromEulerAngles, dRFrom2Axes, dRFromZAxis,
    dQFromAxisAndAngle, dQMultiply0-3, dRfromQ, dQfromR, dDQfromW,
    dSafeNormalize3/4 and dPlaneSpace of the library (host code, no GPU)
    against the reference's dSINGLE build on seeded inputs: bit-identical
    (the reference's transcendentals are the same libm calls)."""
    import ctypes as C
    import numpy as np
    import c_api_util as U
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))
    F = C.c_float
    V4 = F * 4
    M12 = F * 12
    rng = np.random.default_rng(4)
    for lib in (ours, ref):
        for name in ("dRFromAxisAndAngle", "dQFromAxisAndAngle"):
            getattr(lib, name).argtypes = [C.c_void_p, F, F, F, F]
        lib.dRFromEulerAngles.argtypes = [C.c_void_p, F, F, F]
        lib.dRFrom2Axes.argtypes = [C.c_void_p, F, F, F, F, F, F]
        lib.dRFromZAxis.argtypes = [C.c_void_p, F, F, F]
    for _ in range(200):
        a = [float(x) for x in rng.normal(size=7)]
        outs = []
        for lib in (ours, ref):
            R1, R2, R3, R4 = M12(), M12(), M12(), M12()
            q1, q2 = V4(), V4()
            lib.dRFromAxisAndAngle(R1, *a[:4])
            lib.dRFromEulerAngles(R2, *a[:3])
            lib.dRFrom2Axes(R3, *a[:6])
            lib.dRFromZAxis(R4, *a[:3])
            lib.dQFromAxisAndAngle(q1, *a[3:7])
            lib.dQfromR(q2, R1)
            qm = []
            for k in range(4):
                r = V4()
                getattr(lib, f"dQMultiply{k}")(r, q1, q2)
                qm += list(r)
            R5, dq = M12(), V4()
            lib.dRfromQ(R5, q1)
            w = V4(*a[:3], 0.0)
            lib.dDQfromW(dq, w, q1)
            n3, n4 = V4(*a[:3], 0.0), V4(*a[:4])
            r3 = lib.dSafeNormalize3(n3)
            r4 = lib.dSafeNormalize4(n4)
            p, q = V4(), V4()
            lib.dPlaneSpace(n3, p, q)
            outs.append(np.array(list(R1) + list(R2) + list(R3) + list(R4) + list(q1) + list(q2) + qm + list(R5) +
                                 list(dq) + list(n3)[:3] + list(n4) + [r3, r4] + list(p)[:3] + list(q)[:3],
                                 dtype=np.float32))
        assert np.array_equal(outs[0], outs[1]), np.abs(outs[0] - outs[1]).max()
