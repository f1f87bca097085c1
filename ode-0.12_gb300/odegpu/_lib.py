"""Loads libodegpu.so (built in-tree next to this package). There is no CPU
fallback: if the library or a CUDA device is missing, calls fail loudly."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libodegpu.so")


class LibraryMissing(RuntimeError):
    pass


class OdeGpuError(RuntimeError):
    pass


def build(force=False):
    """Compile libodegpu.so for sm_103a with nvcc (make in the package dir)."""
    cmd = ["make", "-s", "-C", PKG_DIR]
    if force:
        cmd.append("-B")
    subprocess.run(cmd + ["libodegpu.so"], check=True)


_lib = None
_P = C.POINTER


def _declare(L):
    v, i, d, f = C.c_void_p, C.c_int, C.c_double, C.c_float
    sig = {
        "odegpuBatchCreate": (i, [v, v, _P(v)]),
        "odegpuBatchDestroy": (None, [v]),
        "odegpuBatchStep": (i, [v, i]),
        "odegpuBatchStepPlain": (i, [v, i]),
        "odegpuBatchStepGraph": (i, [v, i]),
        "odegpuBatchSynchronize": (i, [v]),
        "odegpuBatchSetTiming": (i, [v, i]),
        "odegpuBatchSetControlsF32": (i, [v, i, v, v]),
        "odegpuBatchSetJointStops": (i, [v, i, _P(d)]),
        "odegpuBatchSetFeedback": (i, [v, i]),
        "odegpuBatchSetLaunchConfig": (i, [v, i, i, i]),
        "odegpuBatchGetLaunchConfig": (i, [v, _P(i)]),
        "odegpuBatchSetStepKernels": (i, [v, i]),
        "odegpuBatchSetLaunchConfigEx": (i, [v, i, i, i, i]),
        "odegpuBatchGetLaunchConfigEx": (i, [v, i, _P(i), _P(i), _P(i)]),
        "odegpuBatchGetStepKernels": (i, [v, _P(i), _P(i), _P(i)]),
        "odegpuBatchAutotune": (i, [v, i]),
        "odegpuBatchGetFeedback": (i, [v, _P(d)]),
        "odegpuBatchRolloutForward": (i, [v, i, i]),
        "odegpuBatchRolloutBackward": (i, [v, v, v, v, v]),
        "odegpuBatchAdjointStatus": (i, [v, _P(i)]),
        "odegpuBatchGetKernelTimes": (i, [v, _P(d), _P(C.c_longlong)]),
        "odegpuBatchGetLaunchCount": (i, [v, _P(C.c_longlong)]),
        "odegpuBatchReadState": (i, [v, _P(d)]),
        "odegpuBatchWriteState": (i, [v, _P(d)]),
        "odegpuBatchReadStateF32Async": (i, [v, v]),
        "odegpuBatchWriteStateF32Async": (i, [v, v]),
        "odegpuBatchGetStatus": (i, [v, _P(i)]),
        "odegpuBatchGetCounts": (i, [v, _P(i), _P(i), _P(i)]),
        "odegpuBatchGetSeeds": (i, [v, _P(C.c_uint)]),
        "odegpuBatchSetSeeds": (i, [v, _P(C.c_uint)]),
        "odegpuBatchInfo": (i, [v, _P(i), _P(i), _P(i), _P(C.c_longlong), _P(C.c_longlong)]),
        "odegpuBatchStream": (v, [v]),
        "odegpuBatchSetControls": (i, [v, i, _P(d), _P(d)]),
        "odegpuBatchSetStepIndex": (i, [v, i]),
        "odegpuBatchStepTap": (i, [v, _P(f), _P(f), _P(f), _P(i)]),
        "odegpuBatchGetContacts": (i, [v, i, _P(f), i]),
        "odegpuBatchLargeWorldStats": (i, [v, _P(C.c_longlong), i, i]),
        "odegpuBatchRayCast": (i, [v, v, i, i, v]),
        "odegpuBatchSetStepper": (i, [v, i]),
        "odegpuBatchRayCastAsync": (i, [v, v, i, i, v]),
        "odegpuGetLastError": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                f"{LIB_PATH} is not built; run __graft_entry__.build() (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def check(rc):
    if rc < 0:
        raise OdeGpuError(f"libodegpu error {rc}: {lib().odegpuGetLastError().decode()}")
    return rc
