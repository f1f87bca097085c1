"""The body-update options of ODE's API (damping, the angular speed cap,
finite rotation, moved callbacks, body geom lists: ode/src/ode.cpp:767-806,
:1000-1133, :1930-2011) on the host: every getter's answer after a seeded
sequence of world and body settings equals the reference's dSINGLE build's,
bit for bit. The steps that apply them run on the GPU
(tests/test_gpu_ode_api.py, against tests/golden/body_step_options.npz)."""
import ctypes as C
import os

import numpy as np
import pytest

import body_step_program as BP

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_body_option_getters_match_reference():
    import oracle_lib as O
    g = np.load(os.path.join(ROOT, "tests", "golden", "body_step_options.npz"))
    ours = BP.bind(C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")))
    for s in g["seeds"]:
        got, _, _ = BP.program(ours, int(s), 1)   # the step itself fails without a device
        assert np.array_equal(got, g[f"dWorldQuickStep_{s}_getters"]), int(s)
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ref = BP.bind(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")))
    for s in range(4, 12):
        a, _, _ = BP.program(ours, s, 1)
        b, _, _ = BP.program(ref, s, 1)
        assert np.array_equal(a, b), s
