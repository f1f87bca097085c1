"""ODE's simple and hash spaces (ode/src/collision_space.cpp) on the host,
against the reference's dSINGLE build: seeded programs of geom edits and
collides (tests/space_program.py) give the same near-callback pairs in the
same order, the same space member orders after every edit, and the same
space bounding box. Pair order sets the order in which a program creates its
contact joints, so it has to match exactly."""
import ctypes as C
import os

import numpy as np
import pytest

import space_program as SP

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _libs():
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = SP.bind(C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")))
    ref = SP.bind(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")))
    return ours, ref


@pytest.mark.parametrize("kind", ["simple", "hash", "sap"])
def test_space_pairs_and_orders_match_reference(kind):
    ours, ref = _libs()
    n_pairs = 0
    for seed in range(40):
        a, box_a = SP.ops_program(ours, seed, kind)
        b, box_b = SP.ops_program(ref, seed, kind)
        m = min(len(a), len(b))
        assert a.shape == b.shape and np.array_equal(a, b), (seed, int(np.argmax(a[:m] != b[:m])))
        # within FP32 rounding: a body's orientation goes through a quaternion
        # normalised in FP64 here and in FP32 in the reference
        assert np.allclose(box_a, box_b, rtol=1e-6, atol=1e-6), (seed, box_a, box_b)
        n_pairs += len(a)
    assert n_pairs > 10000


def test_space_order_fixture_prefix_without_gpu():
    """The fixture of spaces reordered by world steps (the reference's
    dSINGLE build, tests/golden/space_order.npz) up to the first step: the
    initial member order and the first near-callback pairs, which need no
    GPU. The steps themselves are checked in tests/test_gpu_ode_api.py."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "space_order.npz"))
    ours = SP.bind(C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")))
    for s in g["seeds"]:
        want = g[f"dWorldQuickStep_{s}"]
        got = SP.step_program(ours, int(s), 1)   # the step itself fails without a device
        n0 = int(np.argmax(want == -9)) + 1
        n1 = n0 + 1 + 2 * int(want[n0])
        assert want[n0] > 0 and np.array_equal(got[:n1], want[:n1])


def test_quadtree_space_pairs_match_reference():
    """dQuadTreeSpaceCreate (ode/src/collision_quadtreespace.cpp): the pairs of
    dSpaceCollide and dSpaceCollide2 over seeded programs of edits
    (tests/space_program.py quad_program) equal the reference's dSINGLE
    build's entry for entry, with ODE 0.12's missing enumeration and
    infinite box."""
    ours, ref = _libs()
    n = 0
    for seed in range(40):
        a, b = SP.quad_program(ours, seed), SP.quad_program(ref, seed)
        m = min(len(a), len(b))
        assert a.shape == b.shape and np.array_equal(a, b), (seed, int(np.argmax(a[:m] != b[:m])))
        n += len(a)
    assert n > 4000
    # ODE 0.12 does not enumerate a quadtree (its getGeom aborts); here it answers 0
    ours.dQuadTreeSpaceCreate.restype = C.c_void_p
    ours.dQuadTreeSpaceCreate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    v = (C.c_float * 4)(0, 0, 0, 0)
    e = (C.c_float * 4)(1, 1, 1, 0)
    q = ours.dQuadTreeSpaceCreate(None, v, e, 2)
    ours.dCreateSphere(q, 0.2)
    assert ours.dSpaceGetNumGeoms(q) == 1 and ours.dSpaceGetGeom(q, 0) is None
    ours.dSpaceDestroy(q)


def test_sap_space_tie_order_matches_reference():
    """Sweep and prune (ode/src/collision_sapspace.cpp) with many equal sort
    keys, negative ones included, over repeated collides: the radix sort's
    order of equal keys and its reuse of the previous order give the
    reference's pairs entry for entry."""
    ours, ref = _libs()
    for seed in range(10):
        a, b = SP.sap_tie_program(ours, seed), SP.sap_tie_program(ref, seed)
        m = min(len(a), len(b))
        assert a.shape == b.shape and np.array_equal(a, b), (seed, int(np.argmax(a[:m] != b[:m])))
        assert len(a) > 500
