"""CPU tests of the oracle (the checker): known-answer tests from the reference,
golden vectors produced by the reference ODE 0.12, and, where the reference was
built in this checkout, live bit-for-bit comparison against it."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from odegpu import scene as S
import oracle_lib as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_P = C.POINTER


def test_rand_kat():
    """dTestRand's first five LCG outputs from seed 0 (ode/src/misc.cpp:52-62)."""
    L = O.oracle()
    assert L.oracle_test_rand() == 1
    L.oracle_rand_set_seed(0)
    expect = [0x3c6ef35f, 0x47502932, 0xd1ccf6e9, 0xaaf95334, 0x6252e503]
    got = []
    for _ in expect:
        L.oracle_rand_int(1 << 30)  # one dRand call each; seed readback below
        got.append(L.oracle_rand_get_seed())
    assert got == expect


def test_rand_int_golden():
    """dRandInt over the xor-fold branches, against reference output."""
    g = np.load(os.path.join(GOLDEN, "rng_kat.npz"))
    L = O.oracle()
    for s, row in zip(g["seeds"], g["vals"]):
        L.oracle_rand_set_seed(int(s))
        got = [L.oracle_rand_int(int(n)) for n in g["ns"] for _ in range(7)]
        assert got == list(row)


def test_collider_kats_golden():
    """Every collider on the path, single dCollide calls on seeded near-contact
    poses, both argument orders: contact count and records bit-exact vs the
    reference."""
    g = np.load(os.path.join(GOLDEN, "collider_kats.npz"))
    L = O.oracle()
    n = len(g["t1"])
    mism = 0
    for i in range(n):
        out = np.zeros((16, 9))
        args = [np.ascontiguousarray(g[k][i], dtype=np.float64) for k in
                ("p1", "pos1", "R1", "p2", "pos2", "R2")]
        nc = L.oracle_collide(int(g["t1"][i]), *(a.ctypes.data_as(_P(C.c_double)) for a in args[:3]),
                              int(g["t2"][i]), *(a.ctypes.data_as(_P(C.c_double)) for a in args[3:]),
                              int(g["flags"][i]), out.ctypes.data_as(_P(C.c_double)))
        if nc != g["nc"][i] or not np.array_equal(out[:nc, :7], g["out"][i][:nc, :7]):
            mism += 1
    assert mism == 0, f"{mism} of {n} collider calls differ"
    assert (g["nc"] > 0).sum() > n // 4  # the poses do exercise contact


def hf_from_golden(g):
    """The heightfield of hf_kats.npz as a ctypes odegpuHeightfield (the
    returned tuple keeps the height array alive)."""
    h = np.ascontiguousarray(g["heights"], dtype=np.float64)
    sp = float(g["spacing"])
    H = S.Heightfield()
    H.nz, H.nx = h.shape
    H.width, H.depth = sp * (H.nx - 1), sp * (H.nz - 1)
    H.scale, H.offset, H.thickness, H.wrap = 1.0, 0.0, 1.0, 0
    H.heights = h.ctypes.data_as(_P(C.c_double))
    H.pos[:] = [float(x) for x in g["hf_pos"]]
    H.R[:] = [float(x) for x in g["hf_R"]]
    return H, h


@pytest.mark.parametrize("fixture", ["hf_kats", "hf_big_kats"])
def test_heightfield_kats_golden(fixture):
    """dCollide(heightfield, sphere / box / capsule) on a placeable fractal
    field (dCollideHeightfield, ode/src/heightfield.cpp:1677-1853): contact
    count and records bit-exact vs the reference. hf_big_kats: geoms of
    several metres (and cylinders) on a 0.25 m field, zones of up to ~60
    samples per axis."""
    g = np.load(os.path.join(GOLDEN, f"{fixture}.npz"))
    H, _h = hf_from_golden(g)
    L = O.oracle()
    f = L.oracle_collide_hf
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_double), C.c_int,
                  _P(C.c_double)]
    n = len(g["t2"])
    mism = 0
    for i in range(n):
        out = np.zeros((64, 9))
        args = [np.ascontiguousarray(g[k][i], dtype=np.float64) for k in ("p2", "pos2", "R2")]
        nc = f(C.byref(H), int(g["t2"][i]), *(a.ctypes.data_as(_P(C.c_double)) for a in args),
               int(g["flags"][i]), out.ctypes.data_as(_P(C.c_double)))
        if nc != g["nc"][i] or not np.array_equal(out[:nc, :7], g["out"][i][:nc, :7]):
            mism += 1
    assert mism == 0, f"{mism} of {n} heightfield calls differ"
    assert (g["nc"] > 0).sum() > n // 2


@pytest.mark.parametrize("fixture,hf_class", [("ray_kats", 5), ("cylinder_kats", 3)])
def test_ray_and_cylinder_kats_golden(fixture, hf_class):
    """Rays (ode/src/ray.cpp:196-698) and cylinders (ode/src/cylinder.cpp,
    collision_cylinder_sphere.cpp, collision_cylinder_box.cpp,
    collision_cylinder_plane.cpp) through dCollide, every collider in both
    argument orders plus the pairs without a collider (ray-ray,
    cylinder-cylinder, capsule-cylinder), and against the placeable field of
    hf_kats.npz (rays take the plane pass only; cylinders have no point-depth
    function, so the vertex pass casts rays, ode/src/heightfield.cpp:1035-1068,
    1562-1584): counts and records bit-exact vs the reference."""
    g = np.load(os.path.join(GOLDEN, f"{fixture}.npz"))
    L = O.oracle()
    n = len(g["t1"])
    mism = 0
    for i in range(n):
        out = np.zeros((16, 9))
        args = [np.ascontiguousarray(g[k][i], dtype=np.float64) for k in
                ("p1", "pos1", "R1", "p2", "pos2", "R2")]
        nc = L.oracle_collide(int(g["t1"][i]), *(a.ctypes.data_as(_P(C.c_double)) for a in args[:3]),
                              int(g["t2"][i]), *(a.ctypes.data_as(_P(C.c_double)) for a in args[3:]),
                              int(g["flags"][i]), out.ctypes.data_as(_P(C.c_double)))
        if nc != g["nc"][i] or not np.array_equal(out[:nc, :7], g["out"][i][:nc, :7]):
            mism += 1
    assert mism == 0, f"{mism} of {n} {fixture} collider calls differ"
    assert (g["nc"] > 0).sum() > n // 4
    H, _h = hf_from_golden(np.load(os.path.join(GOLDEN, "hf_kats.npz")))
    f = L.oracle_collide_hf
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_double), C.c_int,
                  _P(C.c_double)]
    m = len(g["hf_nc"])
    mism = 0
    for i in range(m):
        out = np.zeros((64, 9))
        args = [np.ascontiguousarray(g[k][i], dtype=np.float64) for k in ("hf_p2", "hf_pos2", "hf_R2")]
        nc = f(C.byref(H), hf_class, *(a.ctypes.data_as(_P(C.c_double)) for a in args), int(g["hf_flags"][i]),
               out.ctypes.data_as(_P(C.c_double)))
        if nc != g["hf_nc"][i] or not np.array_equal(out[:nc, :7], g["hf_out"][i][:nc, :7]):
            mism += 1
    assert mism == 0, f"{mism} of {m} heightfield calls differ"
    assert (g["hf_nc"] > 0).sum() > m // 2


@pytest.mark.parametrize("name", ["box_drop", "batched", "hinge", "stack", "capsule", "vehicles", "capsule_pile",
                                  "mechanisms", "cylinder_pile"])
def test_oracle_matches_reference_golden(name):
    """Whole-step parity: contact counts, contact records, RNG seeds, body
    states and joint feedback are bit-identical to the reference (FP64)."""
    g = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    sc = S.Scene.from_arrays(g)
    steps = int(g["n_steps"])
    for w in range(sc.n_worlds):
        r = O.run_world(O.oracle().oracle_run_world, sc, w, steps, max_rec=96, feedback=True)
        assert np.array_equal(r["ncontacts"], g[f"w{w}_ncontacts"])
        assert np.array_equal(r["seeds"], g[f"w{w}_seeds"])
        assert np.array_equal(r["contacts"][:, :64], g[f"w{w}_contacts"])
        assert np.array_equal(r["state"][::10], g[f"w{w}_state"])
        assert np.array_equal(r["state"][-1], g[f"w{w}_final"])
        assert np.array_equal(r["feedback"], g[f"w{w}_feedback"])


@pytest.mark.parametrize("name", ["box_drop", "batched", "mechanisms", "vehicles", "cylinder_pile"])
def test_oracle_exact_stepper_matches_reference_golden(name):
    """dWorldStep (ode/src/step.cpp:187-846: joints ordered unbounded / mixed /
    LCP, A = J invM J' + cfm / h, the Dantzig LCP of ode/src/lcp.cpp with
    ODE's LDL' kernels) on the same scenes: contact counts, RNG seeds, body
    states and joint feedback bit-identical to the reference (FP64)."""
    g = dict(np.load(os.path.join(GOLDEN, f"exact_{name}.npz")))
    sc = S.Scene.from_arrays(g)
    steps = int(g["n_steps"])
    with O.exact_stepper():
        for w in range(sc.n_worlds):
            r = O.run_world(O.oracle().oracle_run_world, sc, w, steps, max_rec=96, feedback=True)
            assert np.array_equal(r["ncontacts"], g[f"w{w}_ncontacts"])
            assert np.array_equal(r["seeds"], g[f"w{w}_seeds"])
            assert np.array_equal(r["contacts"][:, :64], g[f"w{w}_contacts"])
            assert np.array_equal(r["state"][::10], g[f"w{w}_state"])
            assert np.array_equal(r["state"][-1], g[f"w{w}_final"])
            assert np.array_equal(r["feedback"], g[f"w{w}_feedback"])
    assert O.oracle().oracle_lcp_errors() == 0


@pytest.mark.skipif(not O.ref_available("d"), reason="reference not built in this checkout")
def test_oracle_exact_stepper_matches_reference_live():
    """dWorldStep on freshly seeded batched worlds against the reference built
    here: bit-identical states."""
    sc = S.batched_worlds(n_worlds=4, seed=31)
    with O.exact_stepper(O.oracle(), O.ref("d")):
        for w in range(sc.n_worlds):
            o = O.run_world(O.oracle().oracle_run_world, sc, w, 60)
            r = O.run_world(O.ref("d").ref_run_world, sc, w, 60)
            for k in ("ncontacts", "seeds", "state", "contacts"):
                assert np.array_equal(o[k], r[k]), k


@pytest.mark.skipif(not O.ref_available("d"), reason="reference not built in this checkout")
@pytest.mark.parametrize("seed", [21, 22])
def test_oracle_matches_reference_live(seed):
    sc = S.batched_worlds(n_worlds=3, seed=seed)
    for w in range(sc.n_worlds):
        o = O.run_world(O.oracle().oracle_run_world, sc, w, 50)
        r = O.run_world(O.ref("d").ref_run_world, sc, w, 50)
        for k in ("ncontacts", "seeds", "state", "contacts"):
            assert np.array_equal(o[k], r[k]), k


def test_scene_roundtrip():
    sc = S.hinge_chains(n_worlds=2, steps=5)
    sc2 = S.Scene.from_arrays(sc.to_arrays())
    for k in S.Scene._ARRAYS:
        assert np.array_equal(getattr(sc, k), getattr(sc2, k))
    assert np.array_equal(sc.joint_torque, sc2.joint_torque)


def test_multithreaded_baseline_is_deterministic():
    """The CPU-baseline entry (many worlds on host threads) gives the same
    result as running the worlds one by one."""
    sc = S.batched_worlds(n_worlds=6, seed=3)
    out = np.zeros((sc.nb_total, 13))
    O.oracle().oracle_run_worlds(C.byref(sc.c), 0, sc.n_worlds, 15, 4, out.ctypes.data_as(_P(C.c_double)))
    ref = np.concatenate([O.run_world(O.oracle().oracle_run_world, sc, w, 15)["state"][-1]
                          for w in range(sc.n_worlds)])
    assert np.array_equal(out, ref)


def test_vehicle_heightfield_cases_are_reference_precision_splits():
    """tests/golden/vehicle_hf_cases.npz: at each recorded world-step of the
    full-size vehicle rollout (FP32-rounded oracle state), the oracle's FP64
    contact count is the stored dDOUBLE one, and, where the reference is
    built here, its dSINGLE and dDOUBLE builds give the stored per-geom
    heightfield contact counts, which differ."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk_hf_cases", os.path.join(GOLDEN, "make_vehicle_hf_cases.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    from odegpu import scene as S
    g = np.load(os.path.join(GOLDEN, "vehicle_hf_cases.npz"))
    sc = S.vehicles(n_worlds=2048, steps=300)
    for i, (k, w) in enumerate(zip(g["step"], g["world"])):
        x32, n = mk.case_inputs(sc, int(k), int(w))
        assert n == g["contacts_double"][i], (k, w, n)
        if O.ref_available("d") and O.ref_available("s"):
            d = mk.hf_counts(sc, int(w), x32, "d")
            s_ = mk.hf_counts(sc, int(w), x32, "s")
            assert np.array_equal(d, g["hf_double"][i]) and np.array_equal(s_, g["hf_single"][i]), (k, w)
            assert not np.array_equal(d, s_)
