"""Rays (ODE's ray geom, dRayClass) on the GPU: dCollide through the ODE API
on the reference's known-answer calls, and the batched ray query
(odegpuBatchRayCast) against the FP64 oracle's dCollide over every geom of a
world, on stepped vehicle worlds (heightfield, box chassis, sphere wheels) and
on a large world."""
import ctypes as C
import os

import numpy as np
import pytest

from odegpu import scene as S
import oracle_lib as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_D = C.POINTER(C.c_double)


class ContactGeom(C.Structure):
    _fields_ = [("pos", C.c_float * 4), ("normal", C.c_float * 4), ("depth", C.c_float),
                ("g1", C.c_void_p), ("g2", C.c_void_p), ("side1", C.c_int), ("side2", C.c_int)]


def _api():
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dCreateSphere.restype = v; L.dCreateSphere.argtypes = [v, f]
    L.dCreateBox.restype = v; L.dCreateBox.argtypes = [v, f, f, f]
    L.dCreatePlane.restype = v; L.dCreatePlane.argtypes = [v, f, f, f, f]
    L.dCreateCapsule.restype = v; L.dCreateCapsule.argtypes = [v, f, f]
    L.dCreateRay.restype = v; L.dCreateRay.argtypes = [v, f]
    L.dGeomRaySet.argtypes = [v, f, f, f, f, f, f]
    L.dGeomRayGet.argtypes = [v, C.POINTER(f), C.POINTER(f)]
    L.dGeomRaySetLength.argtypes = [v, f]
    L.dGeomRayGetLength.restype = f; L.dGeomRayGetLength.argtypes = [v]
    L.dGeomRaySetParams.argtypes = [v, i, i]
    L.dGeomRayGetParams.argtypes = [v, C.POINTER(i), C.POINTER(i)]
    L.dGeomRaySetClosestHit.argtypes = [v, i]
    L.dGeomRayGetClosestHit.restype = i; L.dGeomRayGetClosestHit.argtypes = [v]
    L.dGeomGetClass.restype = i; L.dGeomGetClass.argtypes = [v]
    L.dGeomSetPosition.argtypes = [v, f, f, f]
    L.dGeomSetRotation.argtypes = [v, C.POINTER(f)]
    L.dGeomDestroy.argtypes = [v]
    L.dCollide.restype = i; L.dCollide.argtypes = [v, v, i, v, i]
    return L


def _R4(R):
    return (C.c_float * 12)(*[R[0], R[1], R[2], 0, R[3], R[4], R[5], 0, R[6], R[7], R[8], 0])


def test_ray_geom_accessors():
    """dCreateRay / dGeomRaySet (normalises the direction) / dGeomRayGet /
    length and flag accessors (ode/src/ray.cpp:92-194)."""
    L = _api()
    r = L.dCreateRay(None, 2.5)
    assert L.dGeomGetClass(r) == 5
    assert abs(L.dGeomRayGetLength(r) - 2.5) < 1e-7
    L.dGeomRaySet(r, 1.0, 2.0, 3.0, 0.0, 3.0, 4.0)
    s, d = (C.c_float * 4)(), (C.c_float * 4)()
    L.dGeomRayGet(r, s, d)
    assert np.allclose(list(s)[:3], [1, 2, 3]) and np.allclose(list(d)[:3], [0, 0.6, 0.8], atol=1e-7)
    L.dGeomRaySetLength(r, 0.5)
    assert abs(L.dGeomRayGetLength(r) - 0.5) < 1e-7
    fc, bc = C.c_int(), C.c_int()
    L.dGeomRaySetParams(r, 1, 0)
    L.dGeomRaySetClosestHit(r, 1)
    L.dGeomRayGetParams(r, C.byref(fc), C.byref(bc))
    assert (fc.value, bc.value, L.dGeomRayGetClosestHit(r)) == (1, 0, 1)
    L.dGeomRaySetClosestHit(r, 0)
    L.dGeomRayGetParams(r, C.byref(fc), C.byref(bc))
    assert (fc.value, bc.value, L.dGeomRayGetClosestHit(r)) == (1, 0, 0)
    L.dGeomDestroy(r)


def test_dcollide_rays_on_reference_kats():
    """dCollide of rays with sphere / box / capsule / plane in both argument
    orders (the reversed call negates the normal) and ray against ray (no
    collider), through the ODE API on the GPU, against the reference's FP64
    outputs: counts equal except for grazing rays (the reference's hit within
    1e-4 of the ray's end or of tangency), records within 1e-4."""
    g = np.load(os.path.join(GOLDEN, "ray_kats.npz"))
    L = _api()
    mk = {0: lambda p: L.dCreateSphere(None, p[0]), 1: lambda p: L.dCreateBox(None, p[0], p[1], p[2]),
          2: lambda p: L.dCreateCapsule(None, p[0], p[1]),
          4: lambda p: L.dCreatePlane(None, p[0], p[1], p[2], p[3]), 5: lambda p: L.dCreateRay(None, p[0])}
    n = len(g["t1"])
    mism, worst = [], 0.0
    for k in range(n):
        geoms = []
        for t, p, pos, R in ((g["t1"][k], g["p1"][k], g["pos1"][k], g["R1"][k]),
                             (g["t2"][k], g["p2"][k], g["pos2"][k], g["R2"][k])):
            h = mk[int(t)](p)
            if t != 4:
                L.dGeomSetPosition(h, *pos)
                L.dGeomSetRotation(h, _R4(R))
            geoms.append(h)
        out = (ContactGeom * 16)()
        nc = L.dCollide(geoms[0], geoms[1], int(g["flags"][k]), out, C.sizeof(ContactGeom))
        ref_n, ref = int(g["nc"][k]), g["out"][k]
        if nc != ref_n:
            mism.append(k)
        else:
            for c in range(nc):
                got = np.array(list(out[c].pos[:3]) + list(out[c].normal[:3]) + [out[c].depth])
                worst = max(worst, np.abs(got - ref[c, :7]).max())
        for h in geoms:
            L.dGeomDestroy(h)
    # a count mismatch is allowed only where FP32 rounding can flip the test:
    # the reference's hit (if any) lies within 1e-4 of the ray's end
    for k in mism:
        ray_len = g["p1"][k][0] if g["t1"][k] == 5 else g["p2"][k][0]
        ref = g["out"][k]
        assert g["nc"][k] == 1 and abs(ref[0, 6] - ray_len) < 1e-4 or g["nc"][k] == 0, k
    assert len(mism) <= n // 200, mism
    assert worst < 1e-4, worst


def _hf_api_geom(L, g):
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dGeomHeightfieldDataCreate.restype = v
    L.dGeomHeightfieldDataBuildDouble.argtypes = [v, _D, i, f, f, i, i, f, f, f, i]
    L.dCreateHeightfield.restype = v
    L.dCreateHeightfield.argtypes = [v, v, i]
    L.dGeomHeightfieldDataDestroy.argtypes = [v]
    h = np.ascontiguousarray(g["heights"], dtype=np.float64)
    sp = float(g["spacing"])
    nz, nx = h.shape
    hd = L.dGeomHeightfieldDataCreate()
    L.dGeomHeightfieldDataBuildDouble(hd, h.ctypes.data_as(_D), 1, sp * (nx - 1), sp * (nz - 1), nx, nz,
                                      1.0, 0.0, 1.0, 0)
    hg = L.dCreateHeightfield(None, hd, 1)
    L.dGeomSetPosition(hg, *[float(x) for x in g["hf_pos"]])
    L.dGeomSetRotation(hg, _R4(g["hf_R"]))
    return hd, hg


def test_dcollide_ray_heightfield_on_reference_kats():
    """dCollide(heightfield, ray) and dCollide(ray, heightfield) on the
    reference's golden calls (the plane pass with dCollideRayPlane,
    ode/src/heightfield.cpp:1035-1040, 1466-1530): counts exact, records
    within 1e-4."""
    g = np.load(os.path.join(GOLDEN, "ray_kats.npz"))
    ghf = np.load(os.path.join(GOLDEN, "hf_kats.npz"))
    L = _api()
    hd, hg = _hf_api_geom(L, ghf)
    m = len(g["hf_nc"])
    mism, worst = [], 0.0
    for k in range(m):
        r = L.dCreateRay(None, float(g["hf_p2"][k][0]))
        L.dGeomSetPosition(r, *g["hf_pos2"][k])
        L.dGeomSetRotation(r, _R4(g["hf_R2"][k]))
        ref_n, ref = int(g["hf_nc"][k]), g["hf_out"][k]
        for order, sgn in (((hg, r), 1.0), ((r, hg), -1.0)):
            out = (ContactGeom * 16)()
            nc = L.dCollide(order[0], order[1], int(g["hf_flags"][k]), out, C.sizeof(ContactGeom))
            if nc != ref_n:
                mism.append((k, nc, ref_n))
                continue
            for c in range(nc):
                got = np.array(list(out[c].pos[:3]) + [sgn * x for x in out[c].normal[:3]] + [out[c].depth])
                worst = max(worst, np.abs(got - ref[c, :7]).max())
        L.dGeomDestroy(r)
    L.dGeomDestroy(hg)
    L.dGeomHeightfieldDataDestroy(hd)
    assert not mism, mism[:10]
    assert worst < 1e-4, worst


# ---------------------------------------------------------------- batched ray queries

def _R_from_q(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _oracle_nearest(sc, state, ray, flags):
    """FP64 nearest hit: dCollide(ray, g, flags) of the oracle over every geom
    of the ray's world, least depth, lower geom index on ties."""
    L = O.oracle()
    w, b = int(ray["world"]), int(ray["body"])
    b0, _ = sc.world_bodies(w)
    g0, g1 = int(sc.geom_off[w]), int(sc.geom_off[w + 1])
    d = np.asarray(ray["dir"], np.float64)
    d = d / np.linalg.norm(d)
    s = np.asarray(ray["start"], np.float64)
    if b >= 0:
        st = state[b0 + b]
        R = _R_from_q(st[3:7] / np.linalg.norm(st[3:7]))
        s = st[0:3] + R @ s
        d = R @ d
    e = np.array([1.0, 0, 0]) if abs(d[0]) < 0.9 else np.array([0, 1.0, 0])
    x = np.cross(e, d); x /= np.linalg.norm(x)
    Rr = np.stack([x, np.cross(d, x), d], axis=1)
    pr = np.array([float(ray["length"]), 0, 0, 0])
    best = (np.inf, -1, None)
    fhf = L.oracle_collide_hf
    fhf.restype = C.c_int
    fhf.argtypes = [C.c_void_p, C.c_int, _D, _D, _D, C.c_int, _D]
    for gi in range(g0, g1):
        t = int(sc.geom_type[gi])
        gb = int(sc.geom_body[gi])
        if b >= 0 and gb == b:
            continue
        out = np.zeros((64, 9))
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in (pr, s, Rr.ravel())]
        if t == S.GEOM_HEIGHTFIELD:
            H = sc.heightfields[int(sc.geom_param[gi][0])]
            nc = fhf(C.byref(H), 5, *(a.ctypes.data_as(_D) for a in args), flags, out.ctypes.data_as(_D))
            out[:nc, 3:6] *= -1.0
        else:
            if gb >= 0:
                st = state[b0 + gb]
                pos, R = st[0:3], _R_from_q(st[3:7] / np.linalg.norm(st[3:7]))
            else:
                pos, R = np.zeros(3), np.eye(3)
            ga = [np.ascontiguousarray(a, dtype=np.float64) for a in (sc.geom_param[gi], pos, R.ravel())]
            nc = L.oracle_collide(5, *(a.ctypes.data_as(_D) for a in args), t,
                                  *(a.ctypes.data_as(_D) for a in ga), flags, out.ctypes.data_as(_D))
        for c in range(nc):
            if out[c, 6] < best[0]:
                best = (out[c, 6], gi - g0, out[c, :7].copy())
    return best


def _compare(sc, state, rays, hits, flags, tol):
    worst, flips = 0.0, 0
    nhit = 0
    for k in range(len(rays)):
        depth, gidx, rec = _oracle_nearest(sc, state, rays[k], flags)
        h = hits[k]
        if gidx < 0:
            assert h["geom"] == -1 or abs(h["depth"] - rays[k]["length"]) < 1e-4, (k, h)
            continue
        nhit += 1
        if h["geom"] != gidx:
            # two geoms at (nearly) the same distance, or a grazing hit
            flips += 1
            assert h["geom"] == -1 or abs(h["depth"] - depth) < 1e-4, (k, h, depth, gidx)
            continue
        got = np.concatenate([h["pos"], h["normal"], [h["depth"]]])
        worst = max(worst, np.abs(got - rec).max())
    assert worst < tol, worst
    assert flips <= max(1, len(rays) // 100), flips
    return nhit


def _vehicle_rays(sc, rng, per_world=12):
    rays = []
    for w in range(sc.n_worlds):
        # four suspension probes on the chassis (body 0), pointing down in its frame
        for ox, oy in ((0.7, 0.6), (0.7, -0.6), (-0.7, 0.6), (-0.7, -0.6)):
            rays.append((w, 0, (ox, oy, 0.0), (0.0, 0.0, -1.0), 2.0))
        b0, _ = sc.world_bodies(w)
        c = sc.body_pos[b0]
        # world-frame rays at the car; short enough that the heightfield zone
        # under each stays within the collider's 10 x 10 samples
        for _ in range(per_world - 4):
            start = c + rng.normal(size=3) * 0.8 + np.array([0, 0, 1.2])
            aim = c + rng.normal(size=3) * 0.6 - start
            rays.append((w, -1, tuple(start), tuple(aim), float(rng.uniform(1.0, 2.5))))
    return np.array(rays, dtype=_ray_dtype())


def _ray_dtype():
    from odegpu.batch import RAY_DTYPE
    return RAY_DTYPE


def test_batch_ray_cast_vehicles_vs_oracle():
    """Vehicle worlds after 30 steps: body-attached suspension probes (the
    chassis' own geoms skipped) and world-frame rays at the cars, against the
    oracle's FP64 dCollide over every geom of the world: the same geom hit,
    records within 2e-4 (rays of up to 2.5 m in FP32; 1e-3 for the rays of
    10 to 30 m)."""
    from odegpu.batch import Batch
    sc = S.vehicles(n_worlds=6, steps=40, hf_samples=64)
    B = Batch(sc)
    B.step(30)
    state = np.asarray(B.state(), np.float64)
    rng = np.random.Generator(np.random.PCG64(3))
    rays = _vehicle_rays(sc, rng)
    for flags in (1, 4):
        hits = B.ray_cast(rays, flags=flags)
        nhit = _compare(sc, state, rays, hits, flags, 2e-4)
        assert nhit > len(rays) // 2, nhit
        # every suspension probe hits the terrain or a wheel
        probes = hits[np.asarray(rays["body"]) == 0]
        assert (probes["geom"] >= 0).all(), probes
    # rays whose heightfield zone exceeds the lane's 10 x 10 samples (10 to
    # 30 m over the 0.5 m field): the host entry casts them again with a
    # workspace per warp and answers them as the oracle does; the device
    # entry, which has no workspace, refuses them (geom -3) rather than
    # answering from part of the zone
    import torch
    from odegpu.batch import HIT_DTYPE
    far = []
    for w in range(sc.n_worlds):
        b0, _ = sc.world_bodies(w)
        for _ in range(6):
            start = sc.body_pos[b0] + np.array([0, 0, 3.0]) + rng.normal(size=3)
            aim = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-0.25, -0.02)])
            far.append((w, -1, tuple(start), tuple(aim), float(rng.uniform(10.0, 30.0))))
    far = np.array(far, dtype=_ray_dtype())
    hits = B.ray_cast(far, flags=1)
    assert (hits["geom"] != -3).all(), hits["geom"]
    nhit = _compare(sc, state, far, hits, 1, 1e-3)
    assert nhit > len(far) // 4, nhit
    d_rays = torch.from_numpy(far.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(far) * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    B.ray_cast_async(d_rays.data_ptr(), len(far), d_hits.data_ptr(), flags=1)
    B.sync()
    assert (d_hits.cpu().numpy().view(HIT_DTYPE)["geom"] == -3).any()
    B.close()


def test_batch_ray_cast_async_and_invalid_rays():
    """The device-pointer entry on the batch stream gives the host entry's
    records; an invalid ray is an error on the host entry and geom = -2 on
    the device entry."""
    import torch
    from odegpu.batch import Batch, HIT_DTYPE
    from odegpu._lib import OdeGpuError
    sc = S.vehicles(n_worlds=3, steps=10, hf_samples=64)
    B = Batch(sc)
    B.step(5)
    rays = _vehicle_rays(sc, np.random.Generator(np.random.PCG64(4)), per_world=8)
    ref = B.ray_cast(rays, flags=2)
    bad = rays.copy()
    bad["world"][3] = 99
    bad["body"][5] = 50
    with pytest.raises(OdeGpuError, match="ray 3"):
        B.ray_cast(bad)
    d_rays = torch.from_numpy(bad.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(rays) * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    B.ray_cast_async(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), flags=2)
    B.sync()
    got = d_hits.cpu().numpy().view(HIT_DTYPE)
    assert got["geom"][3] == -2 and got["geom"][5] == -2
    keep = np.ones(len(rays), bool)
    keep[[3, 5]] = False
    assert np.array_equal(got[keep].view(np.uint8), ref[keep].view(np.uint8))
    B.close()


def test_batch_ray_cast_large_world():
    """A 600-sphere pile in a walled box (one large world): rays from above
    and through the walls against the oracle."""
    from odegpu.batch import Batch
    sc = S.sphere_pile(n=600, box=(2.5, 2.5, 4.0))
    B = Batch(sc)
    B.step(10)
    state = np.asarray(B.state(), np.float64)
    rng = np.random.Generator(np.random.PCG64(9))
    rays = []
    for _ in range(64):
        start = np.array([rng.uniform(-1.2, 1.2), rng.uniform(-1.2, 1.2), 6.0])
        d = np.array([rng.normal() * 0.2, rng.normal() * 0.2, -1.0])
        rays.append((0, -1, tuple(start), tuple(d), 10.0))
    for _ in range(16):
        start = rng.uniform(-1.0, 1.0, 3) + np.array([0, 0, 1.0])
        d = rng.normal(size=3)
        d[2] = -abs(d[2]) - 0.2   # downwards: the box has no lid
        rays.append((0, -1, tuple(start), tuple(d), 8.0))
    rays = np.array(rays, dtype=_ray_dtype())
    hits = B.ray_cast(rays)
    assert (B.status() == 0).all()
    nhit = _compare(sc, state, rays, hits, 1, 2e-4)
    assert nhit == len(rays)   # floor and walls catch every downward ray
    B.close()


def test_scene_rejects_ray_geoms():
    from odegpu.batch import Batch
    from odegpu._lib import OdeGpuError
    b = S.SceneBuilder()
    w = b.new_world()
    s = b.add_surface(0, 1.0)
    bi = b.add_body(w, (0, 0, 1), 1.0, (0.1, 0, 0, 0, 0.1, 0, 0, 0, 0.1))
    b.add_geom(w, S.GEOM_SPHERE, bi, (0.5,), s)
    b.add_geom(w, 5, bi, (1.0,), s)
    with pytest.raises(OdeGpuError, match="ray"):
        Batch(b.build())
