"""Cylinders (ODE's flat-ended dCylinderClass) on the GPU: dCollide through the
ODE API on the reference's known-answer calls, dCollide(heightfield,
cylinder), cylinder mass, and batched ray queries into a stepped cylinder
pile against the oracle.

The FP32 colliders keep the reference's FP32 (dSINGLE) tolerances, so the
bar is the reference's own dSINGLE build on the same calls (out_s / nc_s in
the fixture): contact counts exact, records within 1e-4. Where a
cylinder-box contact normal is a box face normal up to rounding, the
reference's face clipping starts from a vertex chosen by rounding noise (its
dSINGLE and dDOUBLE builds differ there too); the GPU may break that tie
either way but must return points of the reference's full contact set."""
import ctypes as C
import os

import numpy as np
import pytest

from odegpu import scene as S
import oracle_lib as O
from test_gpu_ray import ContactGeom, _R4, _api, _hf_api_geom, _compare, _ray_dtype

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cyl_api():
    L = _api()
    f, v = C.c_float, C.c_void_p
    L.dCreateCylinder.restype = v
    L.dCreateCylinder.argtypes = [v, f, f]
    L.dGeomCylinderGetParams.argtypes = [v, C.POINTER(f), C.POINTER(f)]
    L.dGeomCylinderSetParams.argtypes = [v, f, f]
    return L


def _rows(out, n, sgn=1.0):
    return np.array([list(out[c].pos[:3]) + [sgn * x for x in out[c].normal[:3]] + [out[c].depth]
                     for c in range(n)]).reshape(n, 7)


def test_cylinder_geom_and_mass():
    """dCreateCylinder / dGeomCylinderSet/GetParams (ode/src/cylinder.cpp:76-103)
    and dMassSetCylinder[Total] / dMassSetCapsule[Total] / dMassAdjust
    (ode/src/mass.cpp:140-200, 441-451) against closed forms."""
    from test_gpu_ode_api import Mass
    L = _cyl_api()
    g = L.dCreateCylinder(None, 0.3, 1.2)
    r, l = C.c_float(), C.c_float()
    L.dGeomCylinderGetParams(g, C.byref(r), C.byref(l))
    assert abs(r.value - 0.3) < 1e-7 and abs(l.value - 1.2) < 1e-7
    L.dGeomCylinderSetParams(g, 0.5, 0.25)
    L.dGeomCylinderGetParams(g, C.byref(r), C.byref(l))
    assert abs(r.value - 0.5) < 1e-7 and abs(l.value - 0.25) < 1e-7
    L.dGeomDestroy(g)
    f, i = C.c_float, C.c_int
    m = Mass()
    L.dMassSetCylinder.argtypes = [C.c_void_p, f, i, f, f]
    L.dMassSetCylinder(C.byref(m), 1000.0, 3, 0.3, 1.2)
    M = np.pi * 0.09 * 1.2 * 1000.0
    I = M * (0.25 * 0.09 + 1.44 / 12)
    assert abs(m.mass - M) < 1e-3 * M
    assert np.allclose([m.I[0], m.I[5], m.I[10]], [I, I, 0.5 * M * 0.09], rtol=1e-5)
    L.dMassSetCapsuleTotal.argtypes = [C.c_void_p, f, i, f, f]
    L.dMassSetCapsuleTotal(C.byref(m), 7.0, 1, 0.2, 0.6)
    assert abs(m.mass - 7.0) < 1e-5
    M1, M2 = np.pi * 0.04 * 0.6, 4.0 / 3.0 * np.pi * 0.008
    Ia = M1 * (0.25 * 0.04 + 0.36 / 12) + M2 * (0.4 * 0.04 + 0.375 * 0.2 * 0.6 + 0.25 * 0.36)
    Ib = (M1 * 0.5 + M2 * 0.4) * 0.04
    s = 7.0 / (M1 + M2)
    assert np.allclose([m.I[0], m.I[5], m.I[10]], [Ib * s, Ia * s, Ia * s], rtol=1e-5)


def test_dcollide_cylinders_on_reference_kats():
    """dCollide with cylinders (sphere / box / plane in both orders, rays into
    cylinders, cylinder-cylinder and capsule-cylinder without a collider)
    through the ODE API on the GPU, against the reference's dSINGLE outputs."""
    g = np.load(os.path.join(GOLDEN, "cylinder_kats.npz"))
    L = _cyl_api()
    mk = {0: lambda p: L.dCreateSphere(None, p[0]), 1: lambda p: L.dCreateBox(None, p[0], p[1], p[2]),
          2: lambda p: L.dCreateCapsule(None, p[0], p[1]), 3: lambda p: L.dCreateCylinder(None, p[0], p[1]),
          4: lambda p: L.dCreatePlane(None, p[0], p[1], p[2], p[3]), 5: lambda p: L.dCreateRay(None, p[0])}
    n = len(g["t1"])
    count_mism, value_mism, tie = [], [], 0
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
        for h in geoms:
            L.dGeomDestroy(h)
        ns = int(g["nc_s"][k])
        if nc != ns:
            count_mism.append((k, nc, ns))
            continue
        if nc == 0:
            continue
        got = _rows(out, nc)
        err = np.abs(got - g["out_s"][k][:nc, :7]).max()
        if err < 1e-4:
            continue
        # A tie: the contact normal is a box face normal up to rounding, so
        # which face vertex the clipped polygon starts from (and, when fewer
        # contacts are asked for than the polygon has, which of its equally
        # deep points are returned) hangs on rounding noise. Every returned
        # point must then be one of the reference's full contact set.
        full = g["out_s_all"][k][:int(g["nc_s_all"][k]), :7]
        if all(np.abs(full - r).max(axis=1).min() < 1e-4 for r in got):
            tie += 1
        else:
            value_mism.append((k, int(g["t1"][k]), int(g["t2"][k]), err))
    assert len(count_mism) <= n // 500, count_mism
    assert not value_mism, value_mism[:10]
    assert tie <= n // 50, tie


def test_dcollide_heightfield_cylinder_on_reference_kats():
    """dCollide(heightfield, cylinder) and the reversed call (normals negated):
    the plane pass with dCollideCylinderPlane and, for cylinders wider than
    1.5 cells, the vertex pass casting rays into the cylinder
    (ode/src/heightfield.cpp:1062-1068, 1562-1584); against the reference's
    dSINGLE outputs: counts exact, records within 1e-4."""
    g = np.load(os.path.join(GOLDEN, "cylinder_kats.npz"))
    ghf = np.load(os.path.join(GOLDEN, "hf_kats.npz"))
    L = _cyl_api()
    hd, hg = _hf_api_geom(L, ghf)
    m = len(g["hf_nc"])
    mism, worst = [], 0.0
    for k in range(m):
        p = g["hf_p2"][k]
        cy = L.dCreateCylinder(None, float(p[0]), float(p[1]))
        L.dGeomSetPosition(cy, *g["hf_pos2"][k])
        L.dGeomSetRotation(cy, _R4(g["hf_R2"][k]))
        ns, ref = int(g["hf_nc_s"][k]), g["hf_out_s"][k]
        for order, sgn in (((hg, cy), 1.0), ((cy, hg), -1.0)):
            out = (ContactGeom * 16)()
            nc = L.dCollide(order[0], order[1], int(g["hf_flags"][k]), out, C.sizeof(ContactGeom))
            if nc != ns:
                mism.append((k, nc, ns))
                continue
            if nc:
                worst = max(worst, np.abs(_rows(out, nc, sgn) - ref[:nc, :7]).max())
        L.dGeomDestroy(cy)
    L.dGeomDestroy(hg)
    L.dGeomHeightfieldDataDestroy(hd)
    assert len(mism) <= 2, mism
    assert worst < 1e-4, worst


def test_batch_ray_cast_into_cylinder_pile():
    """Rays from above into the stepped cylinder pile (plane and heightfield
    worlds): the nearest hit among cylinders, spheres, boxes and the ground
    agrees with the oracle's FP64 dCollide over every geom."""
    from odegpu.batch import Batch
    sc = S.cylinder_pile(n_worlds=2)
    B = Batch(sc)
    B.step(60)
    state = np.asarray(B.state(), np.float64)
    rng = np.random.Generator(np.random.PCG64(12))
    rays = []
    for w in range(sc.n_worlds):
        for _ in range(48):
            start = np.array([rng.uniform(-1.0, 1.0), rng.uniform(-1.0, 1.0), 2.0])
            d = np.array([rng.normal() * 0.1, rng.normal() * 0.1, -1.0])
            rays.append((w, -1, tuple(start), tuple(d), 2.6))
    rays = np.array(rays, dtype=_ray_dtype())
    hits = B.ray_cast(rays)
    assert (hits["geom"] != -3).all()
    nhit = _compare(sc, state, rays, hits, 1, 2e-4)
    assert nhit > len(rays) * 3 // 4, nhit
    B.close()
