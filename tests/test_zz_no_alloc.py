"""odegpuCollideNoAlloc: the dCollide variant for callers that cannot
allocate device memory (its contact staging buffer is a fixed device array
inside the library). Checked through the C ABI against the allocating entry
point, dCollide of the ODE-compatible API, on the reference's collider poses
for every class it accepts (sphere, box, capsule, cylinder, plane, ray).

The array keeps the previous call's contents, so before every pose the test
makes a query that fills it (a deep box-box overlap, 8 contacts) and then
checks that the next call reports exactly dCollide's count and records, and
writes nothing past its count (the output is prefilled with a sentinel), on
two calls in a row. Named to be collected last."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_F = C.POINTER(C.c_float)
SENTINEL = -12345.0


class ContactGeom(C.Structure):
    _fields_ = [("pos", C.c_float * 4), ("normal", C.c_float * 4), ("depth", C.c_float),
                ("g1", C.c_void_p), ("g2", C.c_void_p), ("side1", C.c_int), ("side2", C.c_int)]


def _lib():
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.odegpuCollideNoAlloc.restype = i
    L.odegpuCollideNoAlloc.argtypes = [i, _F, _F, _F, i, _F, _F, _F, i, _F]
    L.dCreateSphere.restype = v; L.dCreateSphere.argtypes = [v, f]
    L.dCreateBox.restype = v; L.dCreateBox.argtypes = [v, f, f, f]
    L.dCreatePlane.restype = v; L.dCreatePlane.argtypes = [v, f, f, f, f]
    L.dCreateCapsule.restype = v; L.dCreateCapsule.argtypes = [v, f, f]
    L.dCreateCylinder.restype = v; L.dCreateCylinder.argtypes = [v, f, f]
    L.dCreateRay.restype = v; L.dCreateRay.argtypes = [v, f]
    L.dGeomSetPosition.argtypes = [v, f, f, f]
    L.dGeomSetRotation.argtypes = [v, _F]
    L.dGeomDestroy.argtypes = [v]
    L.dCollide.restype = i; L.dCollide.argtypes = [v, v, i, v, i]
    return L


def _fa(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    return a, a.ctypes.data_as(_F)


def _R4(R9):
    return np.hstack([np.asarray(R9, np.float64).reshape(3, 3), np.zeros((3, 1))]).ravel()


def _no_alloc(L, t1, a1, t2, a2, flags):
    out = np.full((8, 7), SENTINEL, np.float32)
    nc = L.odegpuCollideNoAlloc(t1, *a1, t2, *a2, flags, out.ctypes.data_as(_F))
    return nc, out


def _fill_array(L):
    """A deep face-face overlap of two unit boxes, the upper one turned 0.3 rad
    about z: the clipped faces meet in an octagon, 8 contacts, every slot of
    the array."""
    keep = []

    def geom(pos, ang):
        c, s = np.cos(ang), np.sin(ang)
        R = np.array([[c, -s, 0, 0], [s, c, 0, 0], [0, 0, 1, 0]])
        p, pp = _fa([1.0, 1.0, 1.0, 0.0]); x, px = _fa(pos); r, pr = _fa(R.ravel())
        keep.extend([p, x, r])
        return pp, px, pr
    nc, _ = _no_alloc(L, 1, geom([0, 0, 0], 0.0), 1, geom([0, 0, 0.5], 0.3), 8)
    assert nc == 8
    return keep


@pytest.mark.parametrize("fixture", ["collider_kats", "cylinder_kats", "ray_kats"])
def test_no_alloc_matches_dcollide_twice_in_a_row(fixture):
    g = np.load(os.path.join(GOLDEN, fixture + ".npz"))
    L = _lib()
    mk = {0: lambda p: L.dCreateSphere(None, p[0]), 1: lambda p: L.dCreateBox(None, p[0], p[1], p[2]),
          2: lambda p: L.dCreateCapsule(None, p[0], p[1]), 3: lambda p: L.dCreateCylinder(None, p[0], p[1]),
          4: lambda p: L.dCreatePlane(None, p[0], p[1], p[2], p[3]), 5: lambda p: L.dCreateRay(None, p[0])}
    n = len(g["t1"])
    idx = np.arange(0, n, 5)      # a spread of poses over every class pair
    compared = with_contacts = without = 0
    for k in idx:
        t1, t2, flags = int(g["t1"][k]), int(g["t2"][k]), int(g["flags"][k])
        R4 = [_R4(g["R1"][k]), _R4(g["R2"][k])]
        # existing entry point: dCollide on ODE-API geoms
        geoms = []
        for t, p, pos, R in ((t1, g["p1"][k], g["pos1"][k], R4[0]), (t2, g["p2"][k], g["pos2"][k], R4[1])):
            h = mk[t](p)
            if t != 4:
                L.dGeomSetPosition(h, *[float(x) for x in pos])
                _, rp = _fa(R)
                L.dGeomSetRotation(h, rp)
            geoms.append(h)
        cg = (ContactGeom * 16)()
        n_ref = L.dCollide(geoms[0], geoms[1], flags, cg, C.sizeof(ContactGeom))
        assert n_ref >= 0
        ref = np.array([list(cg[c].pos[:3]) + list(cg[c].normal[:3]) + [cg[c].depth] for c in range(n_ref)])
        for h in geoms:
            L.dGeomDestroy(h)
        # new entry point, twice, after a call that left 8 contacts in the array
        args, keep = [], []
        for p, pos, R in ((g["p1"][k], g["pos1"][k], R4[0]), (g["p2"][k], g["pos2"][k], R4[1])):
            a1, p1 = _fa(p); a2, p2 = _fa(pos); a3, p3 = _fa(R)
            keep += [a1, a2, a3]
            args.append((p1, p2, p3))
        keep += _fill_array(L)
        for _ in range(2):
            nc, out = _no_alloc(L, t1, args[0], t2, args[1], flags)
            assert nc == n_ref, (k, nc, n_ref)
            if nc:
                np.testing.assert_allclose(out[:nc], ref, rtol=0, atol=1e-5)
            assert (out[nc:] == SENTINEL).all(), k
        compared += 1
        with_contacts += n_ref > 0
        without += n_ref == 0
    assert compared > 100 and with_contacts > 20 and without > 5


def test_no_alloc_rejects_too_many_contacts_and_other_classes():
    from odegpu._lib import lib
    L = _lib()
    a, pa = _fa([0.5, 0, 0, 0]); z, pz = _fa([0, 0, 0]); I, pI = _fa(np.eye(3, 4).ravel())
    out = np.full((16, 7), SENTINEL, np.float32)
    rc = L.odegpuCollideNoAlloc(0, pa, pz, pI, 0, pa, pz, pI, 9, out.ctypes.data_as(_F))
    assert rc < 0
    assert b"at most 8" in lib().odegpuGetLastError()
    for bad in (9, 6, -1):           # heightfield, an unknown class, a negative class
        rc = L.odegpuCollideNoAlloc(0, pa, pz, pI, bad, pa, pz, pI, 4, out.ctypes.data_as(_F))
        assert rc < 0 and b"class" in lib().odegpuGetLastError(), bad
    assert (out == SENTINEL).all()
