"""Generates vehicle_hf_cases.npz: the inputs of the full-size vehicle rollout
(2048 cars on the 256 x 256 heightfield, tests/test_gpu_full_size.py) at which
the REFERENCE's two builds, dSINGLE and dDOUBLE, disagree on the heightfield's
contacts with one of the car's geoms, and the contact count of the dSINGLE
build there.

Each case is a step k and world w of the oracle's FP64 rollout, its state
rounded to FP32 (what the GPU stores and steps from). For every geom of the
world, dCollide(heightfield, geom) runs in the reference built from its own
sources (oracle/_ref, make -C oracle ref) in both precisions; the world's
contact count with the dSINGLE answers in place of the dDOUBLE ones is stored.
The GPU's heightfield collider is FP32 and follows the dSINGLE build, so at
these inputs the GPU's count is the dSINGLE one.

The list of (k, w) is the set of world-steps where the GPU's count differed
from the FP64 oracle's in that rollout; this script confirms, from the
reference alone, that every one of them is a dSINGLE / dDOUBLE split.

    make -C oracle ref && python tests/golden/make_vehicle_hf_cases.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ode-0.12_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

from odegpu import scene as S  # noqa: E402
import oracle_lib as O  # noqa: E402

CASES = [(50, 647), (161, 419), (165, 419), (199, 1316), (210, 1053), (211, 1814), (259, 1930)]
_P = C.POINTER(C.c_double)


def r_from_q(q):
    """dRfromQ (ode/src/rotation.cpp:236-255) of the quaternion as given."""
    w, x, y, z = q
    return np.array([[w * w + x * x - y * y - z * z, 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), w * w - x * x + y * y - z * z, 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), w * w - x * x - y * y + z * z]])


def hf_counts(sc, w, x32, prec):
    """dCollide(heightfield, g) contact count of every non-heightfield geom of
    world w at state x32, in the reference built with precision prec."""
    f = O.ref(prec).ref_collide_hf
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, _P, _P, _P, C.c_int, _P]
    out = []
    for g in range(int(sc.geom_off[w]), int(sc.geom_off[w + 1])):
        if sc.geom_type[g] == S.GEOM_HEIGHTFIELD:
            continue
        st = x32[sc.geom_body[g]]
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sc.geom_param[g], st[0:3], r_from_q(st[3:7]).ravel())]
        res = np.zeros((64, 9))
        out.append(f(C.byref(sc.heightfields[0]), int(sc.geom_type[g]), *(v.ctypes.data_as(_P) for v in a),
                     int(sc.world_params[w].max_contacts), res.ctypes.data_as(_P)))
    return np.array(out, np.int32)


def case_inputs(sc, k, w):
    x, seeds, _ = O.step_worlds_from(sc, 0, k, w_begin=w, w_end=w + 1, counts=False)
    x32 = x.astype(np.float32).astype(np.float64)
    _, _, c = O.step_worlds_from(sc, k, 1, state=x32, seeds=seeds, w_begin=w, w_end=w + 1)
    return x32, int(c[0, 0, 0])


def main():
    sc = S.vehicles(n_worlds=2048, steps=300)
    rows = []
    for k, w in CASES:
        x32, n_oracle = case_inputs(sc, k, w)
        d, s = hf_counts(sc, w, x32, "d"), hf_counts(sc, w, x32, "s")
        assert not np.array_equal(d, s), (k, w)
        rows.append((k, w, n_oracle, n_oracle - int(d.sum()) + int(s.sum()), d, s))
    np.savez_compressed(os.path.join(HERE, "vehicle_hf_cases.npz"),
                        step=np.array([r[0] for r in rows], np.int32), world=np.array([r[1] for r in rows], np.int32),
                        contacts_double=np.array([r[2] for r in rows], np.int32),
                        contacts_single=np.array([r[3] for r in rows], np.int32),
                        hf_double=np.stack([r[4] for r in rows]), hf_single=np.stack([r[5] for r in rows]))
    for r in rows:
        print(f"step {r[0]} world {r[1]}: contacts dDOUBLE {r[2]}, dSINGLE {r[3]}")


if __name__ == "__main__":
    main()
