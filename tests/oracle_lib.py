"""ctypes access to the test-only libraries: the CPU oracle (oracle/liboracle.so)
and, where it was built in this checkout, the reference ODE 0.12 harness
(oracle/_ref/libode_ref_d.so). Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_P = C.POINTER


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)


def _bind(lib, prefix):
    f = getattr(lib, prefix + "_run_world")
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_double), _P(C.c_int), _P(C.c_double),
                  C.c_int, _P(C.c_double), _P(C.c_uint)]
    return f


_oracle = None
_ref = {}


def oracle():
    global _oracle
    if _oracle is None:
        path = os.path.join(ORACLE_DIR, "liboracle.so")
        if not os.path.exists(path):
            build_oracle()
        lib = C.CDLL(path)
        _bind(lib, "oracle")
        lib.oracle_run_worlds.restype = C.c_longlong
        lib.oracle_run_worlds.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                          _P(C.c_double)]
        lib.oracle_collide.restype = C.c_int
        lib.oracle_collide.argtypes = [C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_double),
                                       C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_double),
                                       C.c_int, _P(C.c_double)]
        lib.oracle_rand_int.argtypes = [C.c_int]
        lib.oracle_rand_set_seed.argtypes = [C.c_uint]
        lib.oracle_rand_get_seed.restype = C.c_uint
        lib.oracle_run_world_from.restype = C.c_int
        lib.oracle_run_world_from.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_double),
                                              _P(C.c_double)]
        lib.oracle_step_worlds_from.restype = C.c_int
        lib.oracle_step_worlds_from.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                _P(C.c_double), _P(C.c_uint), _P(C.c_double), _P(C.c_uint),
                                                _P(C.c_int)]
        lib.oracle_step_world_contacts.restype = C.c_int
        lib.oracle_step_world_contacts.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(C.c_double), C.c_uint,
                                                   _P(C.c_double), C.c_int, _P(C.c_double)]
        lib.oracle_set_stepper.argtypes = [C.c_int]
        lib.oracle_lcp_errors.restype = C.c_int
        _oracle = lib
    return _oracle


def ref_available(prec="d"):
    return os.path.exists(os.path.join(ORACLE_DIR, "_ref", f"libode_ref_{prec}.so"))


def ref(prec="d"):
    if prec not in _ref:
        lib = C.CDLL(os.path.join(ORACLE_DIR, "_ref", f"libode_ref_{prec}.so"))
        _bind(lib, "ref")
        lib.ref_collide.restype = C.c_int
        lib.ref_collide.argtypes = oracle().oracle_collide.argtypes
        lib.ref_rand_int.argtypes = [C.c_int]
        lib.ref_rand_set_seed.argtypes = [C.c_uint]
        lib.ref_rand_get_seed.restype = C.c_uint
        lib.ref_set_stepper.argtypes = [C.c_int]
        _ref[prec] = lib
    return _ref[prec]


def run_world(fn, scene, w, n_steps, max_rec=512, feedback=False):
    """Call a *_run_world entry; returns dict of numpy arrays."""
    b0, b1 = scene.world_bodies(w)
    j0, j1 = scene.world_joints(w)
    nb, nj = b1 - b0, j1 - j0
    state = np.zeros((n_steps + 1, nb, 13))
    ncont = np.zeros(n_steps, np.int32)
    cont = np.zeros((n_steps, max_rec, 9))
    fb = np.zeros((n_steps, max(nj, 1), 12)) if feedback else None
    seeds = np.zeros(n_steps, np.uint32)
    rc = fn(C.byref(scene.c), w, n_steps, state.ctypes.data_as(_P(C.c_double)),
            ncont.ctypes.data_as(_P(C.c_int)), cont.ctypes.data_as(_P(C.c_double)), max_rec,
            fb.ctypes.data_as(_P(C.c_double)) if feedback else None,
            seeds.ctypes.data_as(_P(C.c_uint)))
    assert rc == 0
    return dict(state=state, ncontacts=ncont, contacts=cont, feedback=fb, seeds=seeds)


class OracleTap(C.Structure):
    _fields_ = [("n_islands", C.c_int), ("island_rows", _P(C.c_int)),
                ("island_bodies", _P(C.c_int)), ("cap_islands", C.c_int),
                ("J", _P(C.c_double)), ("rhs", _P(C.c_double)), ("cfm", _P(C.c_double)),
                ("lo", _P(C.c_double)), ("hi", _P(C.c_double)), ("findex", _P(C.c_int)),
                ("jb", _P(C.c_int)), ("cap_rows", C.c_int), ("body_of", _P(C.c_int)),
                ("cap_bodies", C.c_int), ("lambda_", _P(C.c_double)), ("cforce", _P(C.c_double)),
                ("joint_of_row", _P(C.c_int)), ("seed_before", C.c_uint)]


def tap_step(scene, w, pre_steps, cap_rows=4096, cap_bodies=1024):
    """Oracle stage taps of step `pre_steps` of world w (see ode_oracle.h)."""
    L = oracle()
    L.oracle_tap_step.restype = C.c_int
    L.oracle_tap_step.argtypes = [C.c_void_p, C.c_int, C.c_int, _P(OracleTap)]
    a = dict(island_rows=np.zeros(cap_bodies, np.int32), island_bodies=np.zeros(cap_bodies, np.int32),
             J=np.zeros((cap_rows, 12)), rhs=np.zeros(cap_rows), cfm=np.zeros(cap_rows),
             lo=np.zeros(cap_rows), hi=np.zeros(cap_rows), findex=np.zeros(cap_rows, np.int32),
             jb=np.zeros((cap_rows, 2), np.int32), body_of=np.zeros(cap_bodies, np.int32),
             lam=np.zeros(cap_rows), cforce=np.zeros((cap_bodies, 6)),
             joint_of_row=np.zeros(cap_rows, np.int32))
    t = OracleTap()
    t.cap_islands = cap_bodies
    t.cap_rows = cap_rows
    t.cap_bodies = cap_bodies
    for k in ("island_rows", "island_bodies", "findex", "jb", "body_of", "joint_of_row"):
        setattr(t, k, a[k].ctypes.data_as(_P(C.c_int)))
    for k in ("J", "rhs", "cfm", "lo", "hi", "cforce"):
        setattr(t, k, a[k].ctypes.data_as(_P(C.c_double)))
    t.lambda_ = a["lam"].ctypes.data_as(_P(C.c_double))
    total = L.oracle_tap_step(C.byref(scene.c), w, pre_steps, C.byref(t))
    assert total >= 0
    n = t.n_islands
    a["n_islands"] = n
    a["total_rows"] = total
    a["seed_before"] = t.seed_before
    a["island_rows"] = a["island_rows"][:n]
    a["island_bodies"] = a["island_bodies"][:n]
    return a


def run_world_from(scene, w, n_steps, init_state):
    """Oracle world w built from the scene, body state replaced by init_state
    ([nb, 13]), n_steps steps; returns the final state [nb, 13]."""
    x0 = np.ascontiguousarray(init_state, dtype=np.float64)
    out = np.zeros_like(x0)
    rc = oracle().oracle_run_world_from(C.byref(scene.c), w, n_steps, x0.ctypes.data_as(_P(C.c_double)),
                                        out.ctypes.data_as(_P(C.c_double)))
    assert rc == 0
    return out


def step_worlds_from(scene, step0, n_steps, state=None, seeds=None, w_begin=0, w_end=None, threads=None,
                     counts=True):
    """Worlds [w_begin, w_end) stepped n_steps times (as steps step0, ...)
    from `state` ([bodies of the range, 13], FP64; None: the scene's initial
    state) and `seeds` (None: the scene's), on all host threads. Returns
    (final state [nb, 13], seeds after [n], counts [n, n_steps, 3] of
    contacts / rows / islands with rows, or None)."""
    w_end = scene.n_worlds if w_end is None else w_end
    nbr = int(scene.body_off[w_end] - scene.body_off[w_begin])
    out = np.zeros((nbr, 13))
    so = np.zeros(w_end - w_begin, np.uint32)
    cnt = np.zeros((w_end - w_begin, n_steps, 3), np.int32) if counts else None
    xin = None if state is None else np.ascontiguousarray(state, dtype=np.float64)
    sin = None if seeds is None else np.ascontiguousarray(seeds, dtype=np.uint32)
    rc = oracle().oracle_step_worlds_from(
        C.byref(scene.c), w_begin, w_end, step0, n_steps, threads or (os.cpu_count() or 1),
        None if xin is None else xin.ctypes.data_as(_P(C.c_double)),
        None if sin is None else sin.ctypes.data_as(_P(C.c_uint)),
        out.ctypes.data_as(_P(C.c_double)), so.ctypes.data_as(_P(C.c_uint)),
        None if cnt is None else cnt.ctypes.data_as(_P(C.c_int)))
    assert rc == 0
    return out, so, cnt


def step_world_contacts(scene, w, step, state, seed, max_rec=65536):
    """One oracle step of world w from `state` ([nb, 13]) with `seed`:
    (contacts [n, 9] pos normal depth gi gk, state after [nb, 13])."""
    x = np.ascontiguousarray(state, dtype=np.float64)
    out = np.zeros((max_rec, 9))
    after = np.zeros_like(x)
    n = oracle().oracle_step_world_contacts(C.byref(scene.c), w, step, x.ctypes.data_as(_P(C.c_double)),
                                            int(seed), out.ctypes.data_as(_P(C.c_double)), max_rec,
                                            after.ctypes.data_as(_P(C.c_double)))
    assert n >= 0
    return out[:min(n, max_rec)], after


class exact_stepper:
    """Within the block the oracle (and, when given, the reference library)
    steps worlds with dWorldStep instead of dWorldQuickStep."""

    def __init__(self, *libs):
        self.libs = libs or (oracle(),)

    def __enter__(self):
        for lib in self.libs:
            (lib.oracle_set_stepper if hasattr(lib, "oracle_set_stepper") else lib.ref_set_stepper)(1)
        return self

    def __exit__(self, *exc):
        for lib in self.libs:
            (lib.oracle_set_stepper if hasattr(lib, "oracle_set_stepper") else lib.ref_set_stepper)(0)
        return False
