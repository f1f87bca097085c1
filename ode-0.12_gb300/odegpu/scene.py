"""Seeded scene descriptions (``odegpuScene``) and the workload generators.

A :class:`Scene` owns numpy arrays laid out exactly as ``include/odegpu_scene.h``
describes and exposes them as a ctypes ``odegpuScene`` for libodegpu (and for
the CPU oracle used by the tests). Generators build the workloads this project
measures; each uses numpy's PCG64 generator with an explicit seed so every
consumer sees identical inputs.

Mass properties follow ODE's dMassSetBox / dMassSetSphere formulas
(ode/src/mass.cpp:118-124, :201-215) evaluated in FP64.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

GEOM_SPHERE, GEOM_BOX, GEOM_CAPSULE, GEOM_CYLINDER, GEOM_PLANE, GEOM_RAY, GEOM_HEIGHTFIELD = 0, 1, 2, 3, 4, 5, 9
JOINT_BALL, JOINT_HINGE, JOINT_SLIDER, JOINT_CONTACT, JOINT_UNIVERSAL, JOINT_HINGE2, JOINT_FIXED = \
    1, 2, 3, 4, 5, 6, 7
JOINT_AMOTOR = 9
AMOTOR_USER, AMOTOR_EULER = 0, 1
BODY_GYROSCOPIC, BODY_NO_GRAVITY = 1, 2

CONTACT_MU2 = 0x001
CONTACT_BOUNCE = 0x004
CONTACT_SOFT_ERP = 0x008
CONTACT_SOFT_CFM = 0x010
CONTACT_APPROX1 = 0x3000

GEOM_NPARAM = 4
JOINT_NPARAM = 36
INF = float("inf")


class Surface(C.Structure):
    _fields_ = [("mode", C.c_int)] + [(n, C.c_double) for n in (
        "mu", "mu2", "bounce", "bounce_vel", "soft_erp", "soft_cfm",
        "motion1", "motion2", "motionN", "slip1", "slip2")]


class WorldParams(C.Structure):
    _fields_ = [("gravity", C.c_double * 3), ("erp", C.c_double), ("cfm", C.c_double),
                ("iterations", C.c_int), ("sor_w", C.c_double), ("max_vel", C.c_double),
                ("min_depth", C.c_double), ("dt", C.c_double), ("max_contacts", C.c_int),
                ("seed", C.c_uint)]


class Heightfield(C.Structure):
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("width", C.c_double), ("depth", C.c_double),
                ("scale", C.c_double), ("offset", C.c_double), ("thickness", C.c_double),
                ("wrap", C.c_int), ("heights", C.POINTER(C.c_double)),
                ("pos", C.c_double * 3), ("R", C.c_double * 9)]


_P = C.POINTER


class CScene(C.Structure):
    _fields_ = [
        ("n_worlds", C.c_int),
        ("body_off", _P(C.c_int)), ("geom_off", _P(C.c_int)), ("joint_off", _P(C.c_int)),
        ("world", _P(WorldParams)),
        ("body_pos", _P(C.c_double)), ("body_q", _P(C.c_double)), ("body_lvel", _P(C.c_double)),
        ("body_avel", _P(C.c_double)), ("body_mass", _P(C.c_double)), ("body_I", _P(C.c_double)),
        ("body_flags", _P(C.c_int)),
        ("geom_type", _P(C.c_int)), ("geom_body", _P(C.c_int)), ("geom_param", _P(C.c_double)),
        ("geom_surface", _P(C.c_int)),
        ("surfaces", _P(Surface)), ("n_surfaces", C.c_int),
        ("heightfields", _P(Heightfield)), ("n_heightfields", C.c_int),
        ("joint_type", _P(C.c_int)), ("joint_body", _P(C.c_int)), ("joint_anchor", _P(C.c_double)),
        ("joint_axis1", _P(C.c_double)), ("joint_axis2", _P(C.c_double)),
        ("joint_param", _P(C.c_double)),
        ("n_ctrl_steps", C.c_int), ("joint_torque", _P(C.c_double)), ("body_force", _P(C.c_double)),
        ("joint_stop", _P(C.c_double)),
    ]


def _ptr(a, ctype):
    if a is None:
        return C.cast(None, _P(ctype))
    return a.ctypes.data_as(_P(ctype))


def box_mass(density, lx, ly, lz):
    """dMassSetBox (ode/src/mass.cpp:201-215): mass and diagonal inertia."""
    m = lx * ly * lz * density
    return m, np.diag([m / 12.0 * (ly * ly + lz * lz), m / 12.0 * (lx * lx + lz * lz),
                       m / 12.0 * (lx * lx + ly * ly)])


def box_mass_total(m, lx, ly, lz):
    return m, np.diag([m / 12.0 * (ly * ly + lz * lz), m / 12.0 * (lx * lx + lz * lz),
                       m / 12.0 * (lx * lx + ly * ly)])


def sphere_mass(density, r):
    """dMassSetSphere (ode/src/mass.cpp:118-124)."""
    m = (4.0 / 3.0) * math.pi * r * r * r * density
    return sphere_mass_total(m, r)


def capsule_mass(density, r, length):
    """dMassSetCapsule (ode/src/mass.cpp:125-155) with the axis along z:
    mass and body-frame inertia of a cylinder of `length` with two
    hemispherical caps."""
    M1 = math.pi * r * r * length * density
    M2 = 4.0 / 3.0 * math.pi * r ** 3 * density
    m = M1 + M2
    Ia = M1 * (0.25 * r * r + length * length / 12.0) + \
        M2 * (0.4 * r * r + 0.375 * r * length + 0.25 * length * length)
    Iz = (0.5 * M1 + 0.4 * M2) * r * r
    return m, np.diag([Ia, Ia, Iz])


def cylinder_mass(density, r, length):
    """dMassSetCylinder (ode/src/mass.cpp:173-200) with the axis along z."""
    m = math.pi * r * r * length * density
    i = m * (0.25 * r * r + length * length / 12.0)
    return m, np.diag([i, i, 0.5 * m * r * r])


def sphere_mass_total(m, r):
    ii = 0.4 * m * r * r
    return m, np.diag([ii, ii, ii])


class SceneBuilder:
    """Accumulates worlds object by object; :meth:`build` freezes into a Scene."""

    def __init__(self):
        self.worlds = []
        self.surfaces = []
        self.heightfields = []   # (Heightfield kwargs, heights array)

    def add_surface(self, mode, mu, mu2=0.0, bounce=0.0, bounce_vel=0.0, soft_erp=0.0,
                    soft_cfm=0.0):
        self.surfaces.append(dict(mode=mode, mu=mu, mu2=mu2, bounce=bounce,
                                  bounce_vel=bounce_vel, soft_erp=soft_erp, soft_cfm=soft_cfm))
        return len(self.surfaces) - 1

    def add_heightfield(self, heights, width, depth, scale=1.0, offset=0.0, thickness=1.0,
                        wrap=0, pos=(0, 0, 0), R=np.eye(3)):
        h = np.ascontiguousarray(heights, dtype=np.float64)
        self.heightfields.append((dict(nx=h.shape[1], nz=h.shape[0], width=width, depth=depth,
                                       scale=scale, offset=offset, thickness=thickness,
                                       wrap=wrap, pos=tuple(pos),
                                       R=tuple(np.asarray(R, float).ravel())), h))
        return len(self.heightfields) - 1

    def new_world(self, gravity=(0, 0, -9.81), erp=0.2, cfm=1e-5, iterations=20, sor_w=1.3,
                  max_vel=INF, min_depth=0.0, dt=0.01, max_contacts=4, seed=0):
        w = dict(params=dict(gravity=gravity, erp=erp, cfm=cfm, iterations=iterations,
                             sor_w=sor_w, max_vel=max_vel, min_depth=min_depth, dt=dt,
                             max_contacts=max_contacts, seed=seed),
                 bodies=[], geoms=[], joints=[])
        self.worlds.append(w)
        return w

    @staticmethod
    def add_body(w, pos, mass, I, q=(1, 0, 0, 0), lvel=(0, 0, 0), avel=(0, 0, 0),
                 flags=BODY_GYROSCOPIC):
        w["bodies"].append(dict(pos=pos, q=q, lvel=lvel, avel=avel, mass=mass,
                                I=np.asarray(I, float).reshape(9), flags=flags))
        return len(w["bodies"]) - 1

    @staticmethod
    def add_geom(w, gtype, body, param, surface=0):
        p = list(param) + [0.0] * (GEOM_NPARAM - len(param))
        w["geoms"].append(dict(type=gtype, body=body, param=p, surface=surface))
        return len(w["geoms"]) - 1

    @staticmethod
    def add_joint(w, jtype, b1, b2, anchor=(0, 0, 0), axis1=(1, 0, 0), axis2=(0, 1, 0),
                  param=None):
        p = np.zeros(JOINT_NPARAM)
        if param is not None:
            p[:len(param)] = param
        w["joints"].append(dict(type=jtype, b=(b1, b2), anchor=anchor, axis1=axis1,
                                axis2=axis2, param=p))
        return len(w["joints"]) - 1

    def build(self):
        return Scene(self)


def limot_params(lostop=-INF, histop=INF, vel=0.0, fmax=0.0, fudge=1.0, bounce=0.0,
                 cfm=1e-5, stop_erp=0.2, stop_cfm=1e-5):
    return [lostop, histop, vel, fmax, fudge, bounce, cfm, stop_erp, stop_cfm]


class Scene:
    """Frozen, contiguous arrays + the ctypes view (``self.c``)."""

    def __init__(self, b: SceneBuilder):
        W = b.worlds
        self.n_worlds = len(W)
        nbs = [len(w["bodies"]) for w in W]
        ngs = [len(w["geoms"]) for w in W]
        njs = [len(w["joints"]) for w in W]
        self.body_off = np.concatenate([[0], np.cumsum(nbs)]).astype(np.int32)
        self.geom_off = np.concatenate([[0], np.cumsum(ngs)]).astype(np.int32)
        self.joint_off = np.concatenate([[0], np.cumsum(njs)]).astype(np.int32)
        bodies = [bd for w in W for bd in w["bodies"]]
        geoms = [g for w in W for g in w["geoms"]]
        joints = [j for w in W for j in w["joints"]]
        f64 = np.float64

        def arr(key, objs, width, dtype=f64):
            if not objs:
                return np.zeros((1, width) if width else 1, dtype=dtype)
            return np.ascontiguousarray(np.array([o[key] for o in objs], dtype=dtype))

        self.body_pos = arr("pos", bodies, 3)
        self.body_q = arr("q", bodies, 4)
        self.body_lvel = arr("lvel", bodies, 3)
        self.body_avel = arr("avel", bodies, 3)
        self.body_mass = arr("mass", bodies, 0)
        self.body_I = arr("I", bodies, 9)
        self.body_flags = arr("flags", bodies, 0, np.int32)
        self.geom_type = arr("type", geoms, 0, np.int32)
        self.geom_body = arr("body", geoms, 0, np.int32)
        self.geom_param = arr("param", geoms, GEOM_NPARAM)
        self.geom_surface = arr("surface", geoms, 0, np.int32)
        self.joint_type = arr("type", joints, 0, np.int32)
        self.joint_body = arr("b", joints, 2, np.int32)
        self.joint_anchor = arr("anchor", joints, 3)
        self.joint_axis1 = arr("axis1", joints, 3)
        self.joint_axis2 = arr("axis2", joints, 3)
        self.joint_param = arr("param", joints, JOINT_NPARAM)
        self.world_params = (WorldParams * max(1, self.n_worlds))()
        for i, w in enumerate(W):
            p = w["params"]
            wp = self.world_params[i]
            wp.gravity[:] = list(p["gravity"])
            for k in ("erp", "cfm", "iterations", "sor_w", "max_vel", "min_depth", "dt",
                      "max_contacts", "seed"):
                setattr(wp, k, p[k])
        surfs = b.surfaces or [dict(mode=0, mu=0.0)]
        self.surfaces = (Surface * len(surfs))()
        for i, s in enumerate(surfs):
            for k, v in s.items():
                setattr(self.surfaces[i], k, v)
        self.hf_heights = [h for _, h in b.heightfields]
        self.heightfields = (Heightfield * max(1, len(b.heightfields)))()
        for i, (kw, h) in enumerate(b.heightfields):
            H = self.heightfields[i]
            for k in ("nx", "nz", "width", "depth", "scale", "offset", "thickness", "wrap"):
                setattr(H, k, kw[k])
            H.heights = h.ctypes.data_as(_P(C.c_double))
            H.pos[:] = list(kw["pos"])
            H.R[:] = list(kw["R"])
        self.n_heightfields = len(b.heightfields)
        self.n_ctrl_steps = 0
        self.joint_torque = None
        self.body_force = None
        self.joint_stop = None
        self.nb_total = int(self.body_off[-1])
        self.nj_total = int(self.joint_off[-1])
        self.ng_total = int(self.geom_off[-1])
        self._refresh()

    def set_controls(self, joint_torque=None, body_force=None, joint_stop=None):
        """Per-step controls: joint_torque [S][nj_total][2] (hinge torque,
        hinge2 / universal torque pair, slider force), body_force
        [S][nb_total][6], joint_stop [S][nj_total] (hinge / hinge2 / universal
        / slider limot1 lostop = histop before the step; NaN keeps the joint's
        own stops)."""
        S = 0
        if joint_torque is not None:
            self.joint_torque = np.ascontiguousarray(joint_torque, dtype=np.float64)
            S = self.joint_torque.shape[0]
        if body_force is not None:
            self.body_force = np.ascontiguousarray(body_force, dtype=np.float64)
            S = self.body_force.shape[0]
        if joint_stop is not None:
            self.joint_stop = np.ascontiguousarray(joint_stop, dtype=np.float64)
            S = self.joint_stop.shape[0]
        self.n_ctrl_steps = S
        self._refresh()

    def _refresh(self):
        c = CScene()
        c.n_worlds = self.n_worlds
        c.body_off = _ptr(self.body_off, C.c_int)
        c.geom_off = _ptr(self.geom_off, C.c_int)
        c.joint_off = _ptr(self.joint_off, C.c_int)
        c.world = C.cast(self.world_params, _P(WorldParams))
        for k in ("body_pos", "body_q", "body_lvel", "body_avel", "body_mass", "body_I",
                  "geom_param", "joint_anchor", "joint_axis1", "joint_axis2", "joint_param"):
            setattr(c, k, _ptr(getattr(self, k), C.c_double))
        for k in ("body_flags", "geom_type", "geom_body", "geom_surface", "joint_type",
                  "joint_body"):
            setattr(c, k, _ptr(getattr(self, k), C.c_int))
        c.surfaces = C.cast(self.surfaces, _P(Surface))
        c.n_surfaces = len(self.surfaces)
        c.heightfields = C.cast(self.heightfields, _P(Heightfield))
        c.n_heightfields = self.n_heightfields
        c.n_ctrl_steps = self.n_ctrl_steps
        c.joint_torque = _ptr(self.joint_torque, C.c_double)
        c.body_force = _ptr(self.body_force, C.c_double)
        c.joint_stop = _ptr(self.joint_stop, C.c_double)
        self.c = c

    _ARRAYS = ("body_off", "geom_off", "joint_off", "body_pos", "body_q", "body_lvel",
               "body_avel", "body_mass", "body_I", "body_flags", "geom_type", "geom_body",
               "geom_param", "geom_surface", "joint_type", "joint_body", "joint_anchor",
               "joint_axis1", "joint_axis2", "joint_param")

    def to_arrays(self):
        """Flat dict of numpy arrays that round-trips through from_arrays."""
        out = {k: getattr(self, k) for k in self._ARRAYS}
        out["world_params"] = np.array(
            [[*wp.gravity, wp.erp, wp.cfm, wp.iterations, wp.sor_w, wp.max_vel, wp.min_depth,
              wp.dt, wp.max_contacts, wp.seed] for wp in self.world_params[:self.n_worlds]])
        out["surfaces"] = np.array([[s.mode, s.mu, s.mu2, s.bounce, s.bounce_vel, s.soft_erp,
                                     s.soft_cfm, s.motion1, s.motion2, s.motionN, s.slip1, s.slip2]
                                    for s in self.surfaces])
        if self.joint_torque is not None:
            out["joint_torque"] = self.joint_torque
        if self.body_force is not None:
            out["body_force"] = self.body_force
        if self.joint_stop is not None:
            out["joint_stop"] = self.joint_stop
        if self.n_heightfields > 0:
            out["hf_meta"] = np.array([[H.nx, H.nz, H.width, H.depth, H.scale, H.offset, H.thickness, H.wrap,
                                        *H.pos[:], *H.R[:]] for H in self.heightfields[:self.n_heightfields]])
            for i, h in enumerate(self.hf_heights):
                out[f"hf_heights_{i}"] = h
        return out

    @classmethod
    def from_arrays(cls, a):
        self = cls.__new__(cls)
        for k in cls._ARRAYS:
            setattr(self, k, np.ascontiguousarray(a[k]))
        jp = self.joint_param.reshape(len(self.joint_type), -1)
        if jp.shape[1] < JOINT_NPARAM:   # fixtures written with fewer parameters per joint
            jp = np.concatenate([jp, np.zeros((jp.shape[0], JOINT_NPARAM - jp.shape[1]))], axis=1)
        self.joint_param = np.ascontiguousarray(jp)
        self.n_worlds = len(self.body_off) - 1
        wpa = np.asarray(a["world_params"])
        self.world_params = (WorldParams * max(1, self.n_worlds))()
        for i, r in enumerate(wpa):
            wp = self.world_params[i]
            wp.gravity[:] = [float(x) for x in r[:3]]
            wp.erp, wp.cfm = float(r[3]), float(r[4])
            wp.iterations = int(r[5])
            wp.sor_w, wp.max_vel, wp.min_depth, wp.dt = (float(x) for x in r[6:10])
            wp.max_contacts = int(r[10])
            wp.seed = int(r[11])
        sa = np.asarray(a["surfaces"])
        self.surfaces = (Surface * len(sa))()
        for i, r in enumerate(sa):
            self.surfaces[i].mode = int(r[0])
            for k, v in zip(("mu", "mu2", "bounce", "bounce_vel", "soft_erp", "soft_cfm",
                             "motion1", "motion2", "motionN", "slip1", "slip2"), r[1:]):
                setattr(self.surfaces[i], k, float(v))
        self.hf_heights = []
        self.heightfields = (Heightfield * 1)()
        self.n_heightfields = 0
        if "hf_meta" in a:
            meta = np.asarray(a["hf_meta"])
            self.heightfields = (Heightfield * len(meta))()
            for i, r in enumerate(meta):
                h = np.ascontiguousarray(a[f"hf_heights_{i}"], dtype=np.float64)
                self.hf_heights.append(h)
                H = self.heightfields[i]
                H.nx, H.nz = int(r[0]), int(r[1])
                H.width, H.depth, H.scale, H.offset, H.thickness = (float(x) for x in r[2:7])
                H.wrap = int(r[7])
                H.heights = h.ctypes.data_as(_P(C.c_double))
                H.pos[:] = [float(x) for x in r[8:11]]
                H.R[:] = [float(x) for x in r[11:20]]
            self.n_heightfields = len(meta)
        self.n_ctrl_steps = 0
        self.joint_torque = None
        self.body_force = None
        self.joint_stop = None
        self.nb_total = int(self.body_off[-1])
        self.nj_total = int(self.joint_off[-1])
        self.ng_total = int(self.geom_off[-1])
        jt = a["joint_torque"] if "joint_torque" in a else None
        bf = a["body_force"] if "body_force" in a else None
        js = a["joint_stop"] if "joint_stop" in a else None
        if jt is not None or bf is not None or js is not None:
            self.set_controls(jt, bf, js)
        else:
            self._refresh()
        return self

    def world_bodies(self, w):
        return int(self.body_off[w]), int(self.body_off[w + 1])

    def world_joints(self, w):
        return int(self.joint_off[w]), int(self.joint_off[w + 1])


# --------------------------------------------------------------------------
# workload generators

def _std_surface(b, mu=0.5):
    return b.add_surface(CONTACT_APPROX1 | CONTACT_SOFT_ERP | CONTACT_SOFT_CFM, mu,
                         soft_erp=0.2, soft_cfm=1e-5)


def box_drop(seed=0, n_boxes=20, steps_hint=200):
    """20 boxes, edges U[0.2,1.0] m, density 1000, x,y in U[-3,3], z in U[0.5,5],
    identity orientation, onto plane z=0; g=-9.81, dt=0.01, 20 iterations, w=1.3,
    mu=0.5, Approx1|SoftERP|SoftCFM, soft_erp 0.2, soft_cfm 1e-5, <=4 contacts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    w = b.new_world(cfm=1e-5, seed=seed & 0xFFFFFFFF)
    b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
    for _ in range(n_boxes):
        lx, ly, lz = rng.uniform(0.2, 1.0, 3)
        x, y = rng.uniform(-3, 3, 2)
        z = rng.uniform(0.5, 5)
        m, I = box_mass(1000.0, lx, ly, lz)
        bi = b.add_body(w, (x, y, z), m, I)
        b.add_geom(w, GEOM_BOX, bi, (lx, ly, lz), s)
    return b.build()


def batched_worlds(n_worlds=4096, seed=1, nmin=4, nmax=64):
    """Independent worlds of uneven size: N in [4,64] log-uniform bodies per world,
    each a sphere (r U[0.1,0.5]) or a box (edges U[0.2,1.0]) with p=0.5, density
    1000, on plane z=0; about 25% of bodies linked into ball-joint chains of 2-6
    links. Surface and stepping as in box_drop. Bodies are placed with x,y in
    U[-3,3], z in U[0.5,5]; chain links are laid out along x from their first
    body, 0.6 m apart, ball anchors midway."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    lo, hi = math.log(nmin), math.log(nmax + 1)
    for wi in range(n_worlds):
        n = int(math.floor(math.exp(rng.uniform(lo, hi))))
        n = max(nmin, min(nmax, n))
        w = b.new_world(cfm=1e-5, seed=int(rng.integers(0, 2**32)))
        b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
        # decide chains: pick ~25% of the bodies, group them into chains of 2..6
        n_chain_bodies = int(round(0.25 * n))
        chains = []
        left = n_chain_bodies
        while left >= 2:
            L = int(rng.integers(2, 7))
            L = min(L, left)
            chains.append(L)
            left -= L
        chain_start = {}
        idx = 0
        for L in chains:
            chain_start[idx] = L
            idx += L
        i = 0
        while i < n:
            L = chain_start.get(i, 1)
            x0, y0 = rng.uniform(-3, 3, 2)
            z0 = rng.uniform(0.5, 5)
            prev = -1
            for k in range(L):
                pos = (x0 + 0.6 * k, y0, z0)
                if rng.uniform() < 0.5:
                    r = rng.uniform(0.1, 0.5)
                    m, I = sphere_mass(1000.0, r)
                    bi = b.add_body(w, pos, m, I)
                    b.add_geom(w, GEOM_SPHERE, bi, (r,), s)
                else:
                    lx, ly, lz = rng.uniform(0.2, 1.0, 3)
                    m, I = box_mass(1000.0, lx, ly, lz)
                    bi = b.add_body(w, pos, m, I)
                    b.add_geom(w, GEOM_BOX, bi, (lx, ly, lz), s)
                if prev >= 0:
                    anchor = (x0 + 0.6 * k - 0.3, y0, z0)
                    b.add_joint(w, JOINT_BALL, prev, bi, anchor=anchor, param=(0.2, 1e-5))
                prev = bi
            i += L
    return b.build()


def box_stack(n_worlds=1, height=5, seed=3, spacing=0.0):
    """Non-chaotic stacks: `height` unit boxes (0.5 m, density 1000) resting
    exactly on each other on plane z=0, tiny seeded horizontal offsets (<1 mm)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    for wi in range(n_worlds):
        w = b.new_world(cfm=1e-5, seed=int(rng.integers(0, 2**32)))
        b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
        L = 0.5
        for k in range(height):
            m, I = box_mass(1000.0, L, L, L)
            dx, dy = rng.uniform(-1e-3, 1e-3, 2)
            bi = b.add_body(w, (dx + spacing * wi, dy, L / 2 + k * L - 1e-3 * (k + 1)), m, I)
            b.add_geom(w, GEOM_BOX, bi, (L, L, L), s)
    return b.build()


def hinge_chains(n_worlds=1024, links=8, seed=4, steps=100, plane_z=-2.0):
    """Differentiable batch: each world an 8-link hinge chain of 0.5x0.1x0.1 m,
    1 kg boxes along x, the first link hinged to the static environment, hinge
    axes along y, initial joint angles U[-0.5,0.5] rad (applied as a planar
    rotation about y accumulated down the chain) and joint rates U[-1,1] rad/s;
    per-step hinge torques U[-2,2] N m; the end link can touch plane z=plane_z
    (-2 m)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    L = 0.5
    for wi in range(n_worlds):
        w = b.new_world(cfm=1e-5, seed=int(rng.integers(0, 2**32)))
        b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, plane_z), s)
        angles = rng.uniform(-0.5, 0.5, links)
        rates = rng.uniform(-1.0, 1.0, links)
        theta = 0.0
        omega = 0.0
        joint_pt = np.zeros(3)
        vel_pt = np.zeros(3)
        prev = -1
        for k in range(links):
            theta += angles[k]
            omega += rates[k]
            # link direction in the x-z plane after rotating about y by theta
            d = np.array([math.cos(theta), 0.0, -math.sin(theta)])
            center = joint_pt + 0.5 * L * d
            # rotation about y by theta: q = (cos(t/2), 0, sin(t/2), 0)
            q = (math.cos(theta / 2), 0.0, math.sin(theta / 2), 0.0)
            wvec = np.array([0.0, omega, 0.0])
            vcenter = vel_pt + np.cross(wvec, center - joint_pt)
            m, I = box_mass_total(1.0, L, 0.1, 0.1)
            bi = b.add_body(w, tuple(center), m, I, q=q, lvel=tuple(vcenter), avel=tuple(wvec))
            b.add_geom(w, GEOM_BOX, bi, (L, 0.1, 0.1), s)
            b.add_joint(w, JOINT_HINGE, prev if prev >= 0 else bi, bi if prev >= 0 else -1,
                        anchor=tuple(joint_pt), axis1=(0, 1, 0),
                        param=limot_params(cfm=1e-5, stop_erp=0.2, stop_cfm=1e-5))
            vel_pt = vcenter + np.cross(wvec, joint_pt + L * d - center)
            joint_pt = joint_pt + L * d
            prev = bi
    sc = b.build()
    tq = np.zeros((steps, sc.nj_total, 2))
    tq[:, :, 0] = rng.uniform(-2, 2, (steps, sc.nj_total))
    sc.set_controls(joint_torque=tq)
    return sc


def capsule_mix(seed=6, n_bodies=12):
    """Capsules (r U[0.1,0.3], length U[0.2,0.8]), spheres and boxes dropped on
    plane z=0 on a 2 m grid (so capsules meet only the plane: capsule-box,
    capsule-sphere and capsule-capsule are not on this path); same surface as
    box_drop."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    w = b.new_world(cfm=1e-5, seed=seed)
    b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
    for k in range(n_bodies):
        x, y = 2.0 * (k % 4) + rng.uniform(-0.2, 0.2), 2.0 * (k // 4) + rng.uniform(-0.2, 0.2)
        z = rng.uniform(0.3, 3)
        ang = rng.uniform(-1, 1, 3)
        qv = np.concatenate([[1.0], 0.5 * ang])
        qv /= np.linalg.norm(qv)
        kind = k % 3
        if kind == 0:
            r, L = rng.uniform(0.1, 0.3), rng.uniform(0.2, 0.8)
            m, I = sphere_mass(1000.0, r)  # inertia of a comparable sphere
            bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
            b.add_geom(w, GEOM_CAPSULE, bi, (r, L), s)
        elif kind == 1:
            r = rng.uniform(0.1, 0.4)
            m, I = sphere_mass(1000.0, r)
            bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
            b.add_geom(w, GEOM_SPHERE, bi, (r,), s)
        else:
            lx, ly, lz = rng.uniform(0.2, 0.8, 3)
            m, I = box_mass(1000.0, lx, ly, lz)
            bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
            b.add_geom(w, GEOM_BOX, bi, (lx, ly, lz), s)
    return b.build()


def cylinder_pile(seed=21, n_bodies=14, n_worlds=2):
    """Cylinders (r U[0.1,0.3], length U[0.2,0.8]), spheres and boxes dropped
    into a 1.6 x 1.6 m column, density 1000, same surface as box_drop. World 0
    lands on plane z=0; world 1 on a seeded 32 x 32 fractal heightfield (0.25
    m spacing, heights sigma 0.15) placed with its up axis along world z.
    Covers cylinder-sphere, cylinder-box, cylinder-plane and
    heightfield-cylinder (the field's vertex pass casts rays into the
    cylinder); cylinder-cylinder has no collider without libccd, so cylinders
    pass through each other as in the reference."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    hf = None
    for wi in range(n_worlds):
        w = b.new_world(cfm=1e-5, seed=seed + wi)
        if wi % 2 == 0:
            b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
        else:
            if hf is None:
                h = fractal_heights(32, 0.15, seed=seed)
                hf = b.add_heightfield(h, 0.25 * 31, 0.25 * 31, thickness=1.0, pos=(0, 0, 0), R=np.array(HF_Z_UP))
            b.add_geom(w, GEOM_HEIGHTFIELD, -1, (hf,), s)
        for k in range(n_bodies):
            x, y = rng.uniform(-0.8, 0.8, 2)
            z = 0.6 + 0.45 * k + rng.uniform(0, 0.2)
            qv = rng.normal(size=4)
            qv /= np.linalg.norm(qv)
            kind = k % 3
            if kind == 0 or kind == 2 and k % 2:
                r, L = rng.uniform(0.1, 0.3), rng.uniform(0.2, 0.8)
                m, I = cylinder_mass(1000.0, r, L)
                bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
                b.add_geom(w, GEOM_CYLINDER, bi, (r, L), s)
            elif kind == 1:
                r = rng.uniform(0.1, 0.3)
                m, I = sphere_mass(1000.0, r)
                bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
                b.add_geom(w, GEOM_SPHERE, bi, (r,), s)
            else:
                lx, ly, lz = rng.uniform(0.2, 0.6, 3)
                m, I = box_mass(1000.0, lx, ly, lz)
                bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
                b.add_geom(w, GEOM_BOX, bi, (lx, ly, lz), s)
    return b.build()


def capsule_pile(seed=12, n_bodies=14):
    """Capsules (r U[0.1,0.25], length U[0.2,0.8]), spheres and boxes dropped
    into a 1.6 x 1.6 m column onto plane z=0, so capsules land on each other
    and on spheres and boxes (capsule-sphere, capsule-box, capsule-capsule);
    density 1000, same surface as box_drop."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    w = b.new_world(cfm=1e-5, seed=seed)
    b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
    for k in range(n_bodies):
        x, y = rng.uniform(-0.8, 0.8, 2)
        z = 0.4 + 0.45 * k
        qv = np.concatenate([[1.0], rng.uniform(-1, 1, 3)])
        qv /= np.linalg.norm(qv)
        kind = k % 3
        if kind == 0:
            r, L = rng.uniform(0.1, 0.25), rng.uniform(0.2, 0.8)
            m, I = capsule_mass(1000.0, r, L)
            bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
            b.add_geom(w, GEOM_CAPSULE, bi, (r, L), s)
        elif kind == 1:
            r = rng.uniform(0.1, 0.3)
            m, I = sphere_mass(1000.0, r)
            bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
            b.add_geom(w, GEOM_SPHERE, bi, (r,), s)
        else:
            lx, ly, lz = rng.uniform(0.2, 0.6, 3)
            m, I = box_mass(1000.0, lx, ly, lz)
            bi = b.add_body(w, (x, y, z), m, I, q=tuple(qv))
            b.add_geom(w, GEOM_BOX, bi, (lx, ly, lz), s)
    return b.build()


def sphere_pyramid(n_worlds=1, levels=3, r=0.25, seed=8, spacing=4.0):
    """Non-chaotic stack: a triangular pyramid of equal spheres (levels 3 -> 6
    base + 3 + 1) settled on plane z=0, mu=0.5; sphere-sphere contacts have no
    feature ties, so FP32 and FP64 trajectories stay close. Worlds are placed
    `spacing` apart with sub-mm seeded jitter."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    for wi in range(n_worlds):
        w = b.new_world(cfm=1e-5, seed=int(rng.integers(0, 2**32)))
        b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
        d = 2 * r
        h = d * math.sqrt(2.0 / 3.0)
        for lv in range(levels):
            n = levels - lv
            z = r + lv * h - 1e-4
            # triangular layer of side n, centred over the layer below
            cx = lv * d / 2.0
            cy = lv * d / (2.0 * math.sqrt(3.0))
            for i in range(n):
                for j in range(n - i):
                    x = cx + (j + 0.5 * i) * d + spacing * wi
                    y = cy + i * d * math.sqrt(3.0) / 2.0
                    jit = rng.uniform(-1e-4, 1e-4, 2)
                    m, I = sphere_mass(1000.0, r)
                    bi = b.add_body(w, (x + jit[0], y + jit[1], z), m, I)
                    b.add_geom(w, GEOM_SPHERE, bi, (r,), s)
    return b.build()


def box_tower(n_worlds=1, height=5, seed=9, spacing=4.0, shrink=0.8, yaw=0.3):
    """Stack of boxes of decreasing size (edge 0.6 m * shrink**k), each yawed by
    `yaw`*k rad about z, resting on plane z=0 (1 mm initial overlap)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.5)
    for wi in range(n_worlds):
        w = b.new_world(cfm=1e-5, seed=int(rng.integers(0, 2**32)))
        b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
        z = 0.0
        for k in range(height):
            L = 0.6 * shrink ** k
            H = 0.3 * shrink ** k
            m, I = box_mass(1000.0, L, L, H)
            a = yaw * k + rng.uniform(-0.01, 0.01)
            q = (math.cos(a / 2), 0.0, 0.0, math.sin(a / 2))
            jit = rng.uniform(-1e-3, 1e-3, 2)
            bi = b.add_body(w, (spacing * wi + jit[0], jit[1], z + H / 2 - 1e-3), m, I, q=q)
            b.add_geom(w, GEOM_BOX, bi, (L, L, H), s)
            z += H - 1e-3
    return b.build()


def fractal_heights(n=256, sigma=0.3, beta=3.0, seed=11):
    """Seeded fractal terrain: white noise shaped to a 1/f^beta power spectrum
    (FFT), normalised to standard deviation sigma; [n, n] (z rows, x columns)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    noise = rng.standard_normal((n, n))
    fx = np.fft.fftfreq(n)[None, :]
    fz = np.fft.fftfreq(n)[:, None]
    f = np.sqrt(fx * fx + fz * fz)
    f[0, 0] = 1.0
    spec = np.fft.fft2(noise) / f ** (beta / 2)
    spec[0, 0] = 0.0
    h = np.real(np.fft.ifft2(spec))
    return h * (sigma / h.std())


# rotation about x by +90 degrees: the heightfield's local y (up) becomes world z
HF_Z_UP = ((1.0, 0.0, 0.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))


def _hf_height_at(h, spacing, wx, wy):
    """Bilinear terrain height under world (wx, wy) for a centred HF_Z_UP field."""
    n = h.shape[0]
    half = 0.5 * spacing * (n - 1)
    lx, lz = wx + half, -wy + half
    i, k = lx / spacing, lz / spacing
    i0, k0 = int(np.clip(np.floor(i), 0, n - 2)), int(np.clip(np.floor(k), 0, n - 2))
    fi, fk = i - i0, k - k0
    return ((1 - fi) * (1 - fk) * h[k0, i0] + fi * (1 - fk) * h[k0, i0 + 1] +
            (1 - fi) * fk * h[k0 + 1, i0] + fi * fk * h[k0 + 1, i0 + 1])


def vehicles(n_worlds=2048, seed=10, steps=300, hf_samples=256, spacing=0.5, sigma=0.3):
    """Vehicle batch: per world one car, a 2.0 x 1.0 x 0.5 m box chassis of
    1000 kg on four sphere wheels (r 0.35 m, 20 kg) attached by hinge2 joints
    (axis 1 vertical for steering and suspension, axis 2 the wheel axle;
    suspension ERP 0.4, CFM 0.01), on one shared seeded fractal heightfield of
    hf_samples^2 samples at `spacing` m (heights sigma), placeable with its up
    axis along world z. Wheel surface mu 1.2, mu2 0.8 (Mu2 | Approx1 | SoftERP |
    SoftCFM). Per step: steering angle U[-0.4, 0.4] rad on the front wheels as
    limot1 lostop = histop (the rear wheels' steering held at 0 the same way),
    and throttle U[0,1] * 400 N m as hinge2 torque2 on each rear wheel
    (dJointAddHinge2Torques). Each car starts at a seeded spot and heading of
    the field, just above the terrain."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = fractal_heights(hf_samples, sigma, seed=seed + 1)
    width = spacing * (hf_samples - 1)
    b = SceneBuilder()
    hf = b.add_heightfield(h, width, width, thickness=1.0, pos=(0, 0, 0), R=np.array(HF_Z_UP))
    s_ground = b.add_surface(CONTACT_MU2 | CONTACT_APPROX1 | CONTACT_SOFT_ERP | CONTACT_SOFT_CFM, 1.2,
                             mu2=0.8, soft_erp=0.2, soft_cfm=1e-5)
    r_w, m_w = 0.35, 20.0
    lx, ly, lz = 2.0, 1.0, 0.5
    wheel_off = [(0.7, 0.6), (0.7, -0.6), (-0.7, 0.6), (-0.7, -0.6)]   # front left/right, rear
    drop = 0.3                                                         # wheel centre below chassis
    for wi in range(n_worlds):
        w = b.new_world(cfm=1e-5, seed=int(rng.integers(0, 2**32)))
        b.add_geom(w, GEOM_HEIGHTFIELD, -1, (hf,), s_ground)
        cx, cy = rng.uniform(-0.4 * width, 0.4 * width, 2)
        yaw = rng.uniform(0, 2 * math.pi)
        c, sn = math.cos(yaw), math.sin(yaw)
        wheels = [(cx + c * ox - sn * oy, cy + sn * ox + c * oy) for ox, oy in wheel_off]
        ground = max(_hf_height_at(h, spacing, x, y) for x, y in wheels)
        zc = ground + r_w + 0.05 + drop
        q = (math.cos(yaw / 2), 0.0, 0.0, math.sin(yaw / 2))
        m, I = box_mass_total(1000.0, lx, ly, lz)
        ch = b.add_body(w, (cx, cy, zc), m, I, q=q)
        b.add_geom(w, GEOM_BOX, ch, (lx, ly, lz), s_ground)
        axle = (-sn, c, 0.0)
        for (x, y) in wheels:
            mw, Iw = sphere_mass_total(m_w, r_w)
            wb = b.add_body(w, (x, y, zc - drop), mw, Iw, q=q)
            b.add_geom(w, GEOM_SPHERE, wb, (r_w,), s_ground)
            p = np.zeros(JOINT_NPARAM)
            p[0:9] = limot_params(lostop=0.0, histop=0.0)
            p[9:18] = limot_params()
            p[18], p[19] = 0.4, 0.01
            b.add_joint(w, JOINT_HINGE2, ch, wb, anchor=(x, y, zc - drop), axis1=(0, 0, 1), axis2=axle,
                        param=p)
    sc = b.build()
    nj = sc.nj_total
    steer = rng.uniform(-0.4, 0.4, (steps, n_worlds))
    throttle = rng.uniform(0.0, 1.0, (steps, n_worlds)) * 400.0
    stops = np.zeros((steps, nj))
    tq = np.zeros((steps, nj, 2))
    for wi in range(n_worlds):
        j0 = sc.joint_off[wi]
        stops[:, j0 + 0] = steer[:, wi]
        stops[:, j0 + 1] = steer[:, wi]
        tq[:, j0 + 2, 1] = throttle[:, wi]
        tq[:, j0 + 3, 1] = throttle[:, wi]
    sc.set_controls(joint_torque=tq, joint_stop=stops)
    return sc


def _unit(v):
    v = np.asarray(v, float)
    return v / np.linalg.norm(v)


def mechanisms(n_worlds=256, seed=13, steps=200):
    """Joint-type batch: per world, on a ground plane z=0, five mechanisms
    side by side 2.5 m apart along x (seeded per world):
      0. rail: a 0.4x0.2x0.2 m, 2 kg box on a slider to the environment along a
         near-horizontal axis; stops -/+U[0.2,0.5] m, a motor (vel U[-1,1] m/s,
         fmax 20 N) in half the worlds, stop bounce 0.3 in a third; per-step
         slider force U[-10,10] N, and in every third block of 10 steps a servo
         stop lostop = histop = U[-0.2,0.2] m.
      1. drop rail: a 0.3 m, 1 kg cube on a slider attached the other way round
         (body 1 = environment, so the joint is reversed) along a near-vertical
         axis, falling onto the plane; per-step slider force U[-10,10] N (a
         reversed slider's dJointAddSliderForce adds nothing).
      2. piston: a 0.2x0.2x0.6 m, 3 kg cylinder box hinged to the environment
         about y at its top, tilted U[-0.5,0.5] rad, with a 0.1x0.1x0.4 m, 1 kg
         piston on a body-body slider along its long axis: motor vel
         U[-0.5,0.5] m/s, fmax 30 N, stops -/+0.15 m; per-step slider force
         U[-5,5] N.
      3. chain: a capsule (r 0.06 m, length 0.5 m, 1.5 kg) hanging from the
         environment by a universal joint (axes x, y; axis-1 stops -/+0.6 rad,
         an axis-2 motor in half the worlds), a 0.2 m box below it on a ball
         joint (erp 0.5), a box welded under that by a fixed joint (erp
         U[0.1,0.6], cfm 1e-4) and a box hinged under it about x (stops
         -/+0.8 rad); per-step universal torques U[-1,1] N m and hinge torque
         U[-0.5,0.5] N m; small initial spin.
      4. a pair of 0.3 m, 1 kg cubes glued by a body-body fixed joint, dropped
         from 0.6 m with a random orientation and spin, and a 0.25 m cube
         welded to the environment (reversed fixed joint) given an initial
         velocity.
      5. arm: an upper link (0.15x0.15x0.6 m, 1.5 kg) on a ball joint to the
         environment and a lower link (0.12x0.12x0.6 m, 1 kg) on a ball joint
         below it, spun U[-2,2] rad/s; an Euler-mode angular motor between
         them (axis 0 = x on the upper link, axis 2 = z on the lower; stops
         -/+0.5, -/+0.4, -/+0.6 rad) and a user-mode angular motor on the
         upper link (2 axes: world y powered at vel U[-1,1] rad/s, fmax 3 N m;
         upper-link x with stops [-0.1, 0.2] and user angle 0.3, so its limit
         row is active); per-step torques U[-1,1] N m on that motor's axes.
    Surface mu 0.6 (pyramid friction). Max 4 contacts per pair."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, 0.6)
    NAN = float("nan")
    rail, drop, piston, uni, hinge3, umot = [], [], [], [], [], []
    for wi in range(n_worlds):
        w = b.new_world(cfm=1e-5, seed=int(rng.integers(0, 2**32)))
        b.add_geom(w, GEOM_PLANE, -1, (0, 0, 1, 0), s)
        # 0. rail
        a = rng.uniform(0, 2 * math.pi)
        ax = _unit((math.cos(a), math.sin(a), rng.uniform(-0.3, 0.3)))
        m, I = box_mass_total(2.0, 0.4, 0.2, 0.2)
        bi = b.add_body(w, (0.0, 0.0, 0.6), m, I, lvel=tuple(ax * rng.uniform(-1, 1)))
        b.add_geom(w, GEOM_BOX, bi, (0.4, 0.2, 0.2), s)
        lim = rng.uniform(0.2, 0.5)
        motor = wi % 2 == 0
        rail.append(b.add_joint(w, JOINT_SLIDER, bi, -1, axis1=tuple(ax), param=limot_params(
            lostop=-lim, histop=lim, vel=rng.uniform(-1, 1) if motor else 0.0, fmax=20.0 if motor else 0.0,
            bounce=0.3 if wi % 3 == 0 else 0.0)))
        # 1. drop rail (reversed)
        ax = _unit((rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2), 1.0))
        m, I = box_mass_total(1.0, 0.3, 0.3, 0.3)
        bi = b.add_body(w, (2.5, 0.0, rng.uniform(0.25, 0.6)), m, I)
        b.add_geom(w, GEOM_BOX, bi, (0.3, 0.3, 0.3), s)
        drop.append(b.add_joint(w, JOINT_SLIDER, -1, bi, axis1=tuple(ax), param=limot_params()))
        # 2. piston
        t = rng.uniform(-0.5, 0.5)
        u = np.array([math.sin(t), 0.0, math.cos(t)])
        q = (math.cos(t / 2), 0.0, math.sin(t / 2), 0.0)
        top = np.array([5.0, 0.0, 1.8])
        cc = top - 0.3 * u
        m, I = box_mass_total(3.0, 0.2, 0.2, 0.6)
        cyl = b.add_body(w, tuple(cc), m, I, q=q)
        b.add_geom(w, GEOM_BOX, cyl, (0.2, 0.2, 0.6), s)
        m, I = box_mass_total(1.0, 0.1, 0.1, 0.4)
        pis = b.add_body(w, tuple(cc - 0.5 * u), m, I, q=q)
        b.add_geom(w, GEOM_BOX, pis, (0.1, 0.1, 0.4), s)
        b.add_joint(w, JOINT_HINGE, cyl, -1, anchor=tuple(top), axis1=(0, 1, 0), param=limot_params())
        piston.append(b.add_joint(w, JOINT_SLIDER, cyl, pis, axis1=tuple(u), param=limot_params(
            lostop=-0.15, histop=0.15, vel=rng.uniform(-0.5, 0.5), fmax=30.0)))
        # 3. universal / ball / fixed / hinge chain
        x3 = 7.5
        m, I = capsule_mass(1.0, 0.06, 0.5)
        scale = 1.5 / m
        ca = b.add_body(w, (x3, 0.0, 2.0 - 0.31), 1.5, np.asarray(I) * scale,
                        avel=tuple(rng.uniform(-0.5, 0.5, 3)))
        b.add_geom(w, GEOM_CAPSULE, ca, (0.06, 0.5), s)
        p = np.zeros(JOINT_NPARAM)
        p[0:9] = limot_params(lostop=-0.6, histop=0.6)
        umotor = wi % 2 == 1
        p[9:18] = limot_params(vel=rng.uniform(-1, 1) if umotor else 0.0, fmax=2.0 if umotor else 0.0)
        uni.append(b.add_joint(w, JOINT_UNIVERSAL, ca, -1, anchor=(x3, 0.0, 2.0), axis1=(1, 0, 0),
                               axis2=(0, 1, 0), param=p))
        m, I = box_mass_total(1.0, 0.2, 0.2, 0.2)
        bb = b.add_body(w, (x3, 0.0, 2.0 - 0.62 - 0.1), m, I)
        b.add_geom(w, GEOM_BOX, bb, (0.2, 0.2, 0.2), s)
        b.add_joint(w, JOINT_BALL, ca, bb, anchor=(x3, 0.0, 2.0 - 0.62), param=[0.5, 1e-5])
        bc = b.add_body(w, (x3, 0.0, 2.0 - 0.62 - 0.3), m, I)
        b.add_geom(w, GEOM_BOX, bc, (0.2, 0.2, 0.2), s)
        b.add_joint(w, JOINT_FIXED, bb, bc, param=[rng.uniform(0.1, 0.6), 1e-4])
        bd = b.add_body(w, (x3, 0.0, 2.0 - 0.62 - 0.5), m, I)
        b.add_geom(w, GEOM_BOX, bd, (0.2, 0.2, 0.2), s)
        hinge3.append(b.add_joint(w, JOINT_HINGE, bc, bd, anchor=(x3, 0.0, 2.0 - 0.62 - 0.4), axis1=(1, 0, 0),
                                  param=limot_params(lostop=-0.8, histop=0.8)))
        # 4. glued pair and a welded cube
        qa = _unit(rng.normal(size=4))
        R = _R_from_q(qa)
        c0 = np.array([10.0, 0.0, 0.6])
        m, I = box_mass_total(1.0, 0.3, 0.3, 0.3)
        av = tuple(rng.uniform(-2, 2, 3))
        g1 = b.add_body(w, tuple(c0 - 0.16 * R[:, 0]), m, I, q=tuple(qa), avel=av)
        b.add_geom(w, GEOM_BOX, g1, (0.3, 0.3, 0.3), s)
        g2 = b.add_body(w, tuple(c0 + 0.16 * R[:, 0]), m, I, q=tuple(qa), avel=av)
        b.add_geom(w, GEOM_BOX, g2, (0.3, 0.3, 0.3), s)
        b.add_joint(w, JOINT_FIXED, g1, g2, param=[rng.uniform(0.1, 0.4), 1e-5])
        m, I = box_mass_total(1.0, 0.25, 0.25, 0.25)
        wq = _unit((1.0, *rng.uniform(-0.1, 0.1, 3)))
        wb = b.add_body(w, (11.0, 0.0, 0.5), m, I, q=tuple(wq), lvel=tuple(rng.uniform(-0.5, 0.5, 3)),
                        avel=tuple(rng.uniform(-1, 1, 3)))
        b.add_geom(w, GEOM_BOX, wb, (0.25, 0.25, 0.25), s)
        b.add_joint(w, JOINT_FIXED, -1, wb, param=[0.2, 1e-5])
        # 5. arm with an Euler angular motor and a user-mode angular motor
        x5 = 12.5
        m, I = box_mass_total(1.5, 0.15, 0.15, 0.6)
        ua = b.add_body(w, (x5, 0.0, 1.7), m, I, avel=tuple(rng.uniform(-0.5, 0.5, 3)))
        b.add_geom(w, GEOM_BOX, ua, (0.15, 0.15, 0.6), s)
        m, I = box_mass_total(1.0, 0.12, 0.12, 0.6)
        la = b.add_body(w, (x5, 0.0, 1.1), m, I, avel=tuple(rng.uniform(-2, 2, 3)))
        b.add_geom(w, GEOM_BOX, la, (0.12, 0.12, 0.6), s)
        b.add_joint(w, JOINT_BALL, ua, -1, anchor=(x5, 0.0, 2.0), param=[0.2, 1e-5])
        b.add_joint(w, JOINT_BALL, ua, la, anchor=(x5, 0.0, 1.4), param=[0.2, 1e-5])
        p = np.zeros(JOINT_NPARAM)
        p[0], p[1] = 3, AMOTOR_EULER
        p[2], p[3], p[4] = 1, 0, 2
        p[5:14] = limot_params(lostop=-0.5, histop=0.5)
        p[14:23] = limot_params(lostop=-0.4, histop=0.4)
        p[23:32] = limot_params(lostop=-0.6, histop=0.6)
        b.add_joint(w, JOINT_AMOTOR, ua, la, anchor=(1, 0, 0), axis1=(0, 1, 0), axis2=(0, 0, 1), param=p)
        p = np.zeros(JOINT_NPARAM)
        p[0], p[1] = 2, AMOTOR_USER
        p[2], p[3] = 0, 1
        p[5:14] = limot_params(vel=rng.uniform(-1, 1), fmax=3.0)
        p[14:23] = limot_params(lostop=-0.1, histop=0.2)
        p[32], p[33] = 0.0, 0.3
        umot.append(b.add_joint(w, JOINT_AMOTOR, ua, -1, anchor=(0, 1, 0), axis1=(1, 0, 0), param=p))
    sc = b.build()
    nj = sc.nj_total
    tq = np.zeros((steps, nj, 2))
    stops = np.full((steps, nj), NAN)
    servo = (np.arange(steps) // 10) % 3 == 2
    for wi in range(n_worlds):
        j0 = int(sc.joint_off[wi])
        tq[:, j0 + rail[wi], 0] = rng.uniform(-10, 10, steps)
        tq[:, j0 + drop[wi], 0] = rng.uniform(-10, 10, steps)
        tq[:, j0 + piston[wi], 0] = rng.uniform(-5, 5, steps)
        tq[:, j0 + uni[wi], :] = rng.uniform(-1, 1, (steps, 2))
        tq[:, j0 + hinge3[wi], 0] = rng.uniform(-0.5, 0.5, steps)
        tq[:, j0 + umot[wi], :] = rng.uniform(-1, 1, (steps, 2))
        target = rng.uniform(-0.2, 0.2, steps)
        stops[servo, j0 + rail[wi]] = target[servo]
    sc.set_controls(joint_torque=tq, joint_stop=stops)
    return sc


def _R_from_q(q):
    """3x3 rotation of a unit quaternion (w, x, y, z), as dRfromQ."""
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def sphere_pile(n=10000, seed=14, box=(6.0, 6.0, 20.0), rmin=0.1, rmax=0.3, mu=0.8, iterations=50,
                dt=0.005, jitter=0.05):
    """Large single world: n spheres, r U[rmin, rmax], density 1000, on a
    jittered grid (cells of equal size filling the box, lowest layers first,
    offsets U[-jitter, jitter] of a cell) inside a box[0] x box[1] x box[2] m
    box centred on x = y = 0 whose five static planes are the floor z = 0 and
    the four walls (created first, then one geom per sphere). Surface mu 0.8
    (Approx1 | SoftERP | SoftCFM, soft_erp 0.2, soft_cfm 1e-5), 50 iterations,
    w = 1.3, dt = 0.005, <= 4 contacts per pair. With the defaults neighbouring
    spheres overlap at the start and the pile settles under gravity."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = SceneBuilder()
    s = _std_surface(b, mu)
    bx, by, bz = box
    w = b.new_world(cfm=1e-5, iterations=iterations, dt=dt, seed=int(rng.integers(0, 2**32)))
    for pl in ((0, 0, 1, 0), (1, 0, 0, -bx / 2), (-1, 0, 0, -bx / 2), (0, 1, 0, -by / 2), (0, -1, 0, -by / 2)):
        b.add_geom(w, GEOM_PLANE, -1, pl, s)
    cell = (bx * by * bz / n) ** (1.0 / 3.0)
    nx, ny = max(1, int(bx / cell)), max(1, int(by / cell))
    nz = -(-n // (nx * ny))
    dx, dy, dz = bx / nx, by / ny, bz / nz
    for k in range(n):
        iz, rem = divmod(k, nx * ny)
        iy, ix = divmod(rem, nx)
        j = rng.uniform(-jitter, jitter, 3)
        pos = (-bx / 2 + (ix + 0.5 + j[0]) * dx, -by / 2 + (iy + 0.5 + j[1]) * dy, (iz + 0.5 + j[2]) * dz)
        r = rng.uniform(rmin, rmax)
        m, I = sphere_mass(1000.0, r)
        bi = b.add_body(w, pos, m, I)
        b.add_geom(w, GEOM_SPHERE, bi, (r,), s)
    return b.build()
