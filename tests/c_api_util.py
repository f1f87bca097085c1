"""Builds the plain ODE programs under tests/c_api/ (box_drop_demo.c,
scene_player.c) against libodegpu or the reference, and writes their inputs."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_api", "box_drop_demo.c")
PLAYER = os.path.join(ROOT, "tests", "c_api", "scene_player.c")
PKG = os.path.join(ROOT, "ode-0.12_gb300")
# the reference checkout (headers of the reference build): ODE_REF_SRC, else
# the checkout beside this repository
REF_ROOT = os.environ.get("ODE_REF_SRC") or os.path.normpath(os.path.join(ROOT, "..", "reference", "ode-0.12"))


def build_gpu_demo(out, src=SRC):
    subprocess.run(["gcc", "-O2", "-o", out, src, "-I" + os.path.join(ROOT, "include"), "-L" + PKG,
                    "-lodegpu", "-Wl,-rpath," + PKG, "-lm"], check=True)
    return out


def build_ref_demo(out, ref_root=REF_ROOT, src=SRC):
    lib = os.path.join(ROOT, "oracle", "_ref")
    subprocess.run(["g++", "-O2", "-x", "c++", "-DUSE_REFERENCE_ODE", "-DdSINGLE", "-w", "-o", out, src,
                    "-I" + os.path.join(ref_root, "include"), "-L" + lib, "-l:libode_ref_s.so",
                    "-Wl,-rpath," + lib, "-lm"], check=True)
    return out


def ref_demo_available(ref_root=REF_ROOT):
    return (os.path.isdir(os.path.join(ref_root, "include")) and
            os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")))


def player_input(sc, w, steps, path):
    """Writes scene_player.c's input for world w of a scene (no heightfields)."""
    b0, b1 = sc.world_bodies(w)
    g0, g1 = int(sc.geom_off[w]), int(sc.geom_off[w + 1])
    j0, j1 = sc.world_joints(w)
    P = sc.world_params[w]
    nctrl = int(sc.n_ctrl_steps)
    f = lambda xs: " ".join(repr(float(x)) for x in xs)  # noqa: E731
    lines = [f((b1 - b0, g1 - g0, j1 - j0, len(sc.surfaces), steps, nctrl, P.seed, P.max_contacts)),
             f((*P.gravity, P.erp, P.cfm, P.iterations, P.sor_w, P.max_vel, P.min_depth, P.dt))]
    for S in sc.surfaces:
        lines.append(f((S.mode, S.mu, S.mu2, S.bounce, S.bounce_vel, S.soft_erp, S.soft_cfm, S.motion1,
                        S.motion2, S.motionN, S.slip1, S.slip2)))
    for i in range(b0, b1):
        lines.append(f((*sc.body_pos[i], *sc.body_q[i], *sc.body_lvel[i], *sc.body_avel[i], sc.body_mass[i],
                        *sc.body_I[i], sc.body_flags[i])))
    for g in range(g0, g1):
        assert sc.geom_type[g] in (0, 1, 2, 3, 4), "scene_player takes sphere / box / capsule / cylinder / plane geoms"
        lines.append(f((sc.geom_type[g], sc.geom_body[g], sc.geom_surface[g], *sc.geom_param[g])))
    for j in range(j0, j1):
        lines.append(f((sc.joint_type[j], *sc.joint_body[j], *sc.joint_anchor[j], *sc.joint_axis1[j],
                        *sc.joint_axis2[j], *sc.joint_param[j])))
    nan = float("nan")
    for s in range(nctrl):
        for j in range(j0, j1):
            t = sc.joint_torque[s, j] if sc.joint_torque is not None else (0.0, 0.0)
            st = sc.joint_stop[s, j] if sc.joint_stop is not None else nan
            lines.append(f((*t, st)))
        for i in range(b0, b1):
            lines.append(f(sc.body_force[s, i] if sc.body_force is not None else (0.0,) * 6))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def scene_input(sc, steps, path):
    """Writes the demo's input for world 0 of a box_drop scene."""
    b0, b1 = sc.world_bodies(0)
    lines = [f"{b1 - b0} {steps} {sc.world_params[0].seed}"]
    for i in range(b0, b1):
        g = sc.geom_param[1 + i - b0]
        p = sc.body_pos[i]
        I = sc.body_I[i]
        lines.append(" ".join(repr(float(x)) for x in (*g[:3], *p, sc.body_mass[i], I[0], I[4], I[8])))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def run_demo(exe, inp, *args):
    out = subprocess.run([exe, inp, *args], check=True, capture_output=True, text=True).stdout
    return np.array([[float(x) for x in ln.split()] for ln in out.strip().splitlines()])
