"""Builds tests/c_api/box_drop_demo.c against libodegpu (or the reference)."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_api", "box_drop_demo.c")
PKG = os.path.join(ROOT, "ode-0.12_gb300")


def build_gpu_demo(out):
    subprocess.run(["gcc", "-O2", "-o", out, SRC, "-I" + os.path.join(ROOT, "include"), "-L" + PKG,
                    "-lodegpu", "-Wl,-rpath," + PKG, "-lm"], check=True)
    return out


def build_ref_demo(out, ref_root="/root/reference/ode-0.12"):
    lib = os.path.join(ROOT, "oracle", "_ref")
    subprocess.run(["g++", "-O2", "-x", "c++", "-DUSE_REFERENCE_ODE", "-DdSINGLE", "-w", "-o", out, SRC,
                    "-I" + os.path.join(ref_root, "include"), "-L" + lib, "-l:libode_ref_s.so",
                    "-Wl,-rpath," + lib, "-lm"], check=True)
    return out


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


def run_demo(exe, inp):
    out = subprocess.run([exe, inp], check=True, capture_output=True, text=True).stdout
    return np.array([[float(x) for x in ln.split()] for ln in out.strip().splitlines()])
