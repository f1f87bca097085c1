"""Batched world stepping through libodegpu's C ABI (include/odegpu.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import lib, check

_P = C.POINTER
BODY_REC = 13

# odegpuRay / odegpuRayHit (include/odegpu.h)
RAY_DTYPE = np.dtype([("world", np.int32), ("body", np.int32), ("start", np.float32, 3),
                      ("dir", np.float32, 3), ("length", np.float32)])
HIT_DTYPE = np.dtype([("geom", np.int32), ("pos", np.float32, 3), ("normal", np.float32, 3),
                      ("depth", np.float32)])
assert RAY_DTYPE.itemsize == 36 and HIT_DTYPE.itemsize == 32


class BatchConfig(C.Structure):
    _fields_ = [("contacts_per_body", C.c_int), ("warps_per_block", C.c_int),
                ("device", C.c_int), ("large_world", C.c_int)]


class Batch:
    """A set of independent worlds resident on one GPU.

    ``step(n)`` runs n full steps (collide + QuickStep) of every world in one
    launch; ``state()`` returns [nb_total, 13] FP64 records
    (pos[3], q[4], lvel[3], avel[3])."""

    def __init__(self, scene, contacts_per_body=8, warps_per_block=0, device=0, large_world=False):
        self.scene = scene
        cfg = BatchConfig(contacts_per_body, warps_per_block, device, 1 if large_world else 0)
        h = C.c_void_p()
        check(lib().odegpuBatchCreate(C.byref(scene.c), C.byref(cfg), C.byref(h)))
        self.h = h
        nw, nb, nj = C.c_int(), C.c_int(), C.c_int()
        rc, cc = C.c_longlong(), C.c_longlong()
        check(lib().odegpuBatchInfo(h, C.byref(nw), C.byref(nb), C.byref(nj), C.byref(rc),
                                    C.byref(cc)))
        self.n_worlds, self.nb_total, self.nj_total = nw.value, nb.value, nj.value
        self.row_capacity, self.contact_capacity = rc.value, cc.value

    def close(self):
        if getattr(self, "h", None):
            lib().odegpuBatchDestroy(self.h)
            self.h = None

    __del__ = close

    def step(self, n=1):
        check(lib().odegpuBatchStep(self.h, n))

    def step_plain(self, n=1):
        check(lib().odegpuBatchStepPlain(self.h, n))

    def step_graph(self, n=1):
        check(lib().odegpuBatchStepGraph(self.h, n))

    def large_world_stats(self, reset=True):
        """Device-side diagnostics of a large-world batch: island walk, sweep
        first iterations, level sort and remaining iterations (ms), the
        largest level count, sweep launches and walks."""
        out = (C.c_longlong * 9)()
        check(lib().odegpuBatchLargeWorldStats(self.h, out, 9, 1 if reset else 0))
        v = list(out)
        return dict(walk_ms=v[0] / 1e6, sweep_first_ms=v[1] / 1e6, sort_ms=v[2] / 1e6,
                    sweep_rest_ms=v[3] / 1e6, levels_max=v[4], sweeps=v[5], walks=v[6],
                    walk_copy_ms=v[7] / 1e6, cluster=v[8])

    def set_stepper(self, exact=True):
        """Step with dWorldStep (the exact stepper: dense LCP per island,
        Dantzig pivoting) instead of dWorldQuickStep from now on."""
        check(lib().odegpuBatchSetStepper(self.h, 1 if exact else 0))

    def ray_cast(self, rays, flags=1):
        """Nearest hit of each ray among its world's geoms (odegpuBatchRayCast).
        rays: a RAY_DTYPE array (world, body, start[3], dir[3], length; body -1
        for a world-frame ray, else the world-local body it is attached to, with
        start / dir in that body's frame). Returns a HIT_DTYPE array (geom,
        pos[3], normal[3], depth; geom -1 where nothing is hit)."""
        r = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.zeros(len(r), dtype=HIT_DTYPE)
        rc = lib().odegpuBatchRayCast(self.h, r.ctypes.data, len(r), int(flags), hits.ctypes.data)
        check(rc)
        return hits

    def ray_cast_async(self, d_rays, n, d_hits, flags=1):
        """odegpuBatchRayCastAsync on device pointers (e.g. torch tensors'
        data_ptr()), enqueued on the batch stream."""
        check(lib().odegpuBatchRayCastAsync(self.h, int(d_rays), int(n), int(flags), int(d_hits)))

    def sync(self):
        check(lib().odegpuBatchSynchronize(self.h))

    def set_timing(self, on=True):
        """Record CUDA events around the collide/setup/solve kernels of every
        following (non-graph) step."""
        check(lib().odegpuBatchSetTiming(self.h, 1 if on else 0))

    def kernel_times(self):
        """(ms[collide, setup, solve] summed since the last call, steps covered)."""
        ms = (C.c_double * 3)()
        n = C.c_longlong(0)
        check(lib().odegpuBatchGetKernelTimes(self.h, ms, C.byref(n)))
        return np.array(ms[:]), n.value

    def launch_count(self):
        """Kernels launched by this batch since creation."""
        n = C.c_longlong(0)
        check(lib().odegpuBatchGetLaunchCount(self.h, C.byref(n)))
        return n.value

    def state(self):
        out = np.zeros((self.nb_total, BODY_REC))
        check(lib().odegpuBatchReadState(self.h, out.ctypes.data_as(_P(C.c_double))))
        return out

    def set_state(self, st):
        st = np.ascontiguousarray(st, dtype=np.float64)
        assert st.shape == (self.nb_total, BODY_REC)
        check(lib().odegpuBatchWriteState(self.h, st.ctypes.data_as(_P(C.c_double))))

    def read_state_async(self, ptr):
        check(lib().odegpuBatchReadStateF32Async(self.h, C.c_void_p(ptr)))

    def write_state_async(self, ptr):
        check(lib().odegpuBatchWriteStateF32Async(self.h, C.c_void_p(ptr)))

    def stream_handle(self):
        return lib().odegpuBatchStream(self.h)

    def status(self):
        out = np.zeros(self.n_worlds, np.int32)
        check(lib().odegpuBatchGetStatus(self.h, out.ctypes.data_as(_P(C.c_int))))
        return out

    def counts(self):
        nc = np.zeros(self.n_worlds, np.int32)
        nr = np.zeros(self.n_worlds, np.int32)
        ni = np.zeros(self.n_worlds, np.int32)
        check(lib().odegpuBatchGetCounts(self.h, nc.ctypes.data_as(_P(C.c_int)),
                                         nr.ctypes.data_as(_P(C.c_int)),
                                         ni.ctypes.data_as(_P(C.c_int))))
        return nc, nr, ni

    def seeds(self):
        out = np.zeros(self.n_worlds, np.uint32)
        check(lib().odegpuBatchGetSeeds(self.h, out.ctypes.data_as(_P(C.c_uint))))
        return out

    def set_step_index(self, step):
        check(lib().odegpuBatchSetStepIndex(self.h, int(step)))

    def set_seeds(self, seeds):
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        check(lib().odegpuBatchSetSeeds(self.h, s.ctypes.data_as(_P(C.c_uint))))

    def set_controls(self, joint_torque=None, body_force=None):
        S = 0
        jt = bf = None
        if joint_torque is not None:
            jt = np.ascontiguousarray(joint_torque, dtype=np.float64)
            S = jt.shape[0]
        if body_force is not None:
            bf = np.ascontiguousarray(body_force, dtype=np.float64)
            S = bf.shape[0]
        check(lib().odegpuBatchSetControls(
            self.h, S, jt.ctypes.data_as(_P(C.c_double)) if jt is not None else None,
            bf.ctypes.data_as(_P(C.c_double)) if bf is not None else None))

    def set_controls_f32(self, n_ctrl_steps, joint_torque_ptr=None, body_force_ptr=None):
        """Controls from FP32 arrays at host or device addresses (integers)."""
        check(lib().odegpuBatchSetControlsF32(self.h, int(n_ctrl_steps), joint_torque_ptr,
                                              body_force_ptr))

    def rollout_forward(self, n_steps, ckpt_every=10):
        check(lib().odegpuBatchRolloutForward(self.h, int(n_steps), int(ckpt_every)))

    def rollout_backward(self, grad_final_ptr, grad_init_ptr=None, grad_jt_ptr=None, grad_bf_ptr=None):
        check(lib().odegpuBatchRolloutBackward(self.h, grad_final_ptr, grad_init_ptr, grad_jt_ptr,
                                               grad_bf_ptr))

    def set_feedback(self, on=True):
        """Compute joint feedback (f1 t1 f2 t2 per persistent joint) in every step."""
        check(lib().odegpuBatchSetFeedback(self.h, 1 if on else 0))

    def feedback(self):
        """[nj_total, 12] f1 t1 f2 t2 of the last step."""
        out = np.zeros((max(self.nj_total, 1), 12))
        check(lib().odegpuBatchGetFeedback(self.h, out.ctypes.data_as(_P(C.c_double))))
        return out[:self.nj_total]

    def set_launch_config(self, kernel, warps_per_block, smem_carveout=-1):
        """kernel: 0 collide, 1 setup, 2 solve, 3 adjoint, 4 fused step."""
        check(lib().odegpuBatchSetLaunchConfig(self.h, int(kernel), int(warps_per_block), int(smem_carveout)))

    def set_launch_config_ex(self, kernel, warps_per_block, smem_carveout=-1, variant=0):
        """As set_launch_config, with the kernel variant (1: the solve kernel
        capped at 128 registers per thread for more warps per SM)."""
        check(lib().odegpuBatchSetLaunchConfigEx(self.h, int(kernel), int(warps_per_block),
                                                 int(smem_carveout), int(variant)))

    def launch_config_ex(self, kernel):
        """(warps per block, carveout, variant) of one kernel."""
        w, c, v = C.c_int(), C.c_int(), C.c_int()
        check(lib().odegpuBatchGetLaunchConfigEx(self.h, int(kernel), C.byref(w), C.byref(c), C.byref(v)))
        return w.value, c.value, v.value

    def launch_config(self):
        cfg = (C.c_int * 8)()
        check(lib().odegpuBatchGetLaunchConfig(self.h, cfg))
        return [(cfg[2 * k], cfg[2 * k + 1]) for k in range(4)]

    def set_step_kernels(self, fused=True):
        """One fused kernel per step (collide, setup and solve of each world on
        its warp) or the three separate kernels; the results are the same."""
        check(lib().odegpuBatchSetStepKernels(self.h, 1 if fused else 0))

    def step_kernels(self):
        """(fused, warps per block, carveout) of the step launch."""
        f, w, c = C.c_int(), C.c_int(), C.c_int()
        check(lib().odegpuBatchGetStepKernels(self.h, C.byref(f), C.byref(w), C.byref(c)))
        return bool(f.value), w.value, c.value

    def autotune(self, n_steps=4):
        """Pick each kernel's launch shape by timing candidates on the current state."""
        check(lib().odegpuBatchAutotune(self.h, int(n_steps)))
        return self.launch_config()

    def adjoint_status(self):
        out = np.zeros(self.n_worlds, np.int32)
        check(lib().odegpuBatchAdjointStatus(self.h, out.ctypes.data_as(_P(C.c_int))))
        return out

    def step_tap(self):
        """One step, returning (rows [R,32] f32, lambda [R], fc [nb,6], row_off [W])."""
        rows = np.zeros((self.row_capacity, 32), np.float32)
        lam = np.zeros(self.row_capacity, np.float32)
        fc = np.zeros((self.nb_total, 6), np.float32)
        ro = np.zeros(self.n_worlds, np.int32)
        check(lib().odegpuBatchStepTap(self.h, rows.ctypes.data_as(_P(C.c_float)),
                                       lam.ctypes.data_as(_P(C.c_float)),
                                       fc.ctypes.data_as(_P(C.c_float)),
                                       ro.ctypes.data_as(_P(C.c_int))))
        return rows, lam, fc, ro

    def contacts(self, w, cap=4096):
        out = np.zeros((cap, 9), np.float32)
        n = check(lib().odegpuBatchGetContacts(self.h, w, out.ctypes.data_as(_P(C.c_float)), cap))
        return out[:min(n, cap)]
