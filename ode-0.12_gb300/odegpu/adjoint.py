"""Differentiable rollouts: torch.autograd.Function over the batch's
checkpointed forward rollout and hand-written adjoint (libodegpu's
odegpuBatchRolloutForward / odegpuBatchRolloutBackward).

    B = Batch(scene)
    final = rollout(B, n_steps, init_state, joint_torque, body_force, ckpt_every=10)
    loss = f(final); loss.backward()

``init_state`` is [nb_total, 13] FP32 on the batch's device (pos, q, lvel,
avel); ``joint_torque`` is [S, nj_total, 2] and ``body_force`` [S, nb_total, 6]
(either may be None); the controls of step k are entry k % S, counting from
``step0``. The rollout starts from the batch's current RNG seeds; forward and
backward put those seeds and the step index back afterwards, so repeated
calls give the same result.
"""
from __future__ import annotations

import torch

from .batch import Batch


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, batch: Batch, n_steps: int, ckpt_every: int, step0: int, init_state, joint_torque,
                body_force):
        dev = init_state.device
        x0 = init_state.detach().to(torch.float32).contiguous()
        jt = joint_torque.detach().to(torch.float32).contiguous() if joint_torque is not None else None
        bf = body_force.detach().to(torch.float32).contiguous() if body_force is not None else None
        S = jt.shape[0] if jt is not None else (bf.shape[0] if bf is not None else 0)
        torch.cuda.current_stream(dev).synchronize()
        seeds = batch.seeds()
        batch.set_step_index(step0)
        batch.set_controls_f32(S, jt.data_ptr() if jt is not None else None,
                               bf.data_ptr() if bf is not None else None)
        batch.write_state_async(x0.data_ptr())
        batch.rollout_forward(n_steps, ckpt_every)
        out = torch.empty_like(x0)
        batch.read_state_async(out.data_ptr())
        batch.sync()
        ctx.batch = batch
        ctx.S = S
        ctx.shapes = (jt is not None, bf is not None)
        ctx.restore = (seeds, step0)
        batch.set_seeds(seeds)
        batch.set_step_index(step0)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        B = ctx.batch
        g = grad_out.detach().to(torch.float32).contiguous()
        dev = g.device
        g_init = torch.empty_like(g)
        has_jt, has_bf = ctx.shapes
        g_jt = torch.zeros((max(ctx.S, 1), B.nj_total, 2), dtype=torch.float32, device=dev) if has_jt else None
        g_bf = torch.zeros((max(ctx.S, 1), B.nb_total, 6), dtype=torch.float32, device=dev) if has_bf else None
        torch.cuda.current_stream(dev).synchronize()
        B.rollout_backward(g.data_ptr(), g_init.data_ptr(), g_jt.data_ptr() if has_jt else None,
                           g_bf.data_ptr() if has_bf else None)
        B.sync()
        seeds, step0 = ctx.restore
        B.set_seeds(seeds)
        B.set_step_index(step0)
        return None, None, None, None, g_init, g_jt, g_bf


def rollout(batch: Batch, n_steps: int, init_state, joint_torque=None, body_force=None, ckpt_every=10,
            step0=0):
    """Final state [nb_total, 13] after n_steps, differentiable with respect to
    init_state, joint_torque and body_force."""
    return _Rollout.apply(batch, int(n_steps), int(ckpt_every), int(step0), init_state, joint_torque,
                          body_force)
