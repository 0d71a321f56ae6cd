"""Gradients of a smooth string-core loss through the fused RK4 evolution.

``string_core_loss(state0, lambda0, ...)`` evolves a periodic level with the
fused RK4 kernels and returns

    L = sum_cells exp(-|phi|^2 / width) + <axion kinetic energy density>,   phi = psi / R,

as a differentiable torch scalar. Its backward pass is the hand-written
discrete adjoint in libaxs_gb300.so (``axs_level_rk4_adjoint_step``), driven
with checkpoint-every-k recomputation: the forward pass keeps the state every
k steps, the backward pass re-runs each k-step segment forward, keeping its
states, and reverses it step by step. Gradients are returned with respect to
the initial state (psi1, psi2, Pi1, Pi2) and lambda0 (the coupling scale:
lambda(tau) = lambda0 * lambda_unit(tau)). The integer winding count is never
differentiated.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import torch

from . import _lib as L
from .background import Background
from .level import PeriodicLevel, _stream_ptr


class AdjointBuffers:
    """Adjoint state (level layout, 4 components) and workspace for a level."""

    def __init__(self, level: PeriodicLevel):
        d = level.state
        self.abar = torch.zeros_like(d)
        b = C.c_int64()
        L.call("axs_level_adjoint_work_bytes", level.c.dtype, level.nx, level.ny, level.nz, C.byref(b))
        self.work = torch.zeros(b.value, dtype=torch.uint8, device=d.device)
        self.lambda_bar = torch.zeros(1, dtype=torch.float64, device=d.device)
        self.loss = torch.zeros(1, dtype=torch.float64, device=d.device)
        self.scratch = torch.zeros(8 * 4 * 256, dtype=torch.uint8, device=d.device)

    def abar_valid(self, level: PeriodicLevel) -> torch.Tensor:
        ox, oy = level.layout.x_offset, level.layout.y_offset
        return self.abar[:, :, oy:oy + level.ny, ox:ox + level.nx]


def loss_and_seed(level: PeriodicLevel, buf: AdjointBuffers, R: float, width: float, stream=None) -> torch.Tensor:
    """Write the loss to buf.loss and dL/dy to buf.abar (padding filled)."""
    L.call("axs_level_string_core_loss", C.byref(level.c), float(R), float(width), buf.loss.data_ptr(),
           buf.abar.data_ptr(), buf.scratch.data_ptr(), buf.scratch.numel(), _stream_ptr(stream))
    return buf.loss


def adjoint_step(level: PeriodicLevel, state_buffer: torch.Tensor, buf: AdjointBuffers, bg: Background,
                 tau_i: float, t: float, dt: float, stream=None) -> None:
    """Reverse the step from t whose start state is `state_buffer` (level layout)."""
    c = L.LevelC(state_buffer.data_ptr(), level.work.data_ptr(), level.c.dtype, level.nx, level.ny, level.nz,
                 level.dx, level.c.tile_config)
    L.call("axs_level_rk4_adjoint_step", C.byref(c), buf.abar.data_ptr(), buf.work.data_ptr(), buf.work.numel(),
           C.byref(bg.to_c()), float(tau_i), float(t), float(dt), buf.lambda_bar.data_ptr(), _stream_ptr(stream))


@dataclasses.dataclass
class EvolutionSpec:
    dx: float = 0.5
    dt: float = 0.1
    nsteps: int = 200
    tau_i: float = 1.0
    a_inv: float = 2.0
    c0: float = 1.0
    width: float = 0.1
    checkpoint_every: int = 20


class _StringCoreLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state0: torch.Tensor, lambda0: torch.Tensor, spec: EvolutionSpec):
        _, nz, ny, nx = state0.shape
        lam0 = float(lambda0.detach())
        bg = Background.expanding(spec.a_inv, spec.c0, lambda0=lam0)
        level = PeriodicLevel((nx, ny, nz), spec.dx, dtype=state0.dtype, device=state0.device, pierced_capacity=1)
        level.set_state(state0.detach())
        k = max(1, int(spec.checkpoint_every))
        checkpoints = []
        for s in range(spec.nsteps):
            if s % k == 0:
                checkpoints.append(level.state.clone())
            level.advance(bg, spec.tau_i, s * spec.dt, spec.dt, 1)
        buf = AdjointBuffers(level)
        tau_f = spec.tau_i + spec.nsteps * spec.dt
        loss = loss_and_seed(level, buf, bg.values(tau_f).R, spec.width)
        level.device_status()
        ctx.spec, ctx.bg, ctx.level, ctx.buf, ctx.checkpoints = spec, bg, level, buf, checkpoints
        return loss.clone().reshape(()).to(state0.dtype)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        spec, bg, level, buf = ctx.spec, ctx.bg, ctx.level, ctx.buf
        k = max(1, int(spec.checkpoint_every))
        buf.lambda_bar.zero_()
        nseg = len(ctx.checkpoints)
        for seg in reversed(range(nseg)):
            s0 = seg * k
            s1 = min(spec.nsteps, s0 + k)
            # re-run the segment forward, keeping the state at the start of each step
            level.state.copy_(ctx.checkpoints[seg])
            states = []
            for s in range(s0, s1):
                states.append(level.state.clone())
                level.advance(bg, spec.tau_i, s * spec.dt, spec.dt, 1)
            for s in reversed(range(s0, s1)):
                adjoint_step(level, states[s - s0], buf, bg, spec.tau_i, s * spec.dt, spec.dt)
            del states
        level.device_status()
        g_state = buf.abar_valid(level).clone() * grad_out.to(level.dtype)
        g_lam = (buf.lambda_bar[0] * grad_out.double()).to(grad_out.dtype)
        return g_state, g_lam.reshape(()), None


def string_core_loss(state0: torch.Tensor, lambda0: torch.Tensor, spec: EvolutionSpec | None = None) -> torch.Tensor:
    """Differentiable loss after `spec.nsteps` fused RK4 steps (see module doc).

    state0: CUDA tensor (4, nz, ny, nx) of psi1, psi2, Pi1, Pi2 (float32 or float64);
    lambda0: scalar tensor, the coupling scale."""
    return _StringCoreLoss.apply(state0, lambda0, spec or EvolutionSpec())
