"""torch.autograd bridge over the C ABI's rollout / backward pair.

`rollout(system, stiffness, x0, v0, dt, steps, checkpoint_every)` returns
the final positions and velocities of `steps` updates of `system` started
from (x0, v0) with the given distance-constraint stiffness; its backward is
pbd_backward (hand-written adjoint kernels, checkpoints every
`checkpoint_every` steps, the forward pass recomputed in between).  All
tensors live on the system's CUDA device: x0, v0 and the outputs are
float32 (n, 4) (xyz + inverse mass / unused w), stiffness float32 (m,).
The C++ host does the work; this module only moves device pointers.
"""
from __future__ import annotations

import torch


def _ptr(t):
    return None if t is None else t.data_ptr()


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, stiffness, x0, v0, system, dt, steps, every):
        n = system.num_particles
        stream = torch.cuda.current_stream(x0.device).cuda_stream
        lib, h = system.lib, system.h
        x0c = x0.detach().contiguous()
        v0c = v0.detach().contiguous()
        system._check(lib.pbd_set_positions(h, 0, n, x0c.data_ptr(), 1, stream))
        system._check(lib.pbd_set_velocities(h, 0, n, v0c.data_ptr(), 1, stream))
        if stiffness.numel():
            st = stiffness.detach().contiguous()
            system.set_distance_stiffness(None, device_ptr=st.data_ptr(), stream=stream)
        system.rollout(dt, steps, every, stream)
        xT = torch.empty_like(x0c)
        vT = torch.empty_like(v0c)
        system._check(lib.pbd_get_positions(h, 0, n, xT.data_ptr(), 1, stream))
        system._check(lib.pbd_get_velocities(h, 0, n, vT.data_ptr(), 1, stream))
        ctx.system = system
        ctx.m = stiffness.numel()
        return xT, vT

    @staticmethod
    def backward(ctx, gx, gv):
        system = ctx.system
        dev = gx.device if gx is not None else gv.device
        n = system.num_particles
        gx = None if gx is None else gx.contiguous()
        gv = None if gv is None else gv.contiguous()
        dx0 = torch.empty((n, 4), dtype=torch.float32, device=dev) if ctx.needs_input_grad[1] else None
        dv0 = torch.empty((n, 4), dtype=torch.float32, device=dev) if ctx.needs_input_grad[2] else None
        ds = (torch.empty(ctx.m, dtype=torch.float32, device=dev)
              if ctx.needs_input_grad[0] and ctx.m else None)
        stream = torch.cuda.current_stream(dev).cuda_stream
        system.backward_device(_ptr(gx), _ptr(gv), _ptr(dx0), _ptr(dv0), _ptr(ds), stream)
        if ds is None and ctx.needs_input_grad[0]:
            ds = torch.zeros(ctx.m, dtype=torch.float32, device=dev)
        return ds, dx0, dv0, None, None, None, None


def rollout(system, stiffness: torch.Tensor, x0: torch.Tensor, v0: torch.Tensor, dt: float, steps: int,
            checkpoint_every: int = 10):
    """(x_T, v_T) after `steps` updates, differentiable in stiffness, x0, v0."""
    return _Rollout.apply(stiffness, x0, v0, system, float(dt), int(steps), int(checkpoint_every))


def fit(system, x0: torch.Tensor, target: torch.Tensor, stiffness0: torch.Tensor, v0_init: torch.Tensor, dt: float,
        steps: int, checkpoint_every: int, iterations: int, lr_stiffness: float = 0.01, lr_velocity: float = 0.01,
        stiffness_range=(0.2, 1.0), callback=None):
    """Recovers distance-constraint stiffness and initial velocities from
    final positions: Adam on L = mean |x_T - target|^2 through rollout(),
    stiffness projected to stiffness_range after each update.  Returns
    (stiffness, v0, losses)."""
    st = stiffness0.detach().clone().requires_grad_(True)
    v0 = v0_init.detach().clone().requires_grad_(True)
    opt = torch.optim.Adam([{"params": [st], "lr": lr_stiffness}, {"params": [v0], "lr": lr_velocity}])
    losses = []
    for it in range(iterations):
        opt.zero_grad()
        xT, _ = rollout(system, st, x0, v0, dt, steps, checkpoint_every)
        loss = ((xT[:, :3] - target[:, :3]) ** 2).sum(1).mean()
        loss.backward()
        losses.append(float(loss.detach()))
        opt.step()
        with torch.no_grad():
            st.clamp_(*stiffness_range)
            v0[:, 3] = 0.0
        if callback:
            callback(it, losses[-1])
    return st.detach(), v0.detach(), losses
