"""torch.autograd.Function over the C ABI's forward / vjp pair.

`RK4.apply(state, h0, u0, dt, nsteps, ckpt_every)` runs nsteps sw RK4 steps
on the GPU (mpaso_rk4_forward, keeping checkpoints) and returns (hN, uN);
backward calls mpaso_rk4_vjp, which recomputes stage states segment by
segment from the checkpoints and applies the hand-written adjoint kernels.
PyTorch only carries tensors here; the library itself has no PyTorch in it.
"""
import torch

from . import gpu as G


class RK4(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state, h0, u0, dt, nsteps, ckpt_every):
        h0c = h0.detach().contiguous()
        u0c = u0.detach().contiguous()
        torch.cuda.synchronize()
        state.set(G.FIELD_H, h0c)
        state.set(G.FIELD_U, u0c)
        state.forward(dt, nsteps, ckpt_every)
        hN = torch.empty_like(h0c)
        uN = torch.empty_like(u0c)
        state.get(G.FIELD_H, hN)
        state.get(G.FIELD_U, uN)
        ctx.state = state
        return hN, uN

    @staticmethod
    def backward(ctx, ghN, guN):
        ghN = ghN.contiguous() if ghN is not None else None
        guN = guN.contiguous() if guN is not None else None
        ref = ghN if ghN is not None else guN
        dev = ref.device
        if ghN is None:
            ghN = torch.zeros(ctx.state._shape(G.FIELD_H), dtype=torch.float64, device=dev)
        if guN is None:
            guN = torch.zeros(ctx.state._shape(G.FIELD_U), dtype=torch.float64, device=dev)
        gh0 = torch.empty_like(ghN)
        gu0 = torch.empty_like(guN)
        torch.cuda.synchronize()
        ctx.state.vjp(ghN, guN, out=(gh0, gu0))
        return None, gh0, gu0, None, None, None
