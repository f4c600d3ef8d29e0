"""torch.autograd.Function over the C ABI's forward / vjp pair.

`RK4.apply(state, h0, u0, dt, nsteps, ckpt_every)` runs nsteps sw RK4 steps
on the GPU (mpaso_rk4_forward, keeping checkpoints) and returns (hN, uN);
backward calls mpaso_rk4_vjp, which recomputes stage states segment by
segment from the checkpoints and applies the hand-written adjoint kernels.
`RK4Tracers.apply(state, h0, u0, tr0, dt, nsteps, ckpt_every)` is the same
with the tracers (FCT / del2 as the state was created with), backward through
mpaso_rk4_vjp_tracers.  ckpt_every = 0 stores the whole window instead of
checkpoints.  PyTorch only carries tensors here; the library itself has no
PyTorch in it.
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


def _zeros_like_field(state, field, ref):
    return torch.zeros(state._shape(field), dtype=torch.float64, device=ref.device)


class RK4Tracers(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state, h0, u0, tr0, dt, nsteps, ckpt_every):
        h0c, u0c, t0c = (x.detach().contiguous() for x in (h0, u0, tr0))
        torch.cuda.synchronize()
        state.set(G.FIELD_H, h0c)
        state.set(G.FIELD_U, u0c)
        state.set(G.FIELD_TRACERS, t0c)
        state.forward(dt, nsteps, ckpt_every)
        hN, uN, tN = torch.empty_like(h0c), torch.empty_like(u0c), torch.empty_like(t0c)
        state.get(G.FIELD_H, hN)
        state.get(G.FIELD_U, uN)
        state.get(G.FIELD_TRACERS, tN)
        ctx.state = state
        return hN, uN, tN

    @staticmethod
    def backward(ctx, ghN, guN, gtN):
        ref = next(g for g in (ghN, guN, gtN) if g is not None)
        st = ctx.state
        ghN = ghN.contiguous() if ghN is not None else _zeros_like_field(st, G.FIELD_H, ref)
        guN = guN.contiguous() if guN is not None else _zeros_like_field(st, G.FIELD_U, ref)
        gtN = gtN.contiguous() if gtN is not None else _zeros_like_field(st, G.FIELD_TRACERS, ref)
        out = (torch.empty_like(ghN), torch.empty_like(guN), torch.empty_like(gtN))
        torch.cuda.synchronize()
        st.vjp_tracers(ghN, guN, gtN, out=out)
        return (None,) + out + (None, None, None)
