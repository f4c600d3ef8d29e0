"""Hand-written adjoint of the sw RK4 step (GPU): gradients against FP64
central finite differences of the forward model, independence from the
checkpoint interval, and the torch.autograd.Function contract."""
import numpy as np
import pytest

import mpaso
from mpaso.initial import sw_state

pytestmark = pytest.mark.gpu


def make(level=3, L=2, nu=0.0, seed=4):
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(level)
    dm = G.DeviceMesh(mesh)
    st = G.State(dm, nlev=L, ntr=0, nu=nu)
    h, u, _ = sw_state(mesh, seed, L, 1)
    return mesh, dm, st, h, u


def J(st, h, u, dt, n, wh, wu):
    import mpaso.gpu as G
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.step(dt, n)
    return float((wh * st.get(G.FIELD_H)).sum() + (wu * st.get(G.FIELD_U)).sum())


@pytest.mark.parametrize("nu", [0.0, 2e5])
def test_gradient_matches_central_differences(nu):
    import mpaso.gpu as G
    mesh, dm, st, h, u = make(nu=nu)
    rng = np.random.default_rng(1)
    wh, wu = rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 100
    dt, n = 300.0, 6
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.forward(dt, n, 2)
    gh, gu = st.vjp(wh, wu)
    for _ in range(4):
        dh = rng.standard_normal(h.shape) * 0.05
        du = rng.standard_normal(u.shape) * 2e-4
        eps = 1.0
        fd = (J(st, h + eps * dh, u + eps * du, dt, n, wh, wu) -
              J(st, h - eps * dh, u - eps * du, dt, n, wh, wu)) / (2 * eps)
        ad = float((gh * dh).sum() + (gu * du).sum())
        assert abs(fd - ad) <= 2e-6 * (abs(ad) + 1e-3 * np.abs(gh * dh).sum()), (fd, ad)


def test_checkpoint_interval_does_not_change_gradient():
    import mpaso.gpu as G
    mesh, dm, st, h, u = make(level=2, L=1, nu=1e5)
    rng = np.random.default_rng(2)
    wh, wu = rng.standard_normal(h.shape), rng.standard_normal(u.shape)
    grads = []
    for k in (1, 3, 7, 0):  # 0: the window stored, no recompute
        st.set(G.FIELD_H, h)
        st.set(G.FIELD_U, u)
        st.forward(450.0, 7, k)
        grads.append(st.vjp(wh, wu))
    for g in grads[1:]:
        assert np.array_equal(g[0], grads[0][0]) and np.array_equal(g[1], grads[0][1])


def test_overlapped_recompute_matches_stored_window_at_level5():
    """Level 5 (10,242 cells: two tape sets, the next segment recomputed on a
    side stream while the current one is reversed), 12 steps in segments of 5,
    5 and 2: the gradient equals the stored window's bit for bit, on repeated
    sweeps too."""
    import mpaso.gpu as G
    mesh, dm, st, h, u = make(level=5, L=1, nu=1e4)
    rng = np.random.default_rng(5)
    wh, wu = rng.standard_normal(h.shape), rng.standard_normal(u.shape)
    grads = []
    for k in (0, 5, 5):
        st.set(G.FIELD_H, h)
        st.set(G.FIELD_U, u)
        st.forward(120.0, 12, k)
        grads.append(st.vjp(wh, wu))
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.forward(120.0, 12, 5)
    st.vjp(wh, wu)
    grads.append(st.vjp(wh, wu))  # a second sweep after one forward: every segment recomputed
    for g in grads[1:]:
        assert np.array_equal(g[0], grads[0][0]) and np.array_equal(g[1], grads[0][1])


def test_autograd_function_contract():
    torch = pytest.importorskip("torch")
    import mpaso.gpu as G
    from mpaso.autograd import RK4
    mesh, dm, st, h, u = make(level=3, L=1)
    target = torch.from_numpy(h * 0.999).cuda()
    h0 = torch.from_numpy(h).cuda().requires_grad_(True)
    u0 = torch.from_numpy(u).cuda().requires_grad_(True)
    hN, uN = RK4.apply(st, h0, u0, 300.0, 5, 2)
    loss = 0.5 * ((hN - target) ** 2).sum()
    loss.backward()
    # same cotangent through the raw entry points
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.forward(300.0, 5, 2)
    gh, gu = st.vjp((hN - target).detach().cpu().numpy(), np.zeros_like(u))
    assert np.allclose(h0.grad.cpu().numpy(), gh, rtol=0, atol=1e-12 * np.abs(gh).max())
    assert np.allclose(u0.grad.cpu().numpy(), gu, rtol=0, atol=1e-12 * np.abs(gu).max())


@pytest.mark.parametrize("nu", [0.0, 2e5])
def test_adjoint_dot_product_against_complex_step(nu):
    """<w, J v> from the complex-step tangent of the CPU restatement of the
    reference step equals <J^T w, v> from the CUDA adjoint (relative 1e-10:
    both are exact derivatives, of functions that agree to rounding)."""
    import mpaso.gpu as G
    from sw_complex import SwComplex
    mesh, dm, st, h, u = make(level=3, L=2, nu=nu)
    rng = np.random.default_rng(7)
    wh, wu = rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 100
    dt, n = 300.0, 6
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.forward(dt, n, 2)
    gh, gu = st.vjp(wh, wu)
    C = SwComplex(mesh, 2, nu=nu)
    for _ in range(3):
        vh, vu = rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 1e-3
        jh, ju = C.jvp(h, u, vh, vu, dt, n)
        lhs = float((wh.ravel() * jh.ravel()).sum() + (wu.ravel() * ju.ravel()).sum())
        rhs = float((gh.ravel() * vh.ravel()).sum() + (gu.ravel() * vu.ravel()).sum())
        scale = np.abs(wh.ravel() * jh.ravel()).sum() + np.abs(wu.ravel() * ju.ravel()).sum()
        assert abs(lhs - rhs) <= 1e-10 * scale, (lhs, rhs)
