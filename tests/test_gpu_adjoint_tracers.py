"""Hand-written adjoint of the sw RK4 step with tracers (GPU): FCT advection
and del2 mixing differentiated on the branch the forward takes, checked by
the dot-product identity against the complex-step tangent of the CPU
restatement of the reference step, and against central differences of the
CUDA forward."""
import numpy as np
import pytest

import mpaso
from mpaso.initial import sw_state
from mpaso.setup import fct_statics

pytestmark = pytest.mark.gpu

KAPPA = 2e6


def rough_state(mesh, L, T, seed):
    """Smooth state with tracers 0.7 smooth + 0.3 cell noise: the noise makes
    local extrema everywhere, so about 5% of the FCT limiter factors are
    strictly inside (0, 1) and their derivative is exercised."""
    h, u, tr = sw_state(mesh, seed, L, T)
    rng = np.random.default_rng(seed + 100)
    return h, u, 0.7 * tr + 0.3 * rng.uniform(0.0, 1.0, tr.shape)


def make(L, T, fct, hmix, nu=0.0, level=3, seed=3):
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(level)
    f = fct_statics(mesh, L)
    dm = G.DeviceMesh(mesh, fct=f)
    st = G.State(dm, nlev=L, ntr=T, fct=fct, hmix=hmix, kappa=KAPPA if hmix else 0.0, nu=nu)
    return mesh, f, st, rough_state(mesh, L, T, seed)


def set_state(st, h, u, tr):
    import mpaso.gpu as G
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.set(G.FIELD_TRACERS, tr)


def dot(a, b):
    return float(sum((x.ravel() * y.ravel()).sum() for x, y in zip(a, b)))


@pytest.mark.parametrize("fct,hmix,nu", [(True, True, 0.0), (True, False, 1e5), (False, True, 0.0)])
def test_tracer_adjoint_dot_product_against_complex_step(fct, hmix, nu):
    """<w, J v> from the complex step of the restatement (every max / min /
    clamp decided on the real part) equals <J^T w, v> from the CUDA adjoint to
    1e-10 of the sum of |terms|: both are exact derivatives on the same
    branch of functions that agree to rounding."""
    from sw_complex import SwComplex
    L, T, dt, n = 2, 2, 300.0, 4
    mesh, f, st, (h, u, tr) = make(L, T, fct, hmix, nu)
    rng = np.random.default_rng(11)
    w = (rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 100, rng.standard_normal(tr.shape) * 1e3)
    set_state(st, h, u, tr)
    st.forward(dt, n, 2)
    g = st.vjp_tracers(*w)
    C = SwComplex(mesh, L, fct=f, centred=not fct, T=T, hmix=hmix, kappa=KAPPA if hmix else 0.0, nu=nu)
    for _ in range(2):
        v = (rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 1e-3, rng.standard_normal(tr.shape) * 1e-2)
        jv = C.jvp_tracers(h, u, tr, *v, dt, n)
        lhs, rhs = dot(w, jv), dot(g, v)
        scale = sum(np.abs(x.ravel() * y.ravel()).sum() for x, y in zip(w, jv))
        assert abs(lhs - rhs) <= 1e-10 * scale, (lhs, rhs, scale)
        # the tracer part alone (v = (0, 0, vt)) checks the limiter's transpose in isolation
        vt = (np.zeros(h.shape), np.zeros(u.shape), v[2])
        jt = C.jvp_tracers(h, u, tr, *vt, dt, n)
        lt, rt = dot(w, jt), dot(g, vt)
        st_ = sum(np.abs(x.ravel() * y.ravel()).sum() for x, y in zip(w, jt))
        assert abs(lt - rt) <= 1e-10 * st_, (lt, rt, st_)


def test_tracer_adjoint_matches_central_differences_of_the_cuda_forward():
    """The gradient of J = <w, state_N> against central differences of the CUDA
    forward itself, along directions small enough to keep every limiter branch."""
    import mpaso.gpu as G
    L, T, dt, n = 1, 2, 300.0, 3
    mesh, f, st, (h, u, tr) = make(L, T, True, True)
    rng = np.random.default_rng(5)
    w = (rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 100, rng.standard_normal(tr.shape) * 1e3)

    def J(x):
        set_state(st, *x)
        st.step(dt, n)
        return dot(w, (st.get(G.FIELD_H), st.get(G.FIELD_U), st.get(G.FIELD_TRACERS)))

    set_state(st, h, u, tr)
    st.forward(dt, n, n)
    g = st.vjp_tracers(*w)
    for _ in range(3):
        v = (rng.standard_normal(h.shape) * 0.05, rng.standard_normal(u.shape) * 2e-4,
             rng.standard_normal(tr.shape) * 1e-3)
        eps = 1e-4
        fd = (J([a + eps * b for a, b in zip((h, u, tr), v)]) -
              J([a - eps * b for a, b in zip((h, u, tr), v)])) / (2 * eps)
        ad = dot(g, v)
        assert abs(fd - ad) <= 1e-6 * sum(np.abs(x * y).sum() for x, y in zip(g, v)), (fd, ad)


def test_tracer_adjoint_checkpoint_interval_and_hu_consistency():
    """The checkpoint interval does not change the gradient (bit for bit), and
    with zero tracer cotangents the (h, u) gradient is the tracer-free one."""
    L, T, dt, n = 1, 3, 450.0, 5
    mesh, f, st, (h, u, tr) = make(L, T, True, True, level=2)
    rng = np.random.default_rng(2)
    w = (rng.standard_normal(h.shape), rng.standard_normal(u.shape), rng.standard_normal(tr.shape))
    grads = []
    for k in (1, 2, 5):
        set_state(st, h, u, tr)
        st.forward(dt, n, k)
        grads.append(st.vjp_tracers(*w))
    for gk in grads[1:]:
        for a, b in zip(gk, grads[0]):
            assert np.array_equal(a, b)
    set_state(st, h, u, tr)
    st.forward(dt, n, 2)
    gh, gu, gt = st.vjp_tracers(w[0], w[1], np.zeros(tr.shape))
    assert np.all(gt == 0.0)
    gh2, gu2 = st.vjp(w[0], w[1])
    assert np.array_equal(gh, gh2) and np.array_equal(gu, gu2)


def test_stored_window_gives_the_checkpointed_gradient():
    """ckpt_every = 0 tapes the whole window during the forward: same final state
    and, for the tracer vjp (same kernels both ways), the same gradient bit for
    bit as checkpointing; the (h, u) vjp (tracer-free recompute kernels when
    checkpointing) agrees to rounding."""
    import mpaso.gpu as G
    L, T, dt, n = 1, 2, 300.0, 5
    mesh, f, st, (h, u, tr) = make(L, T, True, True, level=2)
    rng = np.random.default_rng(9)
    w = (rng.standard_normal(h.shape), rng.standard_normal(u.shape), rng.standard_normal(tr.shape))
    out = {}
    for k in (2, 0):
        set_state(st, h, u, tr)
        st.forward(dt, n, k)
        fin = (st.get(G.FIELD_H), st.get(G.FIELD_U), st.get(G.FIELD_TRACERS))
        out[k] = (fin, st.vjp_tracers(*w), st.vjp(w[0], w[1]))
    for a, b in zip(out[0][0], out[2][0]):
        assert np.array_equal(a, b)
    for a, b in zip(out[0][1], out[2][1]):
        assert np.array_equal(a, b)
    for a, b in zip(out[0][2], out[2][2]):
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def test_autograd_function_with_tracers():
    """RK4Tracers through torch.autograd gives the raw vjp_tracers gradient."""
    torch = pytest.importorskip("torch")
    from mpaso.autograd import RK4Tracers
    L, T, dt, n = 1, 1, 300.0, 3
    mesh, f, st, (h, u, tr) = make(L, T, True, True, level=3)
    target = torch.from_numpy(tr * 0.9).cuda()
    h0 = torch.from_numpy(h).cuda().requires_grad_(True)
    u0 = torch.from_numpy(u).cuda().requires_grad_(True)
    t0 = torch.from_numpy(tr).cuda().requires_grad_(True)
    hN, uN, tN = RK4Tracers.apply(st, h0, u0, t0, dt, n, 0)
    loss = 0.5 * ((tN - target) ** 2).sum()
    loss.backward()
    set_state(st, h, u, tr)
    st.forward(dt, n, 0)
    g = st.vjp_tracers(np.zeros_like(h), np.zeros_like(u), (tN - target).detach().cpu().numpy())
    for got, want in zip((h0.grad, u0.grad, t0.grad), g):
        assert np.allclose(got.cpu().numpy(), want, rtol=0, atol=1e-12 * np.abs(want).max())
