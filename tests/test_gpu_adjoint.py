"""Discrete adjoint of the time loop (sg_adjoint_*): the recorded forward is
the ordinary loop, the replay on the recorded meshes reproduces it, and the
backward pass is the exact transpose of the frozen-mesh map: dot-product test,
central finite differences in u0 (exact for the quadratic J up to rounding)
and in a, checkpoint interval invariance, and the torch.autograd binding."""
import numpy as np
import pytest

from advection_cases import cell_volumes, gaussian_target, shapes_2d

pytestmark = pytest.mark.gpu

MINL, MAXL, STEPS, EPS, REG = 3, 7, 40, 1e-3, 2.0
A = (1.0, 0.7)
DT = 0.5 / (1 << MAXL)


@pytest.fixture(scope="module")
def sg():
    from samurai_gb300 import build

    build.build()
    import samurai_gb300

    return samurai_gb300


def initial_sim(sg):
    s = sg.AdvectionSim(2, MINL, MAXL)
    lv, co, _ = s.cells()
    s.set_cell_values(shapes_2d(31, 4, 4)(lv, co))
    s.adapt(EPS, REG)
    return s


def objective(adj, uT):
    lv, co = adj.cells("final")
    tgt = gaussian_target(5)(lv, co)
    vol = cell_volumes(lv)
    J = float(np.sum(vol * (uT - tgt) ** 2))
    return J, 2.0 * vol * (uT - tgt)


def test_record_is_the_loop_and_replay_reproduces_it(sg):
    s = initial_sim(sg)
    adj = sg.Adjoint(s.u, checkpoint_every=8)
    u0 = s.cell_values()
    uT = adj.record(u0, STEPS, EPS, REG, A, DT)
    for _ in range(STEPS):
        s.adapt(EPS, REG)
        s.update_ghost()
        s.upwind(A, DT)
    lv, co = adj.cells("final")
    lg, cg, _ = s.cells()
    assert np.array_equal(lv, lg) and np.array_equal(co, cg)
    assert np.array_equal(uT, s.cell_values())
    assert np.array_equal(adj.replay(u0, A), uT)


def test_dot_product(sg):
    s = initial_sim(sg)
    adj = sg.Adjoint(s.u, checkpoint_every=8)
    u0 = s.cell_values()
    adj.record(u0, STEPS, EPS, REG, A, DT)
    n0, nT, _ = adj.counts()
    rng = np.random.default_rng(3)
    for _ in range(3):
        v = rng.standard_normal(n0)
        w = rng.standard_normal(nT)
        Lv = adj.replay(v, A)  # Dirichlet 0: the frozen map is linear
        LTw, _ = adj.backward(w)
        lhs, rhs = float(Lv @ w), float(v @ LTw)
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs), 1e-300) * 10, (lhs, rhs)


def test_gradient_against_finite_differences(sg):
    s = initial_sim(sg)
    adj = sg.Adjoint(s.u, checkpoint_every=8)
    u0 = s.cell_values()
    uT = adj.record(u0, STEPS, EPS, REG, A, DT)
    J, gT = objective(adj, uT)
    g0, ga = adj.backward(gT)
    rng = np.random.default_rng(11)
    for _ in range(8):
        v = rng.standard_normal(len(u0))
        h = 1e-3
        jp, _ = objective(adj, adj.replay(u0 + h * v, A))
        jm, _ = objective(adj, adj.replay(u0 - h * v, A))
        fd = (jp - jm) / (2 * h)
        assert abs(fd - g0 @ v) <= 1e-8 * max(abs(fd), 1e-12), (fd, g0 @ v)
    for d in range(2):
        h = 1e-6
        ap, am = list(A), list(A)
        ap[d] += h
        am[d] -= h
        jp, _ = objective(adj, adj.replay(u0, ap))
        jm, _ = objective(adj, adj.replay(u0, am))
        fd = (jp - jm) / (2 * h)
        assert abs(fd - ga[d]) <= 1e-6 * max(abs(fd), 1e-12), (d, fd, ga[d])


def test_checkpoint_interval_does_not_change_the_gradient(sg):
    s = initial_sim(sg)
    u0 = s.cell_values()
    res = []
    for k in (1, 8, STEPS):
        adj = sg.Adjoint(s.u, checkpoint_every=k)
        uT = adj.record(u0, STEPS, EPS, REG, A, DT)
        _, gT = objective(adj, uT)
        res.append(adj.backward(gT))
        adj.close()
    for g0, ga in res[1:]:
        np.testing.assert_allclose(g0, res[0][0], rtol=1e-12, atol=1e-18)
        np.testing.assert_allclose(ga, res[0][1], rtol=1e-12)


def test_torch_autograd(sg):
    torch = pytest.importorskip("torch")
    from samurai_gb300.autograd import advection_loop

    s = initial_sim(sg)
    adj = sg.Adjoint(s.u, checkpoint_every=8)
    u0 = torch.tensor(s.cell_values(), dtype=torch.float64, requires_grad=True)
    a = torch.tensor(A, dtype=torch.float64, requires_grad=True)
    uT = advection_loop(u0, a, adj, STEPS, EPS, REG, DT)
    lv, co = adj.cells("final")
    tgt = torch.from_numpy(gaussian_target(5)(lv, co))
    vol = torch.from_numpy(cell_volumes(lv))
    J = (vol * (uT - tgt) ** 2).sum()
    J.backward()
    g0, ga = adj.backward((2 * vol * (uT - tgt)).detach().numpy())
    # the transposed launches accumulate with atomics: equal up to rounding order
    np.testing.assert_allclose(u0.grad.numpy(), g0, rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(a.grad.numpy(), ga, rtol=1e-12)


def test_torch_autograd_cuda_tensors(sg):
    """FP64 CUDA tensors cross the C ABI as device pointers: the same
    gradients as through host arrays, returned on the tensors' device"""
    torch = pytest.importorskip("torch")
    from samurai_gb300.autograd import advection_loop

    s = initial_sim(sg)
    adj = sg.Adjoint(s.u, checkpoint_every=8)
    u0h = s.cell_values()
    u0 = torch.tensor(u0h, dtype=torch.float64, device="cuda", requires_grad=True)
    a = torch.tensor(A, dtype=torch.float64, requires_grad=True)
    uT = advection_loop(u0, a, adj, STEPS, EPS, REG, DT)
    assert uT.is_cuda
    lv, co = adj.cells("final")
    tgt = torch.from_numpy(gaussian_target(5)(lv, co)).cuda()
    vol = torch.from_numpy(cell_volumes(lv)).cuda()
    J = (vol * (uT - tgt) ** 2).sum()
    J.backward()
    assert u0.grad.is_cuda
    uT_host = adj.record(u0h, STEPS, EPS, REG, A, DT)
    assert np.array_equal(uT.detach().cpu().numpy(), uT_host)
    g0, ga = adj.backward((2 * vol * (uT - tgt)).detach().cpu().numpy())
    np.testing.assert_allclose(u0.grad.cpu().numpy(), g0, rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(a.grad.numpy(), ga, rtol=1e-12)
