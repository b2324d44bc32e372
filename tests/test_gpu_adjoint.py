"""GPU checks of the hand-written adjoint (reverse mode of the time step).

Reference gradients come from the host tangent-linear model (oracle/
euler_tlm.c, pinned to the reference's operators on dual numbers by the CPU
tests) through the dot-product identity <J^T w, v> = <w, J v>, and from
central differences of the FP64 GPU solver with dt held at the forward
sequence.  The functional is the one of the differentiation workload: J =
sum of rho(T) * dv over the cells whose centres lie in [0.4, 0.6]^3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 1.4


def implode_noise(O, nx, sigma=1e-3, seed=0):
    """init_implode on an nx^3 interior (ghosts included) with seeded
    Gaussian noise N(0, sigma^2) added to the density of every cell."""
    n = nx + 2
    prim = O.init_implode(n, n, n, (1.0 / nx,) * 3)
    rng = np.random.Generator(np.random.PCG64(seed))
    prim[0] += rng.normal(0.0, sigma, size=prim.shape[1:])
    return prim


def box_weight(nx):
    """dv on cells whose centres ((i-1)+1/2)/nx lie in [0.4, 0.6]^3, else 0."""
    n = nx + 2
    x = (np.arange(n) - 1 + 0.5) / nx
    inside = (x >= 0.4) & (x <= 0.6)
    w = np.zeros((n, n, n))
    w[np.ix_(inside, inside, inside)] = 1.0 / nx ** 3
    return w


def test_godunov_adjoint_dot_product(cuda, euler, oracle_lib):
    torch, O = cuda, oracle_lib
    rng = np.random.default_rng(1)
    for case in ("generic", "rest"):
        prim = O.random_prim(18, 13, 11, seed=4)
        if case == "rest":
            prim[1] = 1.0
            prim[2:] = 0.0
        cons = O.prim_to_cons(prim, GAMMA)
        dx = (0.05, 0.07, 0.06)
        for _ in range(3):
            w = rng.normal(size=prim.shape)
            v = rng.normal(size=prim.shape)
            pb = euler.godunov_adjoint(torch.from_numpy(prim).cuda(), torch.from_numpy(w).cuda(), GAMMA, dx, 1e-3)
            torch.cuda.synchronize()
            _, jv = O.tlm_godunov(prim, v, cons, np.zeros_like(cons), GAMMA, dx, 1e-3)
            lhs = float(np.sum(pb.cpu().numpy() * v))
            rhs = float(np.sum(w * jv))
            assert abs(lhs - rhs) <= 1e-12 * abs(rhs), (case, lhs, rhs)


def test_pointwise_adjoints(cuda, euler, oracle_lib):
    torch, O = cuda, oracle_lib
    rng = np.random.default_rng(2)
    prim = O.random_prim(7, 6, 5, seed=9)
    cons = O.prim_to_cons(prim, GAMMA)
    pt = torch.from_numpy(prim).cuda()
    w = rng.normal(size=prim.shape)
    v = rng.normal(size=prim.shape)
    # cons_to_prim' at cons: <C^T w, v> = <w, C v>
    cb = euler.cons_to_prim_adjoint(pt, torch.from_numpy(w).cuda(), GAMMA)
    _, jv = O.tlm_cons_to_prim(cons, v, GAMMA)
    lhs, rhs = float(np.sum(cb.cpu().numpy() * v)), float(np.sum(w * jv))
    assert abs(lhs - rhs) <= 1e-12 * abs(rhs)
    # prim_to_cons' at prim, accumulating onto an existing gradient
    base = torch.from_numpy(v).cuda()
    pb = euler.prim_to_cons_adjoint(pt, torch.from_numpy(w).cuda(), GAMMA, out=base.clone(), accumulate=True)
    _, jv = O.tlm_prim_to_cons(prim, v, GAMMA)
    lhs = float(np.sum((pb.cpu().numpy() - v) * v))
    rhs = float(np.sum(w * jv))
    assert abs(lhs - rhs) <= 1e-12 * abs(rhs)


@pytest.mark.parametrize("every", [1, 7, 30])
def test_loop_gradient_vs_tangent_linear(cuda, euler, oracle_lib, every):
    """Checkpointed gradient of J against host tangent-linear directional
    derivatives (the dt sequence of the GPU forward pass held fixed in both)."""
    torch, O = cuda, oracle_lib
    nx, nsteps = 24, 30
    prim0 = implode_noise(O, nx, seed=3)
    n = nx + 2
    w = box_weight(nx)
    adj = euler.Adjoint(n, n, n, nsteps, gamma=GAMMA, checkpoint_every=every)
    out = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
    adj.forward(torch.from_numpy(prim0).cuda(), out=out)
    dts = adj.dts()
    gT = torch.zeros_like(out)
    gT[0] = torch.from_numpy(w).cuda()
    g0 = torch.empty_like(out)
    adj.backward(gT, g0)
    grad = g0.cpu().numpy()
    pT_ref, _ = O.tlm_simulate(prim0, np.zeros_like(prim0), GAMMA, (1.0 / nx,) * 3, dts)
    assert np.abs(out.cpu().numpy() - pT_ref).max() <= 1e-12
    rng = np.random.default_rng(5)
    for _ in range(3):
        v = np.zeros_like(prim0)
        v[0] = rng.normal(size=prim0.shape[1:])
        v[1] = rng.normal(size=prim0.shape[1:])
        _, dT = O.tlm_simulate(prim0, v, GAMMA, (1.0 / nx,) * 3, dts)
        ref = float(np.sum(w * dT[0]))
        got = float(np.sum(grad * v))
        assert abs(got - ref) <= 1e-10 * abs(ref), (got, ref)


def test_checkpoint_interval_does_not_change_the_gradient(cuda, euler, oracle_lib):
    torch, O = cuda, oracle_lib
    nx, nsteps = 16, 23
    n = nx + 2
    prim0 = torch.from_numpy(implode_noise(O, nx, seed=8)).cuda()
    gT = torch.zeros((5, n, n, n), dtype=torch.float64, device="cuda")
    gT[0] = torch.from_numpy(box_weight(nx)).cuda()
    grads = []
    for every in (1, 5, 23, 100):
        adj = euler.Adjoint(n, n, n, nsteps, gamma=GAMMA, checkpoint_every=every)
        adj.forward(prim0)
        g0 = torch.empty_like(gT)
        adj.backward(gT, g0)
        grads.append(g0.cpu().numpy())
        adj.close()
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])


def test_autograd_function(cuda, euler, oracle_lib):
    torch, O = cuda, oracle_lib
    from euler_gb300.autograd import evolve

    nx, nsteps = 16, 12
    n = nx + 2
    w = torch.from_numpy(box_weight(nx)).cuda()
    prim0 = torch.from_numpy(implode_noise(O, nx, seed=6)).cuda().requires_grad_(True)
    out = evolve(prim0, nsteps, checkpoint_every=5)
    J = (out[0] * w).sum()
    J.backward()
    adj = euler.Adjoint(n, n, n, nsteps, checkpoint_every=5)
    ref_out = torch.empty_like(out)
    adj.forward(prim0.detach(), out=ref_out)
    gT = torch.zeros_like(out)
    gT[0] = w
    g0 = torch.empty_like(out)
    adj.backward(gT, g0)
    assert torch.equal(out.detach(), ref_out)
    assert torch.equal(prim0.grad, g0)
    # J through autograd matches central differences on the fixed dt sequence
    dts = adj.dts()
    rng = np.random.default_rng(11)
    v = torch.zeros_like(out)
    v[0] = torch.from_numpy(rng.normal(size=(n, n, n))).cuda()
    v[1] = torch.from_numpy(rng.normal(size=(n, n, n))).cuda()
    eps = 1e-6
    with euler.Simulation(n, n, n, GAMMA, (1.0 / nx,) * 3) as sim:
        sim.set_dt_sequence(dts)
        vals = []
        for s in (1.0, -1.0):
            sim.set_prim((prim0.detach() + s * eps * v).contiguous())
            sim.advance(nsteps)
            p = torch.empty_like(out)
            sim.get_state(prim=p)
            vals.append(float((p[0] * w).sum()))
    fd = (vals[0] - vals[1]) / (2 * eps)
    an = float((g0 * v).sum())
    assert abs(fd - an) <= 1e-5 * abs(an), (fd, an)


def test_adjoint_argument_errors(cuda, euler):
    torch = cuda
    n = 10
    adj = euler.Adjoint(n, n, n, 4)
    g = torch.zeros((5, n, n, n), dtype=torch.float64, device="cuda")
    with pytest.raises(euler.EulerError):
        adj.backward(g, torch.empty_like(g))  # no forward pass yet
    with pytest.raises(ValueError):
        adj.forward(g, dts=[1e-3] * 3)  # wrong length
    with pytest.raises(euler.EulerError):
        adj.forward(torch.ones_like(g), dts=[1e-3, -1.0, 1e-3, 1e-3])  # non-positive dt
    with pytest.raises(euler.EulerError):
        euler.Adjoint(n, n, n, 4, checkpoint_every=0)
    prim = torch.ones_like(g)
    with pytest.raises(euler.EulerError):  # output aliases the input
        euler.godunov_adjoint(prim, g, GAMMA, (0.1,) * 3, 1e-3, out=prim)
