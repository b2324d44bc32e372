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


def _c5_case(torch, euler, O, nx, nsteps, every, seed=0):
    n = nx + 2
    prim0 = implode_noise(O, nx, seed=seed)
    w = box_weight(nx)
    adj = euler.Adjoint(n, n, n, nsteps, gamma=GAMMA, checkpoint_every=every)
    out = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
    adj.forward(torch.from_numpy(prim0).cuda(), out=out)
    dts = adj.dts()
    gT = torch.zeros_like(out)
    gT[0] = torch.from_numpy(w).cuda()
    g0 = torch.empty_like(out)
    adj.backward(gT, g0)
    return prim0, w, dts, g0.cpu().numpy(), adj


def _central_differences(torch, euler, prim0, w, dts, grad, ndirs, eps=1e-6, seed=2024):
    n2, n1, n0 = prim0.shape[1:]
    nx = n0 - 2
    rng = np.random.default_rng(seed)
    wt = torch.from_numpy(w).cuda()
    rows = []
    with euler.Simulation(n0, n1, n2, GAMMA, (1.0 / nx,) * 3) as sim:
        sim.set_dt_sequence(dts)
        p = torch.empty((5, n2, n1, n0), dtype=torch.float64, device="cuda")
        for _ in range(ndirs):
            v = np.zeros_like(prim0)
            v[0] = rng.normal(size=prim0.shape[1:])
            v[1] = rng.normal(size=prim0.shape[1:])
            vals = []
            for s in (1.0, -1.0):
                sim.set_prim(torch.from_numpy(prim0 + s * eps * v).cuda())
                sim.advance(len(dts))
                sim.get_state(prim=p)
                vals.append(float((p[0] * wt).sum()))
            rows.append((float(np.sum(grad * v)), (vals[0] - vals[1]) / (2 * eps), v))
    return rows


def test_differentiation_workload_reduced(cuda, euler, oracle_lib):
    """The differentiation workload on a 64^3 grid for 100 steps: gradient
    against the tangent-linear model (tight) and central differences (eps =
    1e-6).  Central differences of this solver carry errors of ~1e-5 of the
    directional derivatives' size: the flux has kinks at the initial state
    (ustar == 0 on every face of the quiet gas) and near it, and the host
    tangent-linear model, which shares no code with the GPU, shows the same
    spread against them; the bound below is that measured spread with margin."""
    torch, O = cuda, oracle_lib
    nx, nsteps = 64, 100
    prim0, w, dts, grad, _ = _c5_case(torch, euler, O, nx, nsteps, 20)
    rng = np.random.default_rng(9)
    for _ in range(2):
        v = np.zeros_like(prim0)
        v[0] = rng.normal(size=prim0.shape[1:])
        v[1] = rng.normal(size=prim0.shape[1:])
        _, dT = O.tlm_simulate(prim0, v, GAMMA, (1.0 / nx,) * 3, dts)
        ref = float(np.sum(w * dT[0]))
        # the GPU forward pass and the oracle's agree to ~1e-12 here, not bit
        # for bit, and the derivative of a piecewise-smooth solver moves with
        # its linearisation point wherever a face sits that close to a kink
        assert abs(float(np.sum(grad * v)) - ref) <= 1e-7 * abs(ref)
    rows = _central_differences(torch, euler, prim0, w, dts, grad, 4)
    rms = float(np.sqrt(np.mean([a * a for a, _, _ in rows])))
    for a, fd, _ in rows:
        assert abs(fd - a) <= 2e-4 * rms, (a, fd)


def test_differentiation_workload_full(cuda, euler, oracle_lib):
    """The differentiation workload as specified: 128^3, 400 steps,
    checkpoints every 20; the gradient against the host tangent-linear model
    along one direction (the host run takes about half a minute on 16
    cores), and 16 central differences; prints one JSON line with the
    figures."""
    import json
    import time

    torch, O = cuda, oracle_lib
    nx, nsteps = 128, 400
    t0 = time.perf_counter()
    prim0, w, dts, grad, adj = _c5_case(torch, euler, O, nx, nsteps, 20)
    t_adj = time.perf_counter() - t0
    rows = _central_differences(torch, euler, prim0, w, dts, grad, 16)
    a, fd, v = rows[0]
    t0 = time.perf_counter()
    _, dT = O.tlm_simulate(prim0, v, GAMMA, (1.0 / nx,) * 3, dts)
    t_tlm = time.perf_counter() - t0
    tlm = float(np.sum(w * dT[0]))
    rms = float(np.sqrt(np.mean([r[0] ** 2 for r in rows])))
    rec = {"differentiation_full": {
        "grid": f"{nx}^3", "steps": nsteps, "checkpoint_every": 20, "adjoint_wall_s": t_adj,
        "tlm_wall_s": t_tlm, "tlm": tlm, "adjoint": a, "adjoint_vs_tlm_rel": abs(a - tlm) / abs(tlm),
        "fd_vs_tlm_rel": abs(fd - tlm) / abs(tlm),
        "fd_rel_errs": [abs(f - g) / abs(g) for g, f, _ in rows],
        "fd_max_err_over_rms": max(abs(f - g) for g, f, _ in rows) / rms}}
    print(json.dumps(rec))
    assert abs(a - tlm) <= 1e-6 * abs(tlm)


def smooth_prim(nx):
    """A smooth, subsonic, everywhere-moving state on an nx^3 interior (ghosts
    included), away from every kink of the HLLC flux: on each axis the normal
    velocity rises strictly from cell to cell (so min/max of un_L, un_R never
    tie), the sound speed rises strictly along every axis (rho falls, p rises),
    every velocity is positive and well below the sound speed (ustar > 0 and
    S_L < 0 < S_R on every face)."""
    n = nx + 2
    x = (np.arange(n) - 1 + 0.5) / nx
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    s = (X + Y + Z) / 3
    prim = np.empty((5, n, n, n))
    prim[0] = 1.0 - 0.1 * s
    prim[1] = 1.0 + 0.3 * s
    prim[2] = np.broadcast_to(0.3 + 0.2 * X, (n, n, n))
    prim[3] = np.broadcast_to(0.2 + 0.15 * Y, (n, n, n))
    prim[4] = np.broadcast_to(0.25 + 0.1 * Z, (n, n, n))
    return prim


def test_smooth_state_central_differences(cuda, euler, oracle_lib):
    """On a kink-free state (64^3, 50 CFL steps held fixed) the adjoint
    gradient of J matches central differences (eps = 1e-6) of the FP64 GPU
    solver to 1e-6 relative along each of 8 seeded random (rho, p)
    directions.  This separates the adjoint's own error from the HLLC kinks
    that spread the differentiation workload's central differences (its quiet
    gas sits on ustar == 0 at every face).  Measured: ~1e-9, the floor of the
    differences' rounding."""
    torch, O = cuda, oracle_lib
    nx, nsteps = 64, 50
    n = nx + 2
    prim0 = smooth_prim(nx)
    w = box_weight(nx)
    adj = euler.Adjoint(n, n, n, nsteps, gamma=GAMMA, checkpoint_every=10)
    out = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
    adj.forward(torch.from_numpy(prim0).cuda(), out=out)
    dts = adj.dts()
    gT = torch.zeros_like(out)
    gT[0] = torch.from_numpy(w).cuda()
    g0 = torch.empty_like(out)
    adj.backward(gT, g0)
    adj.close()
    grad = g0.cpu().numpy()
    rows = _central_differences(torch, euler, prim0, w, dts, grad, 8, seed=77)
    for a, fd, _ in rows:
        assert abs(fd - a) <= 1e-6 * abs(a), (a, fd, abs(fd - a) / abs(a))


def test_ragged_anisotropic_grid_and_all_fields(cuda, euler, oracle_lib):
    """Odd, unequal extents (the forward step's plain-load path), unequal
    spacings, a generic moving state, a cotangent on every final field, and
    a direction in all five initial fields."""
    torch, O = cuda, oracle_lib
    n0, n1, n2 = 21, 17, 13
    dx = (0.05, 0.07, 0.06)
    prim0 = O.random_prim(n0, n1, n2, seed=13)
    prim0[2:] *= 0.3
    nsteps = 8
    adj = euler.Adjoint(n0, n1, n2, nsteps, gamma=1.3, dx=dx, checkpoint_every=3)
    out = torch.empty((5, n2, n1, n0), dtype=torch.float64, device="cuda")
    adj.forward(torch.from_numpy(prim0).cuda(), out=out)
    dts = adj.dts()
    rng = np.random.default_rng(21)
    wT = rng.normal(size=prim0.shape)
    g0 = torch.empty_like(out)
    adj.backward(torch.from_numpy(wT).cuda(), g0)
    grad = g0.cpu().numpy()
    for _ in range(3):
        v = rng.normal(size=prim0.shape)
        _, dT = O.tlm_simulate(prim0, v, 1.3, dx, dts)
        ref = float(np.sum(wT * dT))
        got = float(np.sum(grad * v))
        assert abs(got - ref) <= 1e-10 * abs(ref), (got, ref)
