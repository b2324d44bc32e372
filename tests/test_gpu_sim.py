"""GPU parity of the device-resident simulation (fused step) against the
oracle's reference loop (time_step -> godunov(cfl*dt) -> cons_to_prim).

Tolerances, relative L-infinity per field (max|a-b| / max|ref|):
1e-12 after one step and 1e-10 after 100 steps, FP64."""
import numpy as np
import pytest

from conftest import rel_linf

pytestmark = pytest.mark.gpu

TOL_1 = 1e-12
TOL_100 = 1e-10


def run_oracle_implode(O, nx, steps, cfl=0.4, gamma=1.4):
    n = nx + 2
    dx = (1.0 / nx,) * 3
    prim = O.init_implode(n, n, n, dx)
    cons = O.prim_to_cons(prim, gamma)
    t = O.simulate(prim, cons, gamma, dx, cfl, steps)
    return prim, cons, t


@pytest.mark.parametrize("steps,tol", [(1, TOL_1), (2, TOL_1 * 4), (10, 1e-11), (100, TOL_100)])
def test_implode_64(cuda, euler, oracle_lib, steps, tol):
    nx = 64
    prim_ref, cons_ref, t_ref = run_oracle_implode(oracle_lib, nx, steps)
    n = nx + 2
    with euler.Simulation(n, n, n, 1.4, (1.0 / nx,) * 3, 0.4) as sim:
        sim.init_implode()
        sim.advance(steps)
        prim, cons = sim.state_numpy()
        t, _, st = sim.time()
        assert sim.status() == 0
    assert st == steps
    assert abs(t - t_ref) <= 1e-12 * t_ref
    pe, ce = rel_linf(prim, prim_ref), rel_linf(cons, cons_ref)
    assert max(pe) <= tol and max(ce) <= tol, (pe, ce)


def test_implode_100_steps_time_and_totals(cuda, euler, oracle_lib):
    """The 64^3 / 100-step configuration: simulated time and FP64
    conservation totals against the oracle's."""
    nx = 64
    prim_ref, cons_ref, t_ref = run_oracle_implode(oracle_lib, nx, 100)
    n = nx + 2
    with euler.Simulation(n, n, n, 1.4, (1.0 / nx,) * 3, 0.4) as sim:
        sim.init_implode()
        tot0 = sim.totals()
        sim.advance(100)
        tot = sim.totals()
        t, _, _ = sim.time()
    assert abs(t - 0.121580552) < 1e-9
    interior = cons_ref[:, 1:-1, 1:-1, 1:-1]
    ref_tot = [float(interior[f].sum()) for f in range(5)]
    for f in range(2):  # mass and energy: relative agreement
        assert abs(tot[f] - ref_tot[f]) <= 1e-10 * abs(ref_tot[f])
    for f in range(2, 5):  # momenta: start at 0, stay symmetric
        assert abs(tot[f] - ref_tot[f]) <= 1e-10 * abs(tot0[0])


@pytest.mark.parametrize("shape", [(45, 38, 29), (46, 39, 30)], ids=["odd_n0_plain_loads", "even_n0_tma"])
def test_random_state_steps(cuda, euler, oracle_lib, shape):
    """Seeded random states (rho, p log-uniform [0.1,10], u ~ N(0,1)) on
    ragged grids, 1 and 5 steps: partial tiles at the high edges, staged with
    plain loads (odd n0: rows not a multiple of 16 bytes) and with TMA (even
    n0: the boxes of the edge tiles reach past the array)."""
    O = oracle_lib
    n0, n1, n2 = shape
    dx = (1 / (n0 - 2), 1 / (n1 - 2), 1 / (n2 - 2))
    prim0 = O.random_prim(n0, n1, n2, seed=21)
    for steps, tol in ((1, TOL_1), (5, 1e-11)):
        p = prim0.copy()
        c = O.prim_to_cons(p, 1.4)
        O.simulate(p, c, 1.4, dx, 0.4, steps)
        with euler.Simulation(n0, n1, n2, 1.4, dx, 0.4) as sim:
            sim.set_prim(prim0)
            sim.advance(steps)
            pg, cg = sim.state_numpy()
        pe, ce = rel_linf(pg, p), rel_linf(cg, c)
        assert max(pe) <= tol and max(ce) <= tol, (steps, pe, ce)


@pytest.mark.parametrize("shape", [(514, 20, 12), (515, 18, 10)], ids=["bench_pitch_514_tma", "pitch_515_plain"])
def test_random_state_steps_at_bench_row_pitch(cuda, euler, oracle_lib, shape):
    """The benchmark's row length: 514 cells per row (512 interior, dx =
    1/512), an even n0 whose rows are staged by TMA at the full 4112-byte
    pitch, and 515 (odd: plain loads).  Seeded random states as in the
    benchmark, 1 and 5 steps against the oracle loop."""
    O = oracle_lib
    n0, n1, n2 = shape
    dx = (1 / 512, 1 / 512, 1 / 512)
    prim0 = O.random_prim(n0, n1, n2, seed=514)
    for steps, tol in ((1, TOL_1), (5, 1e-11)):
        p = prim0.copy()
        c = O.prim_to_cons(p, 1.4)
        t_ref = O.simulate(p, c, 1.4, dx, 0.4, steps)
        with euler.Simulation(n0, n1, n2, 1.4, dx, 0.4) as sim:
            sim.set_prim(prim0)
            sim.advance(steps)
            pg, cg = sim.state_numpy()
            t, _, _ = sim.time()
            assert sim.status() == 0
        assert abs(t - t_ref) <= 1e-12 * t_ref
        pe, ce = rel_linf(pg, p), rel_linf(cg, c)
        assert max(pe) <= tol and max(ce) <= tol, (steps, pe, ce)


def test_set_state_and_odd_step_counts(cuda, euler, oracle_lib):
    """advance() in uneven chunks (graph replays plus single steps) equals
    one long advance."""
    O = oracle_lib
    prim0 = O.random_prim(20, 24, 18, seed=2)
    cons0 = O.prim_to_cons(prim0, 1.4)
    dx = (0.05, 0.05, 0.05)
    with euler.Simulation(20, 24, 18, 1.4, dx, 0.3) as a, euler.Simulation(20, 24, 18, 1.4, dx, 0.3) as b:
        a.set_state(prim0, cons0)
        b.set_state(prim0, cons0)
        a.advance(7)
        for k in (1, 3, 2, 1):
            b.advance(k)
        pa, ca = a.state_numpy()
        pb, cb = b.state_numpy()
    assert np.array_equal(pa, pb) and np.array_equal(ca, cb)
    # and both equal the oracle loop: a state loaded with its cons (the
    # load reads e to form e + p) steps like one loaded from prim
    p, c = prim0.copy(), cons0.copy()
    O.simulate(p, c, 1.4, dx, 0.3, 7)
    assert max(rel_linf(pa, p) + rel_linf(ca, c)) <= 1e-11


def test_symmetry_of_implosion(cuda, euler):
    """The implosion is symmetric under axis permutation: density stays
    permutation-symmetric to rounding."""
    nx = 32
    n = nx + 2
    with euler.Simulation(n, n, n, 1.4, (1.0 / nx,) * 3, 0.4) as sim:
        sim.init_implode()
        sim.advance(40)
        prim, _ = sim.state_numpy()
    d = prim[0]
    scale = np.abs(d).max()
    for perm in ((0, 2, 1), (1, 0, 2), (2, 1, 0)):
        assert np.abs(d - d.transpose(perm)).max() <= 1e-12 * scale


def test_tiny_and_degenerate_grids(cuda, euler, oracle_lib):
    O = oracle_lib
    for shape in ((3, 3, 3), (2, 5, 4), (35, 3, 3), (4, 4, 70)):
        prim0 = O.random_prim(*shape, seed=7)
        p = prim0.copy()
        c = O.prim_to_cons(p, 1.4)
        dx = (0.1, 0.1, 0.1)
        O.simulate(p, c, 1.4, dx, 0.4, 3)
        with euler.Simulation(*shape, 1.4, dx, 0.4) as sim:
            sim.set_prim(prim0)
            sim.advance(3)
            pg, cg = sim.state_numpy()
        assert max(rel_linf(pg, p)) <= 1e-11 and max(rel_linf(cg, c)) <= 1e-11, shape


def test_nonphysical_state_is_reported(cuda, euler, oracle_lib):
    """A host-injected negative pressure is flagged, not trapped."""
    prim0 = oracle_lib.random_prim(16, 16, 16, seed=3)
    prim0[1, 8, 8, 8] = -5.0
    with euler.Simulation(16, 16, 16, 1.4, (0.1,) * 3, 0.4) as sim:
        sim.set_prim(prim0)
        sim.advance(2)
        assert sim.status() == -7  # EULR_ERR_NONFINITE


def test_async_state_read_and_fused_load(cuda, euler, oracle_lib):
    """set_prim's one-pass load (prim_to_cons + sound speed + first dt) and the
    asynchronous read agree with the oracle and with the waiting read."""
    torch, O = cuda, oracle_lib
    prim = O.random_prim(20, 18, 16, seed=7)
    gamma, dx = 1.4, (0.05, 0.06, 0.07)
    cons_ref = O.prim_to_cons(prim, gamma)
    dt_ref = 0.4 * O.time_step(prim, gamma, dx)
    host = torch.from_numpy(prim).pin_memory()
    with euler.Simulation(20, 18, 16, gamma, dx, 0.4) as sim:
        sim.set_prim(host)
        p, c = sim.state_numpy()
        assert np.array_equal(c, cons_ref) and np.array_equal(p, prim)
        assert sim.time()[1] == dt_ref
        sim.advance(3)
        a = torch.empty((5, 16, 18, 20), dtype=torch.float64).pin_memory()
        sim.get_state(prim=a, wait=False)
        sim.synchronize()
        b, _ = sim.state_numpy()
        assert np.array_equal(a.numpy(), b)
    with euler.Simulation(20, 18, 16, gamma, dx, 0.4, precision="f32c") as sim:
        sim.set_prim(host)
        with pytest.raises(euler.EulerError):
            sim.get_state(prim=torch.empty((5, 16, 18, 20), dtype=torch.float64), wait=False)


@pytest.mark.parametrize("precision", ["f32c", "f32", "f32c_hilo"])
def test_fp32_tiny_and_ragged_grids(cuda, euler, oracle_lib, precision):
    """The FP32 engines on grids with one interior cell, none, a single partial
    tile (35 x 3 x 3: one row of 33 cells over a 32-wide tile) and long thin
    columns, against the FP64 oracle loop."""
    O = oracle_lib
    for shape in ((3, 3, 3), (2, 5, 4), (35, 3, 3), (4, 4, 70), (37, 12, 5)):
        prim0 = O.random_prim(*shape, seed=9)
        p = prim0.copy()
        c = O.prim_to_cons(p, 1.4)
        dx = (0.1, 0.1, 0.1)
        O.simulate(p, c, 1.4, dx, 0.4, 3)
        with euler.Simulation(*shape, 1.4, dx, 0.4, precision=precision) as sim:
            sim.set_prim(prim0)
            sim.advance(3)
            _, cg = sim.state_numpy()
            assert sim.status() == 0
        assert max(rel_linf(cg, c)) <= 2e-5, (precision, shape, rel_linf(cg, c))


def test_objects_release_their_memory_and_report_oom(cuda, euler):
    """Creating and destroying simulations, batches and adjoints leaves the
    device's free memory where it was; a state larger than the device is an
    out-of-memory status, not a crash."""
    torch = cuda
    free0 = None
    for it in range(6):
        if it == 1:  # after one round: kernels loaded, per-device scratch allocated
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            free0, _ = torch.cuda.mem_get_info()
        with euler.Simulation(66, 66, 66, precision="f64") as s:
            s.init_implode()
            s.advance(2)
        with euler.Simulation(66, 66, 66, precision="f32c") as s:
            s.init_implode()
            s.advance(2)
        with euler.Batch([(34, 26, 18, 1.4, 0.1, 0.1, 0.1)] * 3, precision="f32c") as b:
            for g in range(3):
                b.init_step(g, 0.3, 0.5, 0.5)
            b.advance(2)
        a = euler.Adjoint(18, 18, 18, 4, checkpoint_every=2)
        p = torch.ones((5, 18, 18, 18), dtype=torch.float64, device="cuda")
        p[2:] = 0.0
        a.forward(p)
        g0 = torch.empty_like(p)
        a.backward(torch.zeros_like(p), g0)
        a.close()
        del p, g0
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free1, _ = torch.cuda.mem_get_info()
    assert abs(free1 - free0) < 8 << 20, (free0, free1)
    # 1200^3 cells x 22 FP64 fields is ~300 GB, beyond one GB300
    with pytest.raises(euler.EulerError) as err:
        euler.Simulation(1200, 1200, 1200)
    assert err.value.status == -5  # EULR_ERR_OUT_OF_MEMORY
    # the library keeps working afterwards
    with euler.Simulation(18, 18, 18) as s:
        s.init_implode()
        s.advance(1)
        assert s.status() == 0


def _max_wavespeed_dt(prim, gamma, dx, cfl):
    """cfl / max over cells of sum_d (c + |u_d|) / dx_d (time_step.hpp:28-39),
    c = sqrt(gamma p / rho), in numpy FP64."""
    d, p, u0, u1, u2 = (prim[f].astype(np.float64) for f in range(5))
    c = np.sqrt(gamma * p / d)
    inv = (c + np.abs(u0)) / dx[0] + (c + np.abs(u1)) / dx[1] + (c + np.abs(u2)) / dx[2]
    return cfl / inv.max()


def _screen_state(kind, shape, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    prim = np.empty((5,) + tuple(reversed(shape)), dtype=np.float64)
    if kind == "random":
        prim[0] = np.exp(rng.uniform(np.log(0.1), np.log(10.0), prim[0].shape))
        prim[1] = np.exp(rng.uniform(np.log(0.1), np.log(10.0), prim[1].shape))
        prim[2:] = rng.normal(0.0, 1.0, prim[2:].shape)
    elif kind == "dense_ties":
        # every cell's wavespeed within 1e-7 of the others: far below the
        # FP32 estimate's resolution, so the screen must keep them all
        prim[0] = 1.0
        prim[1] = 1.0
        prim[2] = 0.5 * (1.0 + 1e-7 * rng.uniform(0.0, 1.0, prim[2].shape))
        prim[3] = 0.0
        prim[4] = 0.0
    else:  # wide_range: rho and p over 4 decades, |u| over 4 more (wider contrasts leave the physical states)
        prim[0] = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), prim[0].shape))
        prim[1] = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), prim[1].shape))
        prim[2:] = rng.normal(0.0, 1.0, prim[2:].shape) * np.exp(rng.uniform(np.log(1e-2), np.log(1e2), prim[2:].shape))
    return prim


@pytest.mark.parametrize("kind", ["random", "dense_ties", "wide_range"])
@pytest.mark.parametrize("shape,dx", [((40, 34, 30), (0.02, 0.02, 0.02)), ((41, 34, 30), (0.02, 0.03, 0.025))],
                         ids=["even_n0_tma_cubic", "odd_n0_plain_loads_non_cubic"])
def test_step_dt_is_the_max_wavespeed_of_its_state(cuda, euler, kind, shape, dx):
    """The fused step reduces the next step's CFL wavespeed in the same pass,
    evaluating it in FP64 only for the cells an FP32 estimate cannot rule out.
    After one and three steps the dt it keeps is cfl / max wavespeed of the
    state it wrote, over every cell (ghosts included), within a few ulps of
    numpy's (the step's sound speed is faithful, not correctly rounded); a
    cell wrongly screened out would move it by up to the estimate's 2^-16
    band."""
    gamma, cfl = 1.4, 0.4
    prim0 = _screen_state(kind, shape, seed=sum(shape))
    with euler.Simulation(*shape, gamma, dx, cfl) as sim:
        sim.set_prim(prim0)
        for steps in (1, 2):
            sim.advance(steps)
            prim, _ = sim.state_numpy()
            _, dt, _ = sim.time()
            ref = _max_wavespeed_dt(prim, gamma, dx, cfl)
            assert abs(dt - ref) <= 1e-14 * ref, (kind, steps, dt, ref)
        assert sim.status() == 0


def test_implosion_at_bench_size_symmetry_and_conservation(cuda, euler):
    """The implosion on the bench's 512^3 interior (514^3 with ghosts), 20
    steps: properties that hold at any size, checked at this one.  The state
    is symmetric under every permutation of the axes (each velocity component
    maps to the permuted one) to rounding; and before any wave reaches the
    boundary (the sphere of radius 1/4 is 1/4 from every face; 20 steps reach
    t ~ 0.005) the FP64 totals of mass and energy are conserved to rounding,
    since each face flux is computed once and used by both of its cells."""
    torch = cuda
    nx = 512
    n = nx + 2
    with euler.Simulation(n, n, n, 1.4, (1.0 / nx,) * 3, 0.4) as sim:
        sim.init_implode()
        tot0 = sim.totals()
        sim.advance(20)
        tot = sim.totals()
        assert sim.status() == 0
        t, _, steps = sim.time()
        assert steps == 20 and 0.0 < t < 0.05
        prim = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
        sim.get_state(prim=prim)
    for f in (0, 1):
        assert abs(tot[f] - tot0[f]) <= 1e-12 * abs(tot0[f]), (f, tot[f], tot0[f])
    for f in (2, 3, 4):
        assert abs(tot[f]) <= 1e-12 * abs(tot0[0]), (f, tot[f])
    # dims of a field are (k, j, i); velocity u_a follows its axis
    axes = {0: 2, 1: 1, 2: 0}  # velocity component -> tensor dim of its axis
    for a, b in ((0, 1), (0, 2), (1, 2)):
        da, db = axes[a], axes[b]
        for f in (0, 1):
            x = prim[f]
            scale = x.abs().max()
            assert (x - x.transpose(da, db)).abs().max() <= 1e-12 * scale, (f, a, b)
        ua, ub = prim[2 + a], prim[2 + b]
        scale = max(ua.abs().max(), ub.abs().max())
        assert (ua - ub.transpose(da, db)).abs().max() <= 1e-12 * scale, (a, b)
    del prim
    torch.cuda.empty_cache()
