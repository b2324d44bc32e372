"""GPU parity of the per-operator entry points against the oracle.

prim_to_cons, cons_to_prim, time_step and init_implode are bit-identical to
the reference (separately rounded arithmetic in the reference's order).
godunov solves each face once and shares reciprocals, so it matches within
the stated tolerance: 1e-12 relative L-infinity per field (max|a-b|/max|ref|)
for FP64 after one call."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_linf

pytestmark = pytest.mark.gpu

TOL_F64_STEP = 1e-12
TOL_F32_STEP = 2e-5  # float godunov: a few float ulps of the largest flux term

OPS = sorted(glob.glob(os.path.join(GOLDEN, "ops_*.npz")))


def _t(cuda, a):
    return cuda.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("path", OPS, ids=os.path.basename)
def test_golden_operators(cuda, euler, path):
    z = np.load(path)
    prim = z["prim"]
    g = float(z["gamma"])
    dx = tuple(float(v) for v in z["dx"])
    cfl = float(z["cfl"])
    pg = _t(cuda, prim)
    cg = euler.prim_to_cons(pg, g)
    assert np.array_equal(cg.cpu().numpy(), z["cons"])
    assert np.array_equal(euler.cons_to_prim(cg, g).cpu().numpy(), z["prim_rt"])
    dt = euler.time_step(pg, g, dx)
    assert dt.item() == z["dt"][()]
    euler.godunov(pg, cg, g, dx, cfl * z["dt"][()])
    got = cg.cpu().numpy()
    ref = z["cons_godunov"]
    tol = TOL_F64_STEP if prim.dtype == np.float64 else TOL_F32_STEP
    errs = rel_linf(got, ref)
    assert max(errs) <= tol, errs
    # ghosts are never touched
    n2, n1, n0 = prim.shape[1:]
    mask = np.ones((n2, n1, n0), bool)
    if min(n0, n1, n2) >= 3:
        mask[1:-1, 1:-1, 1:-1] = False
    assert np.array_equal(got[:, mask], z["cons"][:, mask])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_init_implode_bit_exact(cuda, euler, oracle_lib, dtype):
    npdt = np.float64 if dtype == "f64" else np.float32
    tdt = cuda.float64 if dtype == "f64" else cuda.float32
    for n0, n1, n2 in ((18, 18, 18), (66, 34, 20), (7, 5, 3)):
        dx = (1.0 / (n0 - 2), 1.0 / 17, 0.05)
        ref = oracle_lib.init_implode(n0, n1, n2, dx, dtype=npdt)
        got = euler.init_implode(n0, n1, n2, dx, dtype=tdt).cpu().numpy()
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("shape", [(70, 40, 37), (34, 10, 130), (3, 3, 3), (5, 130, 4), (1, 1, 1), (2, 9, 9)])
def test_random_operators_vs_oracle(cuda, euler, oracle_lib, shape):
    O = oracle_lib
    n0, n1, n2 = shape
    prim = O.random_prim(n0, n1, n2, seed=sum(shape))
    dx = (0.02, 0.03, 0.05)
    g = 1.4
    cons = O.prim_to_cons(prim, g)
    dt = O.time_step(prim, g, dx)
    ref = O.godunov(prim, cons, g, dx, 0.4 * dt)
    pg = _t(cuda, prim)
    cg = euler.prim_to_cons(pg, g)
    assert np.array_equal(cg.cpu().numpy(), cons)
    assert euler.time_step(pg, g, dx).item() == dt
    euler.godunov(pg, cg, g, dx, 0.4 * dt)
    errs = rel_linf(cg.cpu().numpy(), ref)
    assert max(errs) <= TOL_F64_STEP, errs


@pytest.mark.parametrize("shape", [(514, 20, 12), (515, 18, 10)], ids=["bench_pitch_514", "pitch_515"])
def test_operators_at_bench_row_pitch(cuda, euler, oracle_lib, shape):
    """The per-operator path at the benchmark's row length (514 cells per row,
    dx = 1/512; and 515): prim_to_cons and time_step bit for bit, godunov to
    1e-12 and its bit-identical variant bit for bit, against the oracle."""
    O = oracle_lib
    prim = O.random_prim(*shape, seed=515)
    dx = (1 / 512,) * 3
    g = 1.4
    cons = O.prim_to_cons(prim, g)
    dt = O.time_step(prim, g, dx)
    ref = O.godunov(prim, cons, g, dx, 0.4 * dt)
    pg = _t(cuda, prim)
    cg = euler.prim_to_cons(pg, g)
    assert np.array_equal(cg.cpu().numpy(), cons)
    assert euler.time_step(pg, g, dx).item() == dt
    ce = cg.clone()
    euler.godunov(pg, cg, g, dx, 0.4 * dt)
    errs = rel_linf(cg.cpu().numpy(), ref)
    assert max(errs) <= TOL_F64_STEP, errs
    euler.godunov(pg, ce, g, dx, 0.4 * dt, exact=True)
    assert np.array_equal(ce.cpu().numpy(), ref)
    assert np.array_equal(euler.cons_to_prim(cg, g).cpu().numpy(), O.cons_to_prim(cg.cpu().numpy(), g))


@pytest.mark.parametrize("path", OPS, ids=os.path.basename)
def test_exact_godunov_matches_reference_fixtures(cuda, euler, path):
    """The exact godunov against the fixtures made by the reference build
    itself: every bit, f64 and f32, interior updated, ghosts untouched.  The
    scalars are passed as the fixture generator passed them (gamma 1.4, its
    CFL 0.4 times the fixture's dt)."""
    z = np.load(path)
    dx = tuple(float(v) for v in z["dx"])
    cg = _t(cuda, z["cons"])
    euler.godunov(_t(cuda, z["prim"]), cg, 1.4, dx, 0.4 * float(z["dt"][()]), exact=True)
    assert np.array_equal(cg.cpu().numpy(), z["cons_godunov"])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("shape,dx", [((70, 40, 37), (0.02, 0.03, 0.05)), ((33, 34, 35), (0.1, 0.1, 0.1)),
                                      ((3, 3, 3), (1.0, 1.0, 1.0)), ((2, 9, 9), (0.5, 0.25, 0.125)),
                                      ((19, 3, 130), (0.05, 0.5, 0.01)), ((3, 27, 12), (0.3, 0.02, 0.1))])
def test_exact_godunov_bit_identical_to_oracle(cuda, euler, oracle_lib, dtype, shape, dx):
    """The exact godunov equals the oracle's, itself bit-identical to the
    reference build, on seeded random states (including supersonic faces),
    ragged, tiny and degenerate grids: partial 16 x 8 tiles in i and j, one
    row or one column of cells, and interiors split into several plane
    chunks."""
    O = oracle_lib
    prim = O.random_prim(*shape, seed=sum(shape))
    if dtype == "f32":
        prim = prim.astype(np.float32)
    cons = O.prim_to_cons(prim, 1.4)
    dt = 0.4 * O.time_step(prim, 1.4, dx)
    ref = O.godunov(prim, cons, 1.4, dx, dt)
    cg = _t(cuda, cons)
    euler.godunov(_t(cuda, prim), cg, 1.4, dx, dt, exact=True)
    assert np.array_equal(cg.cpu().numpy(), ref)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("init", ["implode", "random"])
def test_reference_loop_bit_identical(cuda, euler, oracle_lib, dtype, init):
    """The reference's time loop (simulations/euler_simulation.cpp:56-68:
    time_step -> godunov(cfl*dt) -> cons_to_prim, with cfl*dt formed in T) run
    on the GPU through the bit-identical operators -- time_step, the exact
    godunov, cons_to_prim -- equals the oracle's loop bit for bit after 20
    steps."""
    O = oracle_lib
    npdt = np.float64 if dtype == "f64" else np.float32
    n0, n1, n2 = 26, 22, 18
    dx = (1.0 / (n0 - 2), 1.0 / (n1 - 2), 1.0 / (n2 - 2))
    if init == "implode":
        prim = O.init_implode(n0, n1, n2, dx, dtype=npdt)
    else:
        prim = O.random_prim(n0, n1, n2, seed=12).astype(npdt)
    cons = O.prim_to_cons(prim, 1.4)
    p_ref, c_ref = prim.copy(), cons.copy()
    O.simulate(p_ref, c_ref, 1.4, dx, 0.4, 20)
    pg = _t(cuda, prim)
    cg = euler.prim_to_cons(pg, 1.4)
    for _ in range(20):
        dt = euler.time_step(pg, 1.4, dx).item()
        euler.godunov(pg, cg, 1.4, dx, float(npdt(0.4) * npdt(dt)), exact=True)
        euler.cons_to_prim(cg, 1.4, out=pg)
    assert np.array_equal(cg.cpu().numpy(), c_ref)
    assert np.array_equal(pg.cpu().numpy(), p_ref)


def test_godunov_device_dt_matches_host_dt(cuda, euler, oracle_lib):
    O = oracle_lib
    prim = O.random_prim(40, 33, 20, seed=4)
    g, dx, cfl = 1.4, (0.1, 0.1, 0.1), 0.4
    pg = _t(cuda, prim)
    c1 = euler.prim_to_cons(pg, g)
    c2 = c1.clone()
    dt = euler.time_step(pg, g, dx)
    euler.godunov(pg, c1, g, dx, (dt, cfl))
    euler.godunov(pg, c2, g, dx, cfl * dt.item())
    assert cuda.equal(c1, c2)


def test_uniform_state_steady(cuda, euler):
    for path in sorted(glob.glob(os.path.join(GOLDEN, "uniform_*.npz"))):
        z = np.load(path)
        pg = _t(cuda, z["prim"])
        cg = _t(cuda, z["cons"])
        euler.godunov(pg, cg, float(z["gamma"]), tuple(float(v) for v in z["dx"]), float(z["dt_godunov"]))
        assert np.array_equal(cg.cpu().numpy(), z["cons_godunov"])


def test_time_step_edge_values(cuda, euler, oracle_lib):
    """NaN cells are skipped, as the reference's Kokkos::min skips them."""
    O = oracle_lib
    prim = O.random_prim(9, 8, 7, seed=1)
    prim[1, 3, 3, 3] = np.nan
    dx = (0.1, 0.2, 0.3)
    ref = O.time_step(prim, 1.4, dx)
    got = euler.time_step(_t(cuda, prim), 1.4, dx).item()
    assert got == ref


@pytest.mark.parametrize("case", ["near_ties", "misordered", "wide_range", "large_random"])
def test_time_step_screened_max_is_exact(cuda, euler, oracle_lib, case):
    """time_step and a simulation's first dt evaluate the exact wavespeed
    only where an FP32 estimate says it can be the max; dt stays the
    reference's bit for bit on states built against that screen: wavespeeds
    a few ulps apart everywhere, cells whose estimates order them wrongly,
    values far outside FP32's range (always evaluated exactly), and a large
    grid."""
    O = oracle_lib
    rng = np.random.default_rng(31)
    if case == "near_ties":
        shape = (40, 37, 33)
        prim = np.empty((5,) + shape[::-1])
        prim[0] = 1.0 + rng.integers(-8, 9, prim.shape[1:]) * 2.0 ** -52
        prim[1] = 1.0 + rng.integers(-8, 9, prim.shape[1:]) * 2.0 ** -52
        prim[2:] = 0.3
    elif case == "misordered":
        # the larger exact wavespeed behind the lower FP32 estimate: p 2^-45
        # lower (truncated away) and u0 2^-30 higher (also truncated away)
        shape = (40, 37, 33)
        prim = np.empty((5,) + shape[::-1])
        prim[0] = 1.0
        prim[1] = 1.0 + 2.0 ** -20
        prim[2:] = 0.25
        planted = rng.choice(prim[0].size, 16, replace=False)
        prim[1].reshape(-1)[planted] -= 2.0 ** -45
        prim[2].reshape(-1)[planted] += 2.0 ** -30
    elif case == "wide_range":
        shape = (31, 29, 27)
        prim = O.random_prim(*shape, seed=5)
        prim[0] *= 10.0 ** rng.uniform(-40, 40, prim.shape[1:])
        prim[1] *= 10.0 ** rng.uniform(-40, 40, prim.shape[1:])
        prim[2:] *= 10.0 ** rng.uniform(-20, 20, prim.shape[1:])
    else:
        shape = (130, 130, 130)
        prim = O.random_prim(*shape, seed=6)
    g, dx = 1.4, (0.01, 0.01, 0.01)
    ref = O.time_step(prim, g, dx)
    assert euler.time_step(_t(cuda, prim), g, dx).item() == ref
    host = cuda.from_numpy(prim).pin_memory()
    with euler.Simulation(*shape, g, dx, 0.4) as sim:
        sim.set_prim(host)
        assert sim.time()[1] == 0.4 * ref


def test_canary_guard_bands(cuda, euler, oracle_lib):
    """Every kernel writes only inside its arrays: fields are carved out of
    one buffer with canary gaps that must survive a full operator round."""
    O = oracle_lib
    n0, n1, n2 = 21, 13, 11
    n = n0 * n1 * n2
    gap = 64
    prim = O.random_prim(n0, n1, n2, seed=8)
    buf = cuda.full((10 * (n + gap) + gap,), 12345.0, dtype=cuda.float64, device="cuda")

    def field(i):
        off = gap + i * (n + gap)
        return buf[off:off + n]

    import euler_gb300 as E

    pb = E.Bundle5(*[field(i).data_ptr() for i in range(5)])
    cb = E.Bundle5(*[field(5 + i).data_ptr() for i in range(5)])
    for i in range(5):
        field(i).copy_(cuda.from_numpy(prim[i].ravel()))
    lib = E.load()
    s = cuda.cuda.current_stream().cuda_stream
    import ctypes

    E.check(lib.eulr_prim_to_cons_f64(pb, cb, n0, n1, n2, 1.4, ctypes.c_void_p(s)))
    E.check(lib.eulr_godunov_f64(pb, cb, n0, n1, n2, 1.4, 0.1, 0.1, 0.1, 1e-3, ctypes.c_void_p(s)))
    E.check(lib.eulr_cons_to_prim_f64(cb, pb, n0, n1, n2, 1.4, ctypes.c_void_p(s)))
    cuda.cuda.synchronize()
    for i in range(11):
        off = i * (n + gap)
        assert bool((buf[off:off + gap] == 12345.0).all()), f"canary {i} overwritten"
