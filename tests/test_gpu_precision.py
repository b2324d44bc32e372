"""GPU tests of the FP32 simulation states against the FP64 oracle.

EULR_PRECISION_F32C: FP32 state, compensated update (the three axis flux
differences times dt/dv ds, added to the cell by TwoProduct and TwoSum with
their rounding errors folded back: one rounding at the state's scale), FP64
internal energy for low-pressure cells.  EULR_PRECISION_F32C_HILO: the same with a stored FP32
low word.  EULR_PRECISION_F32: plain FP32 (the reference's real_t = float),
compared with the reference's own float loop as well.

Errors are relative: L1 = sum|a-b| / sum|ref|, Linf = max|a-b| / max|ref|,
over interior cells."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_errors(a, b):
    a = a[1:-1, 1:-1, 1:-1].astype(np.float64)
    b = b[1:-1, 1:-1, 1:-1].astype(np.float64)
    d = np.abs(a - b)
    return d.sum() / np.abs(b).sum(), d.max() / np.abs(b).max()


def implode_oracle(O, nx, steps, dtype=np.float64):
    n = nx + 2
    dx = (1.0 / nx,) * 3
    prim = O.init_implode(n, n, n, dx, dtype=dtype)
    cons = O.prim_to_cons(prim, 1.4)
    t = O.simulate(prim, cons, 1.4, dx, 0.4, steps)
    return prim, cons, t


def run_sim(euler, precision, nx, steps):
    n = nx + 2
    with euler.Simulation(n, n, n, 1.4, (1.0 / nx,) * 3, 0.4, precision=precision) as sim:
        sim.init_implode()
        sim.advance(steps)
        prim, cons = sim.state_numpy()
        t, _, st = sim.time()
        status = sim.status()
    return prim, cons, t, st, status


@pytest.mark.parametrize("precision,tol_l1,tol_linf", [("f32c", 2e-6, 2e-4), ("f32c_hilo", 2e-6, 2e-4),
                                                       ("f32", 1e-5, 1e-3)])
def test_fp32_states_track_fp64_implosion(cuda, euler, oracle_lib, precision, tol_l1, tol_linf):
    prim_ref, cons_ref, t_ref = implode_oracle(oracle_lib, 48, 60)
    prim, cons, t, steps, status = run_sim(euler, precision, 48, 60)
    assert status == 0 and steps == 60
    assert abs(t - t_ref) <= 1e-5 * t_ref
    l1, linf = rel_errors(cons[0], cons_ref[0])
    assert l1 <= tol_l1 and linf <= tol_linf, (precision, l1, linf)
    l1p, _ = rel_errors(prim[1], prim_ref[1])
    assert l1p <= 10 * tol_l1, (precision, l1p)


def test_fp32_plain_tracks_reference_float_loop(cuda, euler, oracle_lib):
    """The plain FP32 state against the reference's real_t = float loop."""
    prim_ref, cons_ref, t_ref = implode_oracle(oracle_lib, 32, 20, dtype=np.float32)
    prim, cons, t, _, status = run_sim(euler, "f32", 32, 20)
    assert status == 0
    assert abs(t - t_ref) <= 1e-5 * t_ref
    for f in range(5):
        scale = max(np.abs(cons_ref[f]).max(), 1e-30)
        assert np.abs(cons[f] - cons_ref[f]).max() <= 1e-5 * max(scale, np.abs(cons_ref[0]).max()), f


def test_compensated_beats_plain_fp32(cuda, euler, oracle_lib):
    """The compensated update is at least as accurate as plain FP32."""
    _, cons_ref, _ = implode_oracle(oracle_lib, 40, 80)
    errs = {}
    for precision in ("f32", "f32c", "f32c_hilo"):
        _, cons, _, _, _ = run_sim(euler, precision, 40, 80)
        errs[precision] = rel_errors(cons[0], cons_ref[0])[0]
    assert errs["f32c"] <= errs["f32"] * 1.05, errs
    assert errs["f32c_hilo"] <= errs["f32c"] * 1.05, errs


def test_fp32_random_state_and_totals(cuda, euler, oracle_lib):
    O = oracle_lib
    n0, n1, n2 = 36, 30, 22
    dx = (1 / 34, 1 / 28, 1 / 20)
    prim0 = O.random_prim(n0, n1, n2, seed=31)
    p = prim0.copy()
    c = O.prim_to_cons(p, 1.4)
    O.simulate(p, c, 1.4, dx, 0.4, 5)
    for precision in ("f32c", "f32c_hilo"):
        with euler.Simulation(n0, n1, n2, 1.4, dx, 0.4, precision=precision) as sim:
            sim.set_prim(prim0)
            sim.advance(5)
            pg, cg = sim.state_numpy()
            tot = sim.totals()
            assert sim.status() == 0
        l1, _ = rel_errors(cg[0], c[0])
        assert l1 < 1e-6, (precision, l1)
        interior = c[:, 1:-1, 1:-1, 1:-1]
        assert abs(tot[0] - interior[0].sum()) <= 1e-6 * abs(interior[0].sum())


def test_state_bytes(cuda, euler):
    n = 18
    expect = {"f64": 2 * 5 * 8, "f32c": 2 * 5 * 4, "f32c_hilo": 2 * 10 * 4, "f32": 2 * 5 * 4}
    for precision, per_cell in expect.items():
        with euler.Simulation(n, n, n, precision=precision) as sim:
            assert sim.state_bytes() == per_cell * 16 ** 3


def test_f32c_implosion_at_bench_size(cuda, euler):
    """The FP32-compensated state on the bench's 512^3 interior, 20 implosion
    steps: axis-permutation symmetry of density, pressure and velocity to FP32
    rounding (1e-5 of the scale), and FP64 totals of mass and energy conserved
    (momentum kept at zero) to 1e-9 before waves reach the boundary: the
    compensated update rounds each cell at state scale, and those roundings
    average out in the sums."""
    torch = cuda
    nx = 512
    n = nx + 2
    with euler.Simulation(n, n, n, 1.4, (1.0 / nx,) * 3, 0.4, precision="f32c") as sim:
        sim.init_implode()
        tot0 = sim.totals()
        sim.advance(20)
        tot = sim.totals()
        assert sim.status() == 0
        prim = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
        sim.get_state(prim=prim)
    for f in (0, 1):
        assert abs(tot[f] - tot0[f]) <= 1e-9 * abs(tot0[f]), (f, tot[f], tot0[f])
    for f in (2, 3, 4):
        assert abs(tot[f]) <= 1e-9 * abs(tot0[0]), (f, tot[f])
    axes = {0: 2, 1: 1, 2: 0}  # velocity component -> tensor dim (k, j, i) of its axis
    for a, b in ((0, 1), (0, 2), (1, 2)):
        da, db = axes[a], axes[b]
        for f in (0, 1):
            x = prim[f]
            assert (x - x.transpose(da, db)).abs().max() <= 1e-5 * x.abs().max(), (f, a, b)
        ua, ub = prim[2 + a], prim[2 + b]
        scale = max(ua.abs().max(), ub.abs().max())
        assert (ua - ub.transpose(da, db)).abs().max() <= 1e-5 * scale, (a, b)
    del prim
    torch.cuda.empty_cache()
