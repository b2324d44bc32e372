"""GPU tests of the multi-grid batch (eulr_batch_*): every grid of a batch
of uneven grids -- each with its own gamma, mesh and dt -- against the oracle
run on that grid alone; tile-shape independence (the autotuned tiling gives
bit-identical results); and identity with the single-grid simulation."""
import numpy as np
import pytest

from conftest import rel_linf

pytestmark = pytest.mark.gpu


def draw_batch(seed, sizes=(24, 32, 48), ngrids=6):
    """Grids like the batched workload: axis lengths from `sizes`, gamma
    U[1.1, 1.67], inner/outer pressure ratio log-U[0.01, 1], density ratio
    log-U[0.05, 1], step on x+y+z < c with c U[0.1, 0.5]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    grids, ics = [], []
    for _ in range(ngrids):
        n = [int(rng.choice(sizes)) for _ in range(3)]
        gamma = float(rng.uniform(1.1, 1.67))
        pr = float(np.exp(rng.uniform(np.log(0.01), 0.0)))
        rr = float(np.exp(rng.uniform(np.log(0.05), 0.0)))
        c = float(rng.uniform(0.1, 0.5))
        grids.append((n[0] + 2, n[1] + 2, n[2] + 2, gamma, 1.0 / n[0], 1.0 / n[1], 1.0 / n[2]))
        ics.append((c, rr, pr))
    return grids, ics


def oracle_grid(O, grid, ic, steps, cfl=0.4):
    n0, n1, n2, gamma, dx0, dx1, dx2 = grid
    c, rr, pr = ic
    prim = O.init_step(n0, n1, n2, (dx0, dx1, dx2), c, rr, pr, 1.0, 1.0)
    cons = O.prim_to_cons(prim, gamma)
    t = O.simulate(prim, cons, gamma, (dx0, dx1, dx2), cfl, steps)
    return prim, cons, t


def test_batch_grids_match_oracle(cuda, euler, oracle_lib):
    grids, ics = draw_batch(5)
    steps = 12
    with euler.Batch(grids, cfl=0.4) as b:
        for g, (c, rr, pr) in enumerate(ics):
            b.init_step(g, c, rr, pr)
        b.advance(steps)
        assert b.status() == 0
        for g in range(len(grids)):
            prim, cons = b.state_numpy(g)
            pref, cref, tref = oracle_grid(oracle_lib, grids[g], ics[g], steps)
            t, _, st = b.time(g)
            assert st == steps
            assert abs(t - tref) <= 1e-12 * tref, g
            errs = rel_linf(cons, cref) + rel_linf(prim, pref)
            assert max(errs) <= 1e-11, (g, errs)


def test_autotuned_tiling_is_bit_identical(cuda, euler):
    grids, ics = draw_batch(9, sizes=(24, 48, 32), ngrids=5)
    out = []
    for tune in (False, True):
        with euler.Batch(grids, cfl=0.4) as b:
            for g, (c, rr, pr) in enumerate(ics):
                b.init_step(g, c, rr, pr)
            if tune:
                choice = b.autotune(trial_steps=1)
                assert choice["kchunk"] in (8, 16, 32, 64)
                assert choice["tile"] in ((32, 8), (16, 8), (16, 16))
            b.advance(7)
            out.append([b.state_numpy(g) for g in range(len(grids))])
    for g in range(len(grids)):
        assert np.array_equal(out[0][g][0], out[1][g][0]) and np.array_equal(out[0][g][1], out[1][g][1])


def test_batch_equals_single_grid_simulation(cuda, euler):
    grid = (34, 26, 50, 1.3, 1 / 32, 1 / 24, 1 / 48)
    with euler.Batch([grid, (26, 26, 26, 1.5, 1 / 24, 1 / 24, 1 / 24)], cfl=0.4) as b:
        b.init_step(0, 0.3, 0.2, 0.05)
        b.init_step(1, 0.4, 0.5, 0.5)
        b.advance(9)
        pb, cb = b.state_numpy(0)
        tb = b.time(0)
    import oracle as O

    prim0 = O.init_step(34, 26, 50, grid[4:], 0.3, 0.2, 0.05, 1.0, 1.0)
    with euler.Simulation(34, 26, 50, 1.3, grid[4:], 0.4) as s:
        s.set_prim(prim0)
        s.advance(9)
        ps, cs = s.state_numpy()
        ts = s.time()
    assert np.array_equal(pb, ps) and np.array_equal(cb, cs)
    assert tb[0] == ts[0]


def test_batch_fp32c_tracks_fp64(cuda, euler):
    grids, ics = draw_batch(3, sizes=(32, 48), ngrids=4)
    res = {}
    for precision in ("f64", "f32c"):
        with euler.Batch(grids, cfl=0.4, precision=precision) as b:
            for g, (c, rr, pr) in enumerate(ics):
                b.init_step(g, c, rr, pr)
            b.advance(20)
            assert b.status() == 0
            res[precision] = [b.state_numpy(g)[1][0] for g in range(len(grids))]
    for g in range(len(grids)):
        a, ref = res["f32c"][g][1:-1, 1:-1, 1:-1], res["f64"][g][1:-1, 1:-1, 1:-1]
        assert np.abs(a - ref).sum() / np.abs(ref).sum() < 1e-6


def test_batch_rejects_bad_input(cuda, euler):
    with pytest.raises(euler.EulerError):
        euler.Batch([(10, 10, 10, 0.9, 0.1, 0.1, 0.1)])
    with euler.Batch([(10, 10, 10, 1.4, 0.1, 0.1, 0.1)]) as b:
        with pytest.raises(euler.EulerError):
            b.advance(1)  # nothing loaded
        with pytest.raises(euler.EulerError):
            b.init_step(3, 0.2, 1, 1)  # grid index out of range


@pytest.mark.parametrize("precision", ["f32c", "f32"])
def test_fp32_batch_equals_single_grid_simulation(cuda, euler, precision):
    """The FP32 batch's default 32x8 shape runs the same column engine as a
    single FP32 simulation: bit-identical states, for cubic cells (exact
    six-term sum) and for uneven spacings (per-term compensated sum)."""
    import oracle as O

    for grid in [(34, 26, 50, 1.3, 1 / 32, 1 / 32, 1 / 32), (34, 26, 50, 1.3, 1 / 32, 1 / 24, 1 / 48)]:
        with euler.Batch([grid, (26, 26, 26, 1.5, 1 / 24, 1 / 24, 1 / 24)], cfl=0.4, precision=precision) as b:
            b.init_step(0, 0.3, 0.2, 0.05)
            b.init_step(1, 0.4, 0.5, 0.5)
            b.advance(9)
            pb, cb = b.state_numpy(0)
        prim0 = O.init_step(34, 26, 50, grid[4:], 0.3, 0.2, 0.05, 1.0, 1.0)
        with euler.Simulation(34, 26, 50, 1.3, grid[4:], 0.4, precision=precision) as s:
            s.set_prim(prim0)
            s.advance(9)
            ps, cs = s.state_numpy()
        assert np.array_equal(pb, ps) and np.array_equal(cb, cs)


@pytest.mark.parametrize("precision", ["f64", "f32c"])
def test_batch_with_grids_without_interior(cuda, euler, oracle_lib, precision):
    """Grids with no interior cell have no work item: the step launch's last
    CTA finalizes them (dt of their state, clock), as a finalize kernel did.
    Their clock matches the oracle's loop on that grid; the other grids are
    unaffected (FP64 against the oracle, FP32c against the FP64 batch)."""
    grids, ics = draw_batch(17, ngrids=3)
    grids.insert(1, (3, 3, 2, 1.3, 0.5, 0.5, 0.5))
    ics.insert(1, (0.3, 0.5, 0.2))
    grids.append((2, 5, 4, 1.5, 0.25, 0.2, 0.25))
    ics.append((0.6, 0.3, 0.4))
    steps = 7
    with euler.Batch(grids, cfl=0.4, precision=precision) as b:
        for g, (c, rr, pr) in enumerate(ics):
            b.init_step(g, c, rr, pr)
        b.advance(steps)
        assert b.status() == 0
        for g in range(len(grids)):
            _, cref_state, tref = oracle_grid(oracle_lib, grids[g], ics[g], steps)
            t, _, st = b.time(g)
            assert st == steps
            tol = 1e-12 if precision == "f64" else 1e-5
            assert abs(t - tref) <= tol * tref, (g, t, tref)
            if precision == "f64":
                _, cons = b.state_numpy(g)
                assert max(rel_linf(cons, cref_state)) <= 1e-11, g


def test_batch_reload_after_even_steps(cuda, euler, oracle_lib):
    """A grid loaded again after an even number of steps restarts from its new
    state while the others run on: its ghost layer is set again (copy 1 at
    load, copy 0 after its next step) and its clock starts from zero."""
    grids, ics = draw_batch(23, ngrids=4)
    with euler.Batch(grids, cfl=0.4) as b:
        for g, (c, rr, pr) in enumerate(ics):
            b.init_step(g, c, rr, pr)
        b.advance(4)
        c, rr, pr = ics[2]
        b.init_step(2, c, rr, pr)
        b.advance(6)
        for g in range(len(grids)):
            steps = 6 if g == 2 else 10
            pref, cref, tref = oracle_grid(oracle_lib, grids[g], ics[g], steps)
            t, _, st = b.time(g)
            assert st == steps, g
            assert abs(t - tref) <= 1e-12 * tref, g
            prim, cons = b.state_numpy(g)
            assert max(rel_linf(cons, cref) + rel_linf(prim, pref)) <= 1e-11, g


def test_one_launch_per_step(cuda, euler):
    n = 20
    with euler.Simulation(n, n, n, precision="f64") as sim:
        assert sim.launches_per_step() == 1
        sim.init_implode()
        ms = sim.profile_step()
        assert ms[1] > 0.0
