"""The screened exact max wavespeed of time_step, the state load and the
fused FP64 step (csrc/step_common.cuh: WaveScreen), emulated on the host with IEEE float32
arithmetic: the FP32 estimate built from the doubles' high words stays within
its stated error bound, and the warp scan (running max of the estimates'
bit patterns, exact evaluation within 128 FP32 ulps of it, out-of-range cells
always exact) never misses the cell that holds the exact max -- on random
states, on states whose wavespeeds are a few ulps apart everywhere, and on
values spread over +-40 decades.  The GPU tests check the kernels themselves
against the oracle; this pins the argument they rest on."""
import numpy as np

GAMMA = 1.4
BAND = 128  # FP32 ulps, as in WaveScreen::exact_needed
BOUND = 2.0 ** -20 + 5 * 2.0 ** -24  # first-order relative error of the estimate


def high_word_float(x):
    """The device's high_word_float: mantissa truncated to 20 bits, 0 below
    FP32's normal range, infinity above it (and for NaN)."""
    hi = (x.view(np.uint64) >> np.uint64(32)).astype(np.int64)
    e = ((hi >> 20) & 0x7FF) - (1023 - 127)
    mag = np.where(e <= 0, 0, np.where(e >= 255, 0x7F800000, (np.clip(e, 0, 254) << 23) | ((hi & 0xFFFFF) << 3)))
    return ((hi & 0x80000000) | mag).astype(np.uint32).view(np.float32)


def exact_invdt(d, p, u, ix):
    c = np.sqrt(GAMMA * p / d)
    return ((c + np.abs(u[0])) * ix[0] + (c + np.abs(u[1])) * ix[1]) + (c + np.abs(u[2])) * ix[2]


def screen(d, p, u, ix):
    f = np.float32
    d32, p32 = high_word_float(d), high_word_float(p)
    x32 = (f(GAMMA) * p32) / d32
    c32 = np.sqrt(x32)
    v32 = ((c32 + np.abs(high_word_float(u[0]))) * f(ix[0]) + (c32 + np.abs(high_word_float(u[1]))) * f(ix[1])
           + (c32 + np.abs(high_word_float(u[2]))) * f(ix[2]))
    inr = lambda x: (x >= f(1e-30)) & (x <= f(1e30))  # noqa: E731
    sure = inr(d32) & inr(p32) & inr(x32) & (v32 <= f(1e30))
    return sure, v32, np.where(sure, v32.view(np.uint32), np.uint32(0)).astype(np.int64)


def warp_scan(sure, key):
    """One warp's scan: 32 lanes per iteration, running max of the keys."""
    run = 0
    evaluated = np.zeros(key.size, bool)
    for it in range(key.size // 32):
        sl = slice(32 * it, 32 * it + 32)
        run = max(run, int(key[sl].max()))
        evaluated[sl] = (~sure[sl]) | (key[sl] + BAND >= run)
    return evaluated


def cases(rng, n):
    d = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))
    p = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))
    u = rng.normal(0.0, 1.0, (3, n))
    yield "random", d, p, u
    ties = np.ones(n)
    yield ("near_ties", ties * (1 + rng.integers(-8, 9, n) * 2.0 ** -52), ties * (1 + rng.integers(-8, 9, n) * 2.0 ** -52),
           np.full((3, n), 0.3))
    yield ("wide_range", d * 10.0 ** rng.uniform(-40, 40, n), p * 10.0 ** rng.uniform(-40, 40, n),
           u * 10.0 ** rng.uniform(-20, 20, (3, n)))
    # estimates in the wrong order: most cells have p = 1 + 2^-20 and u = 0.25
    # (exact in 20 mantissa bits); a few have p 2^-45 lower (truncated to 1)
    # and u0 2^-30 higher (lost in truncation) -- the larger exact wavespeed
    # behind an estimate about 4 FP32 ulps lower
    pm = np.full(n, 1.0 + 2.0 ** -20)
    um = np.full((3, n), 0.25)
    planted = rng.choice(n, 8, replace=False)
    pm[planted] -= 2.0 ** -45
    um[0, planted] += 2.0 ** -30
    yield "misordered", np.ones(n), pm, um


def test_screen_error_bound_and_no_missed_max():
    rng = np.random.default_rng(2024)
    worst = 0.0
    with np.errstate(all="ignore"):
        for trial in range(60):
            ix = (64.0, 64.0, 64.0) if trial % 2 else (64.0, 57.0, 71.0)
            for name, d, p, u in cases(rng, 32 * 64):
                v = exact_invdt(d, p, u, ix)
                sure, v32, key = screen(d, p, u, ix)
                if sure.any():
                    rel = np.abs(v32[sure].astype(np.float64) / v[sure] - 1.0)
                    worst = max(worst, float(rel.max()))
                evaluated = warp_scan(sure, key)
                finite = np.isfinite(v)
                m = v[finite].max()
                assert (evaluated & (v == m)).any(), (name, trial)
    assert worst <= BOUND, worst


def test_screen_evaluates_few_cells_on_random_states():
    """On the bench's random-state distribution the exact FP64 wavespeed is
    taken for a fraction of a percent of the cells."""
    rng = np.random.default_rng(7)
    n = 32 * 440  # one warp's cells at 514^3 with 8 CTAs of 256 threads per SM
    _, d, p, u = next(cases(rng, n))
    sure, _, key = screen(d, p, u, (512.0, 512.0, 512.0))
    assert sure.all()
    assert warp_scan(sure, key).mean() < 0.005


STEP_BOUND = 2.0 ** -20 + 6 * 2.0 ** -24  # WaveScreen::step_exact_needed


def step_screen(cs, u, ix, cubic):
    """WaveScreen::step_exact_needed: the estimate from the step's own sound
    speed and velocities (separately rounded FP32; the device may contract a
    product and a sum into one FMA, which only removes a rounding)."""
    f = np.float32
    c32 = high_word_float(cs)
    a = [np.abs(high_word_float(u[k])) for k in range(3)]
    if cubic:
        v32 = (((f(3.0) * c32 + a[0]) + a[1]) + a[2]) * f(ix[0])
    else:
        v32 = ((c32 + a[0]) * f(ix[0]) + (c32 + a[1]) * f(ix[1])) + (c32 + a[2]) * f(ix[2])
    inr = (c32 >= f(1e-30)) & (c32 <= f(1e30))
    sure = inr & (v32 <= f(1e30))
    return sure, v32, np.where(sure, v32.view(np.uint32), np.uint32(0)).astype(np.int64)


def step_exact(cs, u, ix, cubic):
    if cubic:
        return (3.0 * cs + np.abs(u[0]) + np.abs(u[1]) + np.abs(u[2])) * ix[0]
    return (cs + np.abs(u[0])) * ix[0] + (cs + np.abs(u[1])) * ix[1] + (cs + np.abs(u[2])) * ix[2]


def step_cases(rng, n):
    for name, d, p, u in cases(rng, n):
        yield name, np.sqrt(GAMMA * p / d), u  # the step's sound speed, to within an ulp
    # estimates in the wrong order for this form: most cells have
    # c = 1 + 2^-20 (exact in 20 mantissa bits) and u = 0.25; a few have c
    # 2^-45 lower (truncated a whole 2^-20 lower) and u0 2^-30 higher (lost in
    # truncation) -- the larger exact wavespeed behind an estimate about 12
    # FP32 ulps lower
    cm = np.full(n, 1.0 + 2.0 ** -20)
    um = np.full((3, n), 0.25)
    planted = rng.choice(n, 8, replace=False)
    cm[planted] -= 2.0 ** -45
    um[0, planted] += 2.0 ** -30
    yield "misordered", cm, um


def test_step_screen_error_bound_and_no_missed_max():
    """The fused step's form of the screen: within its bound, and the warp
    scan keeps the cell holding the exact max, on the same state families
    and on one whose estimates are misordered."""
    rng = np.random.default_rng(99)
    worst = 0.0
    with np.errstate(all="ignore"):
        for trial in range(60):
            cubic = trial % 2 == 1
            ix = (64.0, 64.0, 64.0) if cubic else (64.0, 57.0, 71.0)
            for name, cs, u in step_cases(rng, 32 * 64):
                v = step_exact(cs, u, ix, cubic)
                sure, v32, key = step_screen(cs, u, ix, cubic)
                if sure.any():
                    rel = np.abs(v32[sure].astype(np.float64) / v[sure] - 1.0)
                    worst = max(worst, float(rel.max()))
                evaluated = warp_scan(sure, key)
                finite = np.isfinite(v)
                m = v[finite].max()
                assert (evaluated & (v == m)).any(), (name, trial)
    assert worst <= STEP_BOUND, worst
