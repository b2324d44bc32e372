"""The argument the bit-identical godunov (csrc/godunov_exact.cu) rests on,
checked on the host: the reference (euler_operators/godunov.hpp:32-91)
solves every interior face twice, once from each of its cells, but both
solves are the same function of the same two cells, and so is each cell's
sound speed and total energy.  Solving each face once, computing each cell's
quantities once, and summing each cell's three axes from zero in the
reference's order (x, y, z) must therefore give the reference's bits.

Here that algorithm is written in numpy (IEEE double or single, every
operation rounded separately, no FMA) and compared with the oracle, which is
pinned bit for bit to the reference build: equal arrays, on random states
with supersonic faces, ragged grids and both precisions."""
import numpy as np
import pytest


def _kmin(a, b):  # Kokkos::min: the first argument unless the second is smaller
    return np.where(b < a, b, a)


def _kmax(a, b):  # Kokkos::max: the first argument unless the second is larger
    return np.where(a < b, b, a)


def _hllc(dL, pL, uL, cL, eL, dR, pR, uR, cR, eR, dirn, T):
    """hllc::operator() (hllc.hpp:50-105) on arrays of faces; uL/uR are the
    three velocity components, eL/eR the cells' total energies.  The flux
    comes back in the global field order (d, e, m0, m1, m2)."""
    unL, unR = uL[dirn], uR[dirn]
    cmax = _kmax(cL, cR)
    SL = _kmin(unL, unR) - cmax
    SR = _kmax(unL, unR) + cmax
    rcL = dL * (SL - unL)
    rcR = dR * (SR - unR)
    ustar = (((pR - pL) + rcL * unL) - rcR * unR) / (rcL - rcR)
    pstar = T(0.5) * (((pL + pR) + rcL * (ustar - unL)) + rcR * (ustar - unR))
    left = ustar > 0
    S = np.where(left, SL, SR)
    d = np.where(left, dL, dR)
    p = np.where(left, pL, pR)
    un = np.where(left, unL, unR)
    etot = np.where(left, eL, eR)
    u = [np.where(left, uL[a], uR[a]) for a in range(3)]
    sup = (SL * SR) > 0
    un_o = np.where(sup, un, ustar)
    ptot_o = np.where(sup, p, pstar)
    ratio = (S - un) / (S - un_o)
    d_o = ratio * d
    etot_o = ratio * etot + (ptot_o * un_o - p * un) / (S - ustar)
    m = d_o * un_o
    flux = [m, (etot_o + ptot_o) * un_o, None, None, None]
    for a in range(3):
        flux[2 + a] = (m * un_o + ptot_o) if a == dirn else m * u[a]
    return flux


def godunov_faces_once(prim, cons, gamma, dx, dt):
    """cons after godunov, each face solved once (arrays are [k, j, i])."""
    T = prim.dtype.type
    gamma = T(gamma)
    gm1 = gamma - T(1)
    dx0, dx1, dx2 = (T(v) for v in dx)
    ds = (dx1 * dx2, dx2 * dx0, dx0 * dx1)
    dtodv = T(dt) / ((dx0 * dx1) * dx2)
    d, p = prim[0], prim[1]
    u = [prim[2], prim[3], prim[4]]
    c = np.sqrt((gamma * p) / d)
    e = p / gm1 + (d * ((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2])) / T(2)
    n2, n1, n0 = d.shape
    inner = (slice(1, n2 - 1), slice(1, n1 - 1), slice(1, n0 - 1))
    total = [np.zeros(d[inner].shape, dtype=d.dtype) for _ in range(5)]
    for a in range(3):
        # faces between cell c and c+1 along axis a (array axis 2 - a), each solved once
        ax = 2 - a
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, d.shape[ax] - 1)
        hi[ax] = slice(1, d.shape[ax])
        lo, hi = tuple(lo), tuple(hi)
        F = _hllc(d[lo], p[lo], [v[lo] for v in u], c[lo], e[lo], d[hi], p[hi], [v[hi] for v in u], c[hi], e[hi],
                  a, T)
        # the interior cell's left face is face index i-1, its right face index i
        left = [inner[0], inner[1], inner[2]]
        right = [inner[0], inner[1], inner[2]]
        left[ax] = slice(0, d.shape[ax] - 2)
        right[ax] = slice(1, d.shape[ax] - 1)
        for f in range(5):
            total[f] = total[f] + ds[a] * (F[f][tuple(right)] - F[f][tuple(left)])
    out = cons.copy()
    for f in range(5):
        out[f][inner] = cons[f][inner] - dtodv * total[f]
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape,dx", [((20, 12, 10), (0.05, 0.083, 0.1)), ((9, 17, 6), (0.1, 0.1, 0.1)),
                                      ((3, 3, 3), (1.0, 1.0, 1.0))])
def test_faces_once_equals_reference_bits(oracle_lib, dtype, shape, dx):
    O = oracle_lib
    prim = O.random_prim(*shape, seed=sum(shape) + 3).astype(dtype)
    # a few supersonic cells, so both branches of the flux are exercised
    rng = np.random.default_rng(1)
    fast = rng.random(prim[2].shape) < 0.15
    prim[2] = np.where(fast, prim[2] * dtype(6), prim[2])
    cons = O.prim_to_cons(prim, 1.4)
    dt = 0.4 * O.time_step(prim, 1.4, dx)
    ref = O.godunov(prim, cons, 1.4, dx, dt)
    with np.errstate(all="ignore"):
        got = godunov_faces_once(prim, cons, 1.4, dx, dt)
    assert got.dtype == ref.dtype
    assert np.array_equal(got, ref)
