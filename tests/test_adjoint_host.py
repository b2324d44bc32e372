"""CPU checks of the adjoint's building blocks (no GPU).

* The host tangent-linear model (oracle/euler_tlm.c) against the reference's
  own operators instantiated on dual numbers (oracle/ref_tlm.cpp): values
  bit-identical to the oracle, tangents equal to rounding, at generic states
  (no ties) where both define the same derivative.
* The tie rule: a gas at rest with uniform pressure and uneven density puts
  every face at ustar == 0 and un_L == un_R; the mean of the one-sided
  derivatives is what central differences converge to, the reference's
  one-sided pick is not.
* The transposed face arithmetic of the reverse step
  (csrc/adjoint_face.cuh, compiled here as host C++ by tests/adjoint_host.cpp)
  against the tangent-linear model: dot-product identity <J^T w, v> =
  <w, J v> and, on a small grid, the whole transposed Jacobian applied to w
  element by element.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, ROOT

GAMMA = 1.4
DX = (0.1, 0.12, 0.09)
DT = 1e-3


@pytest.fixture(scope="module")
def tlm(oracle_lib):
    return oracle_lib


@pytest.fixture(scope="module")
def host_adj(tmp_path_factory):
    out = tmp_path_factory.mktemp("adjhost") / "libadjoint_host.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(PKG_DIR, "csrc"),
                    os.path.join(ROOT, "tests", "adjoint_host.cpp"), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))

    def run(prim, cbar, gamma=GAMMA, dx=DX, dt=DT):
        P = lambda a: (ctypes.c_void_p * 5)(*[a[f].ctypes.data for f in range(5)])  # noqa: E731
        pbar = np.zeros_like(prim)
        n2, n1, n0 = prim.shape[1:]
        D = ctypes.c_double
        lib.host_godunov_adjoint(P(prim), P(cbar), P(pbar), n0, n1, n2, D(gamma), D(dx[0]), D(dx[1]), D(dx[2]),
                                 D(dt))
        return pbar

    return run


def rest_state(O, n0, n1, n2, seed):
    prim = O.random_prim(n0, n1, n2, seed=seed)
    prim[1] = 1.0
    prim[2:] = 0.0
    return prim


def maxrel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("shape", [(6, 5, 4), (10, 9, 8)])
def test_tlm_matches_dual_reference(tlm, shape):
    O = tlm
    if not (O.have_ref_tlm() or os.path.isdir(os.path.join(O.REFERENCE_DIR, "euler_operators"))):
        pytest.skip("the reference checkout is not present")
    O.build(ref=True)
    rng = np.random.default_rng(3)
    prim = O.random_prim(*shape, seed=5)
    dprim = rng.normal(size=prim.shape)
    cons, dcons = O.tlm_prim_to_cons(prim, dprim, GAMMA)
    c2, d2 = O.tlm_prim_to_cons(prim, dprim, GAMMA, impl="ref")
    assert np.array_equal(cons, c2) and np.array_equal(cons, O.prim_to_cons(prim, GAMMA))
    assert maxrel(dcons, d2) <= 1e-14
    p1, dp1 = O.tlm_cons_to_prim(cons, dcons, GAMMA)
    p2, dp2 = O.tlm_cons_to_prim(cons, dcons, GAMMA, impl="ref")
    assert np.array_equal(p1, p2)
    assert maxrel(dp1, dp2) <= 1e-14
    o1, do1 = O.tlm_godunov(prim, dprim, cons, dcons, GAMMA, DX, DT)
    o2, do2 = O.tlm_godunov(prim, dprim, cons, dcons, GAMMA, DX, DT, impl="ref")
    assert np.array_equal(o1, o2) and np.array_equal(o1, O.godunov(prim, cons, GAMMA, DX, DT))
    assert maxrel(do1, do2) <= 1e-14


def test_tlm_simulate_follows_oracle(tlm):
    """The tangent run's values are the oracle's fixed-dt trajectory."""
    O = tlm
    prim0 = O.random_prim(8, 7, 6, seed=2)
    prim0[2:] *= 0.1
    dts = [1e-3, 2e-3, 1.5e-3]
    pT, _ = O.tlm_simulate(prim0, np.zeros_like(prim0), GAMMA, DX, dts)
    prim, cons = prim0.copy(), O.prim_to_cons(prim0, GAMMA)
    for dt in dts:
        cons = O.godunov(prim, cons, GAMMA, DX, dt)
        prim = O.cons_to_prim(cons, GAMMA)
    assert np.array_equal(pT, prim)


def test_tlm_central_difference_generic(tlm):
    O = tlm
    rng = np.random.default_rng(4)
    prim = O.random_prim(9, 8, 7, seed=6)
    prim[2:] *= 0.2
    v = rng.normal(size=prim.shape)
    dts = [1e-3] * 3
    _, dT = O.tlm_simulate(prim, v, GAMMA, DX, dts)
    eps = 1e-6
    pp, _ = O.tlm_simulate(prim + eps * v, v, GAMMA, DX, dts)
    pm, _ = O.tlm_simulate(prim - eps * v, v, GAMMA, DX, dts)
    assert maxrel((pp - pm) / (2 * eps), dT) <= 1e-8


def test_tie_rule_is_the_central_difference_limit(tlm):
    O = tlm
    rng = np.random.default_rng(3)
    prim = rest_state(O, 10, 9, 8, seed=5)
    v = rng.normal(size=prim.shape)
    dts = [1e-3] * 3
    _, dT = O.tlm_simulate(prim, v, GAMMA, (0.1,) * 3, dts)
    errs = []
    for eps in (1e-5, 1e-6):
        pp, _ = O.tlm_simulate(prim + eps * v, v, GAMMA, (0.1,) * 3, dts)
        pm, _ = O.tlm_simulate(prim - eps * v, v, GAMMA, (0.1,) * 3, dts)
        errs.append(maxrel((pp - pm) / (2 * eps), dT))
    # first-order convergence: at a kink the central difference carries an
    # O(eps) term from the curvature jump, and no O(1) error
    assert errs[1] <= 5e-6 and errs[1] <= 0.2 * errs[0], errs
    if O.have_ref_tlm():
        cons, dcons = O.tlm_prim_to_cons(prim, v, GAMMA)
        _, one_sided = O.tlm_godunov(prim, v, cons, dcons, GAMMA, (0.1,) * 3, DT, impl="ref")
        _, mean_rule = O.tlm_godunov(prim, v, cons, dcons, GAMMA, (0.1,) * 3, DT)
        assert maxrel(one_sided, mean_rule) > 1e-3  # the reference's pick is a different (one-sided) derivative


@pytest.mark.parametrize("case", ["generic", "rest"])
@pytest.mark.parametrize("dx", [DX, (0.1,) * 3], ids=["anisotropic", "cubic"])
def test_face_adjoint_dot_product(tlm, host_adj, case, dx):
    """<J^T w, v> = <w, J v>; cubic cells take the path with the face area
    folded into the weights."""
    O = tlm
    rng = np.random.default_rng(7)
    prim = O.random_prim(9, 8, 7, seed=11) if case == "generic" else rest_state(O, 9, 8, 7, seed=11)
    cons = O.prim_to_cons(prim, GAMMA)
    for _ in range(3):
        w = rng.normal(size=prim.shape)
        v = rng.normal(size=prim.shape)
        _, jv = O.tlm_godunov(prim, v, cons, np.zeros_like(cons), GAMMA, dx, DT)
        lhs = float(np.sum(host_adj(prim, w, dx=dx) * v))
        rhs = float(np.sum(w * jv))
        assert abs(lhs - rhs) <= 1e-13 * abs(rhs)


def test_face_adjoint_full_transpose(tlm, host_adj):
    """Every entry of J^T w on a 5x5x5 grid (one tangent run per input)."""
    O = tlm
    rng = np.random.default_rng(8)
    prim = O.random_prim(5, 5, 5, seed=12)
    prim[2:] *= 0.3
    cons = O.prim_to_cons(prim, GAMMA)
    w = rng.normal(size=prim.shape)
    adj = host_adj(prim, w)
    ref = np.zeros_like(prim)
    zero = np.zeros_like(cons)
    for idx in np.ndindex(*prim.shape):
        e = np.zeros_like(prim)
        e[idx] = 1.0
        _, je = O.tlm_godunov(prim, e, cons, zero, GAMMA, DX, DT)
        ref[idx] = np.sum(w * je)
    assert maxrel(adj, ref) <= 1e-13
