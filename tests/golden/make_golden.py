"""Generate the golden fixtures in this folder from the reference itself.

The reference operators (euler_operators/*.hpp) are compiled unmodified
through the test-only Kokkos shim into ``oracle/_ref/libeuler_ref.so``
(``make -C oracle ref``).  This script runs them on small seeded inputs and
stores inputs and outputs as ``.npz`` files.  The tests then pin both the C
oracle and the CUDA library against these files; the reference checkout is not
needed at test time.

Usage (from the repository root):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
GAMMA = 1.4
CFL = 0.4


def operator_case(name, n0, n1, n2, dx, seed, dtype):
    """One call of each operator on a seeded random state (the per-operator
    benchmark inputs: rho, p log-uniform on [0.1, 10], u ~ N(0, 1))."""
    prim = O.random_prim(n0, n1, n2, seed=seed, dtype=dtype)
    cons = O.prim_to_cons(prim, GAMMA, impl="ref")
    prim_rt = O.cons_to_prim(cons, GAMMA, impl="ref")
    dt = O.time_step(prim, GAMMA, dx, impl="ref")
    cons_gd = O.godunov(prim, cons, GAMMA, dx, CFL * dt, impl="ref")
    np.savez_compressed(
        os.path.join(OUT, f"{name}.npz"),
        prim=prim, cons=cons, prim_rt=prim_rt, dt=np.array(dt, dtype=dtype),
        cons_godunov=cons_gd, dx=np.array(dx, dtype=dtype), gamma=np.array(GAMMA, dtype=dtype),
        cfl=np.array(CFL, dtype=dtype),
    )


def uniform_case(name, n, dtype):
    """The reference benchmark fill (benchmark_godunov.cpp:33-35): d=1, p=1,
    u=0 everywhere, dx=1, dt=1e-9.  godunov leaves cons unchanged."""
    prim = O.empty_bundle(n, n, n, dtype)
    prim[0] = 1
    prim[1] = 1
    cons = O.prim_to_cons(prim, GAMMA, impl="ref")
    dx = (1.0, 1.0, 1.0)
    dt = O.time_step(prim, GAMMA, dx, impl="ref")
    cons_gd = O.godunov(prim, cons, GAMMA, dx, 1e-9, impl="ref")
    np.savez_compressed(
        os.path.join(OUT, f"{name}.npz"),
        prim=prim, cons=cons, dt=np.array(dt, dtype=dtype), cons_godunov=cons_gd,
        dx=np.array(dx, dtype=dtype), gamma=np.array(GAMMA, dtype=dtype), dt_godunov=np.array(1e-9, dtype=dtype),
    )


def implode_case(name, nx, steps, dtype):
    """init_implode + prim_to_cons, then the euler_simulation loop
    (time_step, godunov(cfl*dt), cons_to_prim) for each count in ``steps``."""
    n = nx + 2
    dx = (1.0 / nx,) * 3
    prim = O.init_implode(n, n, n, dx, dtype=dtype, impl="ref")
    cons = O.prim_to_cons(prim, GAMMA, impl="ref")
    arrays = {"prim0": prim.copy(), "cons0": cons.copy(), "dx": np.array(dx, dtype=dtype),
              "gamma": np.array(GAMMA, dtype=dtype), "cfl": np.array(CFL, dtype=dtype)}
    done = 0
    t = 0.0
    for s in steps:
        t += O.simulate(prim, cons, GAMMA, dx, CFL, s - done, impl="ref")
        done = s
        arrays[f"prim_{s}"] = prim.copy()
        arrays[f"cons_{s}"] = cons.copy()
        arrays[f"t_{s}"] = np.array(t)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)


def main():
    if not O.have_ref():
        O.build(ref=True)
    for dtype, tag in ((np.float64, "f64"), (np.float32, "f32")):
        operator_case(f"ops_7x9x6_{tag}", 7, 9, 6, (1 / 5, 1 / 7, 1 / 4), seed=11, dtype=dtype)
        operator_case(f"ops_20x12x10_{tag}", 20, 12, 10, (1 / 18, 1 / 10, 1 / 8), seed=12, dtype=dtype)
        operator_case(f"ops_3x3x3_{tag}", 3, 3, 3, (1.0, 1.0, 1.0), seed=13, dtype=dtype)
        operator_case(f"ops_2x5x4_{tag}", 2, 5, 4, (0.5, 0.25, 1 / 3), seed=14, dtype=dtype)
        uniform_case(f"uniform_10_{tag}", 10, dtype)
        implode_case(f"implode_16_{tag}", 16, (1, 10), dtype)
    # NPY files written by the reference's own writer (simulations/save_npy.cpp)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "npy"], check=True)
    subprocess.run([os.path.join(ROOT, "oracle", "_ref", "npy_golden"), OUT], check=True)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
