"""CPU oracle for the Euler operators -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg and
reference arm of ``bench.py`` use this module, and only as the parity
reference or as the timed CPU baseline.  The product path (the CUDA library)
never imports it.

Two implementations sit behind the same numpy interface:

* ``impl="port"`` -- ``oracle/euler_oracle.c``, a plain-C restatement of the
  reference's ``euler_operators/*.hpp`` (built into
  ``oracle/_build/libeuler_oracle.so``).  It builds anywhere gcc does.
* ``impl="ref"`` -- the reference's own headers compiled unmodified through the
  test-only Kokkos shim (``oracle/_ref/libeuler_ref.so``).  It can only be built
  where the reference checkout exists; it pins the port and generated the
  golden fixtures in ``tests/golden/``.

A bundle is a numpy array of shape ``(5, n2, n1, n0)``: field-major, and each
field is a layout_left block (i fastest), matching the reference's SoA
``EulerPrimArrays`` / ``EulerConsArrays`` (euler_arrays.hpp:77-85, 228-236).
prim fields are (d, p, ux0, ux1, ux2); cons fields are (d, e, mx0, mx1, mx2).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libeuler_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libeuler_ref.so")
REF_TLM_SO = os.path.join(HERE, "_ref", "libeuler_ref_tlm.so")
# The reference checkout: $EULER_REFERENCE_DIR, else a directory named
# "reference" beside this repository's root.
REFERENCE_DIR = os.environ.get("EULER_REFERENCE_DIR") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")

_DT = {"f64": (np.float64, ctypes.c_double), "f32": (np.float32, ctypes.c_float)}
_libs: dict[str, ctypes.CDLL] = {}


def build(ref: bool | None = None) -> None:
    """Compile the C port, and the reference build when its sources exist."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is None:
        ref = os.path.isdir(os.path.join(REFERENCE_DIR, "euler_operators"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_DIR}"], check=True)


def have_ref() -> bool:
    return os.path.exists(REF_SO)


def have_ref_tlm() -> bool:
    return os.path.exists(REF_TLM_SO)


def _lib(impl: str) -> tuple[ctypes.CDLL, str]:
    if impl not in ("port", "ref"):
        raise ValueError(f"unknown oracle implementation {impl!r}")
    if impl not in _libs:
        path = PORT_SO if impl == "port" else REF_SO
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} is not built (run oracle.build())")
        _libs[impl] = ctypes.CDLL(path)
    return _libs[impl], ("oracle_" if impl == "port" else "ref_")


def _suffix(arr: np.ndarray) -> str:
    if arr.dtype == np.float64:
        return "f64"
    if arr.dtype == np.float32:
        return "f32"
    raise TypeError(f"unsupported dtype {arr.dtype}")


def _ptrs(bundle: np.ndarray):
    if bundle.ndim != 4 or bundle.shape[0] != 5 or not bundle.flags.c_contiguous:
        raise ValueError("a bundle is a C-contiguous array of shape (5, n2, n1, n0)")
    return (ctypes.c_void_p * 5)(*[bundle[f].ctypes.data for f in range(5)])


def _dims(bundle: np.ndarray) -> tuple[int, int, int]:
    n2, n1, n0 = bundle.shape[1:]
    return int(n0), int(n1), int(n2)


def _fn(impl: str, name: str, suf: str, restype=None):
    lib, prefix = _lib(impl)
    f = getattr(lib, f"{prefix}{name}_{suf}")
    f.restype = restype
    return f


def empty_bundle(n0: int, n1: int, n2: int, dtype=np.float64) -> np.ndarray:
    return np.zeros((5, n2, n1, n0), dtype=dtype)


def init_implode(n0, n1, n2, dx, dtype=np.float64, impl="port") -> np.ndarray:
    """init_implode (init_implode.hpp:7-45) over an (n0, n1, n2) grid incl. ghosts."""
    prim = empty_bundle(n0, n1, n2, dtype)
    suf = _suffix(prim)
    c = _DT[suf][1]
    _fn(impl, "init_implode", suf)(_ptrs(prim), n0, n1, n2, c(dx[0]), c(dx[1]), c(dx[2]))
    return prim


def init_step(n0, n1, n2, dx, c, rho_in, p_in, rho_out=1.0, p_out=1.0, dtype=np.float64) -> np.ndarray:
    """Step initial condition of the batched workload (x0 + x1 + x2 < c), port only."""
    prim = empty_bundle(n0, n1, n2, dtype)
    suf = _suffix(prim)
    D = ctypes.c_double
    _fn("port", "init_step", suf)(_ptrs(prim), n0, n1, n2, D(dx[0]), D(dx[1]), D(dx[2]), D(c), D(rho_in), D(p_in),
                                  D(rho_out), D(p_out))
    return prim


def prim_to_cons(prim: np.ndarray, gamma: float, impl="port") -> np.ndarray:
    cons = np.zeros_like(prim)
    suf = _suffix(prim)
    _fn(impl, "prim_to_cons", suf)(_ptrs(prim), _ptrs(cons), *_dims(prim), _DT[suf][1](gamma))
    return cons


def cons_to_prim(cons: np.ndarray, gamma: float, impl="port") -> np.ndarray:
    prim = np.zeros_like(cons)
    suf = _suffix(cons)
    _fn(impl, "cons_to_prim", suf)(_ptrs(cons), _ptrs(prim), *_dims(cons), _DT[suf][1](gamma))
    return prim


def time_step(prim: np.ndarray, gamma: float, dx, impl="port") -> float:
    suf = _suffix(prim)
    c = _DT[suf][1]
    f = _fn(impl, "time_step", suf, restype=c)
    return f(_ptrs(prim), *_dims(prim), c(gamma), c(dx[0]), c(dx[1]), c(dx[2]))


def godunov(prim: np.ndarray, cons: np.ndarray, gamma: float, dx, dt: float, impl="port") -> np.ndarray:
    """Returns the updated copy of ``cons`` (the reference updates in place)."""
    out = cons.copy()
    suf = _suffix(prim)
    c = _DT[suf][1]
    _fn(impl, "godunov", suf)(
        _ptrs(prim), _ptrs(out), *_dims(prim), c(gamma), c(dx[0]), c(dx[1]), c(dx[2]), c(dt)
    )
    return out


def hllc_faces(direction: int, gamma: float, qL: np.ndarray, qR: np.ndarray, impl="port") -> np.ndarray:
    """HLLC fluxes (d, e, m0, m1, m2) of faces normal to axis `direction`
    between primitive states qL[k] and qR[k] (arrays of shape (N, 5): d, p,
    u0, u1, u2), one call of the solver per face (hllc.hpp:50-105)."""
    qL = np.ascontiguousarray(qL)
    qR = np.ascontiguousarray(qR)
    if qL.shape != qR.shape or qL.ndim != 2 or qL.shape[1] != 5 or qL.dtype != qR.dtype:
        raise ValueError("face states are two arrays of shape (N, 5) of one dtype")
    suf = _suffix(qL)
    c = _DT[suf][1]
    fn = _fn(impl, "hllc_face", suf)
    out = np.empty_like(qL)
    P = ctypes.POINTER(c)
    for k in range(qL.shape[0]):
        fn(int(direction), c(gamma), qL[k].ctypes.data_as(P), qR[k].ctypes.data_as(P), out[k].ctypes.data_as(P))
    return out


def simulate(prim: np.ndarray, cons: np.ndarray, gamma: float, dx, cfl: float, nsteps: int, impl="port"):
    """nsteps of the reference loop (euler_simulation.cpp:56-68), in place.

    Returns the simulated time, accumulated in double."""
    suf = _suffix(prim)
    c = _DT[suf][1]
    t = ctypes.c_double(0.0)
    _fn(impl, "simulate", suf)(
        _ptrs(prim), _ptrs(cons), *_dims(prim), c(gamma), c(dx[0]), c(dx[1]), c(dx[2]), c(cfl),
        int(nsteps), ctypes.byref(t),
    )
    return t.value


# ---------------------------------------------------- tangent-linear model
# Forward-mode derivative of the step with dt fixed (oracle/euler_tlm.c, and
# with impl="ref" the reference's own operators instantiated on dual numbers,
# oracle/ref_tlm.cpp).  Each function takes and returns (value, tangent)
# bundles.

def _tlm_fn(impl: str, name: str):
    if impl == "port":
        lib, _ = _lib("port")
        return getattr(lib, f"oracle_tlm_{name}_f64")
    if impl == "ref":
        if "ref_tlm" not in _libs:
            if not os.path.exists(REF_TLM_SO):
                raise FileNotFoundError(f"oracle library {REF_TLM_SO} is not built (run oracle.build())")
            _libs["ref_tlm"] = ctypes.CDLL(REF_TLM_SO)
        return getattr(_libs["ref_tlm"], f"ref_tlm_{name}_f64")
    raise ValueError(f"unknown oracle implementation {impl!r}")


def _f64(*arrays):
    for a in arrays:
        if a.dtype != np.float64:
            raise TypeError("the tangent-linear model is FP64")


def tlm_prim_to_cons(prim, dprim, gamma, impl="port"):
    _f64(prim, dprim)
    cons, dcons = np.zeros_like(prim), np.zeros_like(prim)
    _tlm_fn(impl, "prim_to_cons")(_ptrs(prim), _ptrs(dprim), _ptrs(cons), _ptrs(dcons), *_dims(prim),
                                  ctypes.c_double(gamma))
    return cons, dcons


def tlm_cons_to_prim(cons, dcons, gamma, impl="port"):
    _f64(cons, dcons)
    prim, dprim = np.zeros_like(cons), np.zeros_like(cons)
    _tlm_fn(impl, "cons_to_prim")(_ptrs(cons), _ptrs(dcons), _ptrs(prim), _ptrs(dprim), *_dims(cons),
                                  ctypes.c_double(gamma))
    return prim, dprim


def tlm_godunov(prim, dprim, cons, dcons, gamma, dx, dt, impl="port"):
    """Updated copies of (cons, dcons) after godunov(prim, cons, dt)."""
    _f64(prim, dprim, cons, dcons)
    out, dout = cons.copy(), dcons.copy()
    D = ctypes.c_double
    _tlm_fn(impl, "godunov")(_ptrs(prim), _ptrs(dprim), _ptrs(out), _ptrs(dout), *_dims(prim), D(gamma), D(dx[0]),
                             D(dx[1]), D(dx[2]), D(dt))
    return out, dout


def tlm_simulate(prim0, dprim0, gamma, dx, dts):
    """(prim, dprim) after len(dts) steps of fixed dt from (prim0, dprim0) (port)."""
    _f64(prim0, dprim0)
    prim, dprim = prim0.copy(), dprim0.copy()
    cons, dcons = np.zeros_like(prim), np.zeros_like(prim)
    D = ctypes.c_double
    arr = (ctypes.c_double * max(len(dts), 1))(*[float(v) for v in dts])
    _tlm_fn("port", "simulate")(_ptrs(prim), _ptrs(dprim), _ptrs(cons), _ptrs(dcons), *_dims(prim), D(gamma),
                                D(dx[0]), D(dx[1]), D(dx[2]), arr, len(dts))
    return prim, dprim


def random_prim(n0, n1, n2, seed=0, dtype=np.float64) -> np.ndarray:
    """Seeded random primitive state: rho and p log-uniform on [0.1, 10], each
    velocity component N(0, 1) (numpy PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    prim = empty_bundle(n0, n1, n2, np.float64)
    shape = prim.shape[1:]
    prim[0] = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=shape))
    prim[1] = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=shape))
    for f in (2, 3, 4):
        prim[f] = rng.normal(0.0, 1.0, size=shape)
    return np.ascontiguousarray(prim.astype(dtype))
