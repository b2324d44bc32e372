"""ctypes bindings of libeuler_gb300.so (the C ABI in include/euler_gb300.h).

This is host plumbing for tests, benchmarks and Python users: device memory
comes from PyTorch tensors, every call goes through the C ABI, and there is no
CPU fallback -- if the CUDA library is missing, loading fails loudly.

A bundle is a contiguous tensor (or numpy array) of shape (5, n2, n1, n0):
field-major, each field a layout_left block (i fastest), the layout of the
reference's EulerPrimArrays/EulerConsArrays (euler_arrays.hpp:77-85,
228-236).  prim fields are (d, p, ux0, ux1, ux2); cons fields are
(d, e, mx0, mx1, mx2).
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB_PATH, build  # noqa: F401

EULR_SUCCESS = 0
STATUS_NAMES = {
    0: "EULR_SUCCESS", -1: "EULR_ERR_INVALID_ARGUMENT", -2: "EULR_ERR_INVALID_VALUE",
    -3: "EULR_ERR_MISALIGNED", -4: "EULR_ERR_CUDA", -5: "EULR_ERR_OUT_OF_MEMORY",
    -6: "EULR_ERR_TOO_LARGE", -7: "EULR_ERR_NONFINITE", -8: "EULR_ERR_NO_DEVICE",
    -9: "EULR_ERR_UNSUPPORTED",
}
PRECISION = {"f64": 0, "f32c": 1, "f32": 2, "f32c_hilo": 3}


class EulerError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class GridDesc(ctypes.Structure):
    """eulr_grid_desc: extents (ghosts included), gamma, spacings."""
    _fields_ = [("n0", ctypes.c_int), ("n1", ctypes.c_int), ("n2", ctypes.c_int), ("gamma", ctypes.c_double),
                ("dx0", ctypes.c_double), ("dx1", ctypes.c_double), ("dx2", ctypes.c_double)]


class Bundle5(ctypes.Structure):
    """Five field pointers (eulr_prim_* / eulr_cons_*; const or not)."""
    _fields_ = [("f0", ctypes.c_void_p), ("f1", ctypes.c_void_p), ("f2", ctypes.c_void_p),
                ("f3", ctypes.c_void_p), ("f4", ctypes.c_void_p)]


_lib: ctypes.CDLL | None = None

# (name, restype, argtypes); D = c_double, F = c_float, I = c_int, P = c_void_p
_D, _F, _I, _P = ctypes.c_double, ctypes.c_float, ctypes.c_int, ctypes.c_void_p
_SIGNATURES = [
    ("eulr_version", _I, []),
    ("eulr_status_string", ctypes.c_char_p, [_I]),
    ("eulr_last_error", ctypes.c_char_p, []),
    ("eulr_init_implode_f64", _I, [Bundle5, _I, _I, _I, _D, _D, _D, _P]),
    ("eulr_init_implode_f32", _I, [Bundle5, _I, _I, _I, _F, _F, _F, _P]),
    ("eulr_prim_to_cons_f64", _I, [Bundle5, Bundle5, _I, _I, _I, _D, _P]),
    ("eulr_prim_to_cons_f32", _I, [Bundle5, Bundle5, _I, _I, _I, _F, _P]),
    ("eulr_cons_to_prim_f64", _I, [Bundle5, Bundle5, _I, _I, _I, _D, _P]),
    ("eulr_cons_to_prim_f32", _I, [Bundle5, Bundle5, _I, _I, _I, _F, _P]),
    ("eulr_time_step_f64", _I, [Bundle5, _I, _I, _I, _D, _D, _D, _D, _P, _P]),
    ("eulr_time_step_f32", _I, [Bundle5, _I, _I, _I, _F, _F, _F, _F, _P, _P]),
    ("eulr_time_step_noalloc_f64", _I, [Bundle5, _I, _I, _I, _D, _D, _D, _D, _P, _P]),
    ("eulr_godunov_f64", _I, [Bundle5, Bundle5, _I, _I, _I, _D, _D, _D, _D, _D, _P]),
    ("eulr_godunov_f32", _I, [Bundle5, Bundle5, _I, _I, _I, _F, _F, _F, _F, _F, _P]),
    ("eulr_godunov_devdt_f64", _I, [Bundle5, Bundle5, _I, _I, _I, _D, _D, _D, _D, _P, _D, _P]),
    ("eulr_godunov_exact_f64", _I, [Bundle5, Bundle5, _I, _I, _I, _D, _D, _D, _D, _D, _P]),
    ("eulr_godunov_exact_f32", _I, [Bundle5, Bundle5, _I, _I, _I, _F, _F, _F, _F, _F, _P]),
    ("eulr_sim_create", _I, [_I, _I, _I, _I, _D, _D, _D, _D, _D, _P, ctypes.POINTER(_P)]),
    ("eulr_sim_destroy", _I, [_P]),
    ("eulr_sim_set_prim_f64", _I, [_P, Bundle5]),
    ("eulr_sim_set_state_f64", _I, [_P, Bundle5, Bundle5]),
    ("eulr_sim_init_implode", _I, [_P]),
    ("eulr_sim_advance", _I, [_P, _I]),
    ("eulr_sim_set_dt_sequence", _I, [_P, ctypes.POINTER(_D), ctypes.c_longlong]),
    ("eulr_sim_get_state_f64", _I, [_P, Bundle5, Bundle5]),
    ("eulr_sim_get_state_async_f64", _I, [_P, Bundle5, Bundle5]),
    ("eulr_sim_synchronize", _I, [_P]),
    ("eulr_sim_time", _I, [_P, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_longlong)]),
    ("eulr_sim_status", _I, [_P]),
    ("eulr_sim_launches_per_step", _I, [_P]),
    ("eulr_sim_profile_step", _I, [_P, ctypes.POINTER(_F)]),
    ("eulr_sim_totals", _I, [_P, ctypes.POINTER(_D)]),
    ("eulr_sim_state_bytes", _I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    ("eulr_probe_fma_rate", _I, [_I, _I, ctypes.POINTER(_D)]),
    ("eulr_godunov_adjoint_workspace_bytes", ctypes.c_size_t, [_I, _I, _I]),
    ("eulr_godunov_adjoint_f64", _I, [Bundle5, Bundle5, Bundle5, _I, _I, _I, _D, _D, _D, _D, _D, _P,
                                      ctypes.c_size_t, _P]),
    ("eulr_cons_to_prim_adjoint_f64", _I, [Bundle5, Bundle5, Bundle5, _I, _I, _I, _D, _I, _P]),
    ("eulr_prim_to_cons_adjoint_f64", _I, [Bundle5, Bundle5, Bundle5, _I, _I, _I, _D, _I, _P]),
    ("eulr_adjoint_create", _I, [_I, _I, _I, _D, _D, _D, _D, _D, _I, _I, _P, ctypes.POINTER(_P)]),
    ("eulr_adjoint_destroy", _I, [_P]),
    ("eulr_adjoint_forward", _I, [_P, Bundle5, ctypes.POINTER(_D), Bundle5]),
    ("eulr_adjoint_dts", _I, [_P, ctypes.POINTER(_D)]),
    ("eulr_adjoint_backward", _I, [_P, Bundle5, Bundle5]),
    ("eulr_adjoint_timing", _I, [_P, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    ("eulr_batch_create", _I, [_I, _I, _P, _D, _P, ctypes.POINTER(_P)]),
    ("eulr_batch_destroy", _I, [_P]),
    ("eulr_batch_set_prim_f64", _I, [_P, _I, Bundle5]),
    ("eulr_batch_init_step", _I, [_P, _I, _D, _D, _D, _D, _D]),
    ("eulr_batch_autotune", _I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_D)]),
    ("eulr_batch_advance", _I, [_P, _I]),
    ("eulr_batch_get_state_f64", _I, [_P, _I, Bundle5, Bundle5]),
    ("eulr_batch_time", _I, [_P, _I, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_longlong)]),
    ("eulr_batch_status", _I, [_P]),
    ("eulr_batch_info", _I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_I), ctypes.POINTER(_I),
                             ctypes.POINTER(_I)]),
]

# Every symbol include/euler_gb300.h declares (checked by the CPU tests).
EXPORTED = [s[0] for s in _SIGNATURES]


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the CUDA library (build it first with build()); raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            f"{p} is missing: the Euler operators have no CPU fallback; build the CUDA library first")
    lib = ctypes.CDLL(p)
    for name, res, args in _SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != EULR_SUCCESS:
        msg = load().eulr_last_error().decode(errors="replace")
        raise EulerError(status, msg)


# ------------------------------------------------------------ tensor helpers
def _torch():
    import torch
    return torch


def bundle(t) -> Bundle5:
    """Field pointers of a (5, n2, n1, n0) contiguous tensor or numpy array."""
    if hasattr(t, "data_ptr"):
        if not t.is_contiguous() or t.dim() != 4 or t.shape[0] != 5:
            raise ValueError("a bundle is a contiguous tensor of shape (5, n2, n1, n0)")
        step = t[0].numel() * t.element_size()
        base = t.data_ptr()
    else:
        if not t.flags.c_contiguous or t.ndim != 4 or t.shape[0] != 5:
            raise ValueError("a bundle is a C-contiguous array of shape (5, n2, n1, n0)")
        step = t[0].nbytes
        base = t.ctypes.data
    return Bundle5(*[base + f * step for f in range(5)])


def null_bundle() -> Bundle5:
    return Bundle5(None, None, None, None, None)


def dims(t) -> tuple[int, int, int]:
    n2, n1, n0 = t.shape[1:]
    return int(n0), int(n1), int(n2)


def _sfx(t) -> str:
    torch = _torch()
    if t.dtype == torch.float64:
        return "f64"
    if t.dtype == torch.float32:
        return "f32"
    raise TypeError(f"unsupported dtype {t.dtype}")


def _stream(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _scalar(sfx):
    return _D if sfx == "f64" else _F


def init_implode(n0, n1, n2, dx, dtype=None, device="cuda", stream=None):
    torch = _torch()
    dtype = dtype or torch.float64
    prim = torch.empty((5, n2, n1, n0), dtype=dtype, device=device)
    sfx = _sfx(prim)
    c = _scalar(sfx)
    check(getattr(load(), f"eulr_init_implode_{sfx}")(bundle(prim), n0, n1, n2, c(dx[0]), c(dx[1]), c(dx[2]),
                                                       _stream(stream)))
    return prim


def prim_to_cons(prim, gamma, out=None, stream=None):
    cons = out if out is not None else _torch().empty_like(prim)
    sfx = _sfx(prim)
    check(getattr(load(), f"eulr_prim_to_cons_{sfx}")(bundle(prim), bundle(cons), *dims(prim),
                                                       _scalar(sfx)(gamma), _stream(stream)))
    return cons


def cons_to_prim(cons, gamma, out=None, stream=None):
    prim = out if out is not None else _torch().empty_like(cons)
    sfx = _sfx(cons)
    check(getattr(load(), f"eulr_cons_to_prim_{sfx}")(bundle(cons), bundle(prim), *dims(cons),
                                                       _scalar(sfx)(gamma), _stream(stream)))
    return prim


def time_step(prim, gamma, dx, out=None, stream=None):
    """Device scalar tensor holding time_step(prim) (not multiplied by CFL)."""
    torch = _torch()
    dt = out if out is not None else torch.empty((), dtype=prim.dtype, device=prim.device)
    sfx = _sfx(prim)
    c = _scalar(sfx)
    check(getattr(load(), f"eulr_time_step_{sfx}")(bundle(prim), *dims(prim), c(gamma), c(dx[0]), c(dx[1]),
                                                    c(dx[2]), ctypes.c_void_p(dt.data_ptr()), _stream(stream)))
    return dt


def godunov(prim, cons, gamma, dx, dt, stream=None, exact=False):
    """In-place update of cons (interior cells) from prim; dt is a float or a
    device scalar tensor (then dt_used = cfl * dt with cfl given as a tuple
    (tensor, cfl)).  exact=True: bit-identical to the reference
    (eulr_godunov_exact_*; a float dt only)."""
    sfx = _sfx(prim)
    c = _scalar(sfx)
    if exact:
        if isinstance(dt, tuple):
            raise ValueError("the exact godunov takes dt as a number")
        check(getattr(load(), f"eulr_godunov_exact_{sfx}")(bundle(prim), bundle(cons), *dims(prim), c(gamma),
                                                            c(dx[0]), c(dx[1]), c(dx[2]), c(dt), _stream(stream)))
        return cons
    if isinstance(dt, tuple):
        dt_t, cfl = dt
        check(load().eulr_godunov_devdt_f64(bundle(prim), bundle(cons), *dims(prim), c(gamma), c(dx[0]),
                                            c(dx[1]), c(dx[2]), ctypes.c_void_p(dt_t.data_ptr()), c(cfl),
                                            _stream(stream)))
    else:
        check(getattr(load(), f"eulr_godunov_{sfx}")(bundle(prim), bundle(cons), *dims(prim), c(gamma), c(dx[0]),
                                                      c(dx[1]), c(dx[2]), c(dt), _stream(stream)))
    return cons


class Simulation:
    """Device-resident simulation (eulr_sim_*): state, CUDA-graph step loop."""

    def __init__(self, n0, n1, n2, gamma=1.4, dx=None, cfl=0.4, precision="f64", stream=None):
        self.shape = (n0, n1, n2)
        if dx is None:
            dx = (1.0 / (n0 - 2), 1.0 / (n1 - 2), 1.0 / (n2 - 2))
        self.dx = tuple(float(v) for v in dx)
        self.gamma = float(gamma)
        self.cfl = float(cfl)
        self.precision = precision
        h = ctypes.c_void_p()
        s = ctypes.c_void_p(stream.cuda_stream) if stream is not None else ctypes.c_void_p(None)
        check(load().eulr_sim_create(PRECISION[precision], n0, n1, n2, self.gamma, *self.dx, self.cfl, s,
                                     ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().eulr_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_prim(self, prim):
        check(load().eulr_sim_set_prim_f64(self._h, bundle(prim)))

    def set_state(self, prim, cons):
        check(load().eulr_sim_set_state_f64(self._h, bundle(prim), bundle(cons)))

    def init_implode(self):
        check(load().eulr_sim_init_implode(self._h))

    def advance(self, nsteps):
        check(load().eulr_sim_advance(self._h, int(nsteps)))

    def set_dt_sequence(self, dts):
        """Fix step n's dt to dts[n] (applies from the next load)."""
        arr = (ctypes.c_double * len(dts))(*[float(v) for v in dts])
        check(load().eulr_sim_set_dt_sequence(self._h, arr, len(dts)))

    def get_state(self, prim=None, cons=None, wait=True):
        """Copy the state into the given bundles (host numpy or device tensors).
        With wait=False (FP64) the copies are only enqueued; see synchronize()."""
        fn = load().eulr_sim_get_state_f64 if wait else load().eulr_sim_get_state_async_f64
        check(fn(self._h, bundle(prim) if prim is not None else null_bundle(),
                 bundle(cons) if cons is not None else null_bundle()))

    def synchronize(self):
        check(load().eulr_sim_synchronize(self._h))

    def state_numpy(self):
        import numpy as np
        n0, n1, n2 = self.shape
        prim = np.zeros((5, n2, n1, n0))
        cons = np.zeros((5, n2, n1, n0))
        self.get_state(prim, cons)
        return prim, cons

    def time(self):
        t, dt, st = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        check(load().eulr_sim_time(self._h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(st)))
        return t.value, dt.value, st.value

    def status(self) -> int:
        return load().eulr_sim_status(self._h)

    def launches_per_step(self) -> int:
        return load().eulr_sim_launches_per_step(self._h)

    def profile_step(self):
        """One step with per-launch CUDA-event times (ms): ghost, flux, finalize."""
        ms = (ctypes.c_float * 3)()
        check(load().eulr_sim_profile_step(self._h, ms))
        return list(ms)

    def totals(self):
        out = (ctypes.c_double * 5)()
        check(load().eulr_sim_totals(self._h, out))
        return list(out)

    def state_bytes(self) -> int:
        out = ctypes.c_longlong()
        check(load().eulr_sim_state_bytes(self._h, ctypes.byref(out)))
        return out.value


class Batch:
    """Multi-grid batch (eulr_batch_*): uneven grids, one persistent launch per step."""

    def __init__(self, grids, cfl=0.4, precision="f64", stream=None):
        """grids: sequence of (n0, n1, n2, gamma, dx0, dx1, dx2), extents with ghosts."""
        self.shapes = [tuple(int(v) for v in g[:3]) for g in grids]
        arr = (GridDesc * len(grids))(*[GridDesc(*[int(v) for v in g[:3]], *[float(v) for v in g[3:7]])
                                        for g in grids])
        h = ctypes.c_void_p()
        s = ctypes.c_void_p(stream.cuda_stream) if stream is not None else ctypes.c_void_p(None)
        check(load().eulr_batch_create(PRECISION[precision], len(grids), ctypes.cast(arr, ctypes.c_void_p),
                                       float(cfl), s, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().eulr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_prim(self, g, prim):
        check(load().eulr_batch_set_prim_f64(self._h, int(g), bundle(prim)))

    def init_step(self, g, c, rho_in, p_in, rho_out=1.0, p_out=1.0):
        check(load().eulr_batch_init_step(self._h, int(g), float(c), float(rho_in), float(p_in), float(rho_out),
                                          float(p_out)))

    def autotune(self, trial_steps=2):
        shape, kc, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        check(load().eulr_batch_autotune(self._h, int(trial_steps), ctypes.byref(shape), ctypes.byref(kc),
                                         ctypes.byref(ms)))
        return {"tile": (shape.value // 1000, shape.value % 1000), "kchunk": kc.value, "step_ms": ms.value}

    def advance(self, nsteps):
        check(load().eulr_batch_advance(self._h, int(nsteps)))

    def state_numpy(self, g):
        import numpy as np
        n0, n1, n2 = self.shapes[g]
        prim = np.zeros((5, n2, n1, n0))
        cons = np.zeros((5, n2, n1, n0))
        check(load().eulr_batch_get_state_f64(self._h, int(g), bundle(prim), bundle(cons)))
        return prim, cons

    def time(self, g):
        t, dt, st = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        check(load().eulr_batch_time(self._h, int(g), ctypes.byref(t), ctypes.byref(dt), ctypes.byref(st)))
        return t.value, dt.value, st.value

    def status(self) -> int:
        return load().eulr_batch_status(self._h)

    def info(self):
        cells, items, shape, kc = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(load().eulr_batch_info(self._h, ctypes.byref(cells), ctypes.byref(items), ctypes.byref(shape),
                                     ctypes.byref(kc)))
        return {"interior_cells": cells.value, "items": items.value,
                "tile": (shape.value // 1000, shape.value % 1000), "kchunk": kc.value}


def godunov_adjoint(prim, cons_bar, gamma, dx, dt, out=None, workspace=None, stream=None):
    """prim_bar = (d godunov / d prim)^T cons_bar (device tensors, FP64)."""
    torch = _torch()
    n0, n1, n2 = dims(prim)
    need = load().eulr_godunov_adjoint_workspace_bytes(n0, n1, n2)
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=prim.device)
    prim_bar = out if out is not None else torch.empty_like(prim)
    check(load().eulr_godunov_adjoint_f64(bundle(prim), bundle(cons_bar), bundle(prim_bar), n0, n1, n2,
                                          float(gamma), float(dx[0]), float(dx[1]), float(dx[2]), float(dt),
                                          ctypes.c_void_p(workspace.data_ptr()), workspace.numel(),
                                          _stream(stream)))
    return prim_bar


def cons_to_prim_adjoint(prim, prim_bar, gamma, out=None, accumulate=False, stream=None):
    """cons_bar (+)= cons_to_prim'(state with primitive variables prim)^T prim_bar."""
    cons_bar = out if out is not None else _torch().empty_like(prim)
    check(load().eulr_cons_to_prim_adjoint_f64(bundle(prim), bundle(prim_bar), bundle(cons_bar), *dims(prim),
                                               float(gamma), int(bool(accumulate)), _stream(stream)))
    return cons_bar


def prim_to_cons_adjoint(prim, cons_bar, gamma, out=None, accumulate=False, stream=None):
    """prim_bar (+)= prim_to_cons'(prim)^T cons_bar."""
    prim_bar = out if out is not None else _torch().empty_like(prim)
    check(load().eulr_prim_to_cons_adjoint_f64(bundle(prim), bundle(cons_bar), bundle(prim_bar), *dims(prim),
                                               float(gamma), int(bool(accumulate)), _stream(stream)))
    return prim_bar


class Adjoint:
    """Checkpointed time-loop adjoint (eulr_adjoint_*): forward from prim0,
    backward from dJ/d(final prim) to dJ/d prim0."""

    def __init__(self, n0, n1, n2, nsteps, gamma=1.4, dx=None, cfl=0.4, checkpoint_every=20, stream=None):
        self.shape = (n0, n1, n2)
        if dx is None:
            dx = (1.0 / (n0 - 2), 1.0 / (n1 - 2), 1.0 / (n2 - 2))
        self.dx = tuple(float(v) for v in dx)
        self.gamma = float(gamma)
        self.nsteps = int(nsteps)
        h = ctypes.c_void_p()
        s = ctypes.c_void_p(stream.cuda_stream) if stream is not None else ctypes.c_void_p(None)
        check(load().eulr_adjoint_create(n0, n1, n2, self.gamma, *self.dx, float(cfl), self.nsteps,
                                         int(checkpoint_every), s, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().eulr_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, prim0, dts=None, out=None):
        """Runs the forward pass; dts fixes every step's dt (else CFL steps).
        Writes the final prim into out (a bundle) when given."""
        arr = None
        if dts is not None:
            if len(dts) != self.nsteps:
                raise ValueError(f"need {self.nsteps} step lengths, got {len(dts)}")
            arr = (ctypes.c_double * self.nsteps)(*[float(v) for v in dts])
        check(load().eulr_adjoint_forward(self._h, bundle(prim0), arr,
                                          bundle(out) if out is not None else null_bundle()))
        return out

    def dts(self):
        arr = (ctypes.c_double * max(self.nsteps, 1))()
        check(load().eulr_adjoint_dts(self._h, arr))
        return [arr[i] for i in range(self.nsteps)]

    def backward(self, prim_final_bar, out):
        check(load().eulr_adjoint_backward(self._h, bundle(prim_final_bar), bundle(out)))
        return out

    def timing(self):
        f, r, v = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(load().eulr_adjoint_timing(self._h, ctypes.byref(f), ctypes.byref(r), ctypes.byref(v)))
        return {"forward_ms": f.value, "recompute_ms": r.value, "reverse_ms": v.value}


def fma_rate(kind: str = "f64", iters: int = 20000) -> float:
    """Measured FMA throughput in FLOP/s (FMA = 2 FLOP) of the FP64 or FP32 pipe."""
    out = ctypes.c_double()
    check(load().eulr_probe_fma_rate(0 if kind == "f64" else 1, int(iters), ctypes.byref(out)))
    return out.value
