"""eulr_time_step_noalloc_f64: the CFL reduction for callers that cannot
allocate device memory (their device memory belongs to a pool or arena that
forbids hidden allocations).  Its scratch is a fixed array inside the
library's device image instead of a cudaMalloc made on first use.

Called through the C ABI and compared with eulr_time_step_f64 on the same
inputs, on two calls in a row (the second call reuses the array the first
one left behind).  time_step is bit-identical to the reference, so the
tolerance is exact equality.  This file is collected last on purpose."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _call(lib, name, torch, prim, g, dx, out):
    import euler_gb300 as E

    n2, n1, n0 = prim.shape[1:]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = getattr(lib, name)(E.bundle(prim), n0, n1, n2, g, dx[0], dx[1], dx[2], ctypes.c_void_p(out.data_ptr()),
                            stream)
    assert st == 0, lib.eulr_last_error()


def test_noalloc_time_step_matches_allocating_entry(cuda, euler, oracle_lib):
    torch = cuda
    lib = euler.load()
    cases = [((70, 40, 37), 0, (0.02, 0.03, 0.05)), ((514, 66, 9), 1, (1 / 512, 1 / 64, 1 / 7)),
             ((3, 3, 3), 2, (1.0, 1.0, 1.0))]
    for shape, seed, dx in cases:
        prim = torch.from_numpy(oracle_lib.random_prim(*shape, seed=seed)).cuda()
        ref = torch.empty((), dtype=torch.float64, device="cuda")
        got = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
        _call(lib, "eulr_time_step_f64", torch, prim, 1.4, dx, ref)
        # two calls in a row through the no-alloc entry point
        _call(lib, "eulr_time_step_noalloc_f64", torch, prim, 1.4, dx, got[0])
        _call(lib, "eulr_time_step_noalloc_f64", torch, prim, 1.4, dx, got[1])
        torch.cuda.synchronize()
        assert got[0].item() == ref.item(), shape
        assert got[1].item() == ref.item(), shape
        assert ref.item() == oracle_lib.time_step(prim.cpu().numpy(), 1.4, dx)


def test_noalloc_time_step_rejects_bad_sizes(cuda, euler):
    import euler_gb300 as E

    lib = euler.load()
    ok = E.Bundle5(8, 16, 24, 32, 40)
    assert lib.eulr_time_step_noalloc_f64(ok, 2000, 2000, 2000, 1.4, 0.1, 0.1, 0.1, 4096, None) == -6
    assert lib.eulr_time_step_noalloc_f64(ok, 0, 4, 4, 1.4, 0.1, 0.1, 0.1, 4096, None) == -1
