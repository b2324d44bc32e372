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


_FRESH_PROCESS = r'''
import sys
sys.path[:0] = [{root!r}, {pkg!r}]
import ctypes
import torch
import euler_gb300 as E

lib = E.load()
torch.cuda.set_device(0)
n0, n1, n2 = 70, 40, 37
g = torch.Generator(device="cuda")
g.manual_seed(3)
prim = torch.rand((5, n2, n1, n0), dtype=torch.float64, device="cuda", generator=g) + 0.5
out = torch.zeros(8, dtype=torch.float64, device="cuda")
stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
b = E.bundle(prim)


def call(name, k):
    st = getattr(lib, name)(b, n0, n1, n2, 1.4, 0.02, 0.03, 0.05, ctypes.c_void_p(out[k].data_ptr()), stream)
    assert st == 0, lib.eulr_last_error()
    torch.cuda.synchronize()


# first call on the device: looks up the fixed array's device address (and
# loads the library's kernel if nothing has yet)
call("eulr_time_step_noalloc_f64", 0)
free0 = torch.cuda.mem_get_info()[0]
for k in range(1, 4):
    call("eulr_time_step_noalloc_f64", k)
free1 = torch.cuda.mem_get_info()[0]
# control: the allocating entry point takes its scratch from cudaMalloc on
# its first call in this process, which the same measurement sees
call("eulr_time_step_f64", 4)
free2 = torch.cuda.mem_get_info()[0]
vals = out[:5].tolist()
print(free0, free1, free2, *[float(v).hex() for v in vals])
'''


def test_noalloc_time_step_allocates_nothing(cuda, euler):
    """In a fresh process that has made no other library call: after the
    first call on the device, further calls of the no-alloc entry point leave
    the device's free memory (cudaMemGetInfo) unchanged, and the allocating
    eulr_time_step_f64, called afterwards, still has to allocate its scratch
    then -- so the no-alloc calls did not create it either.  All five results
    are equal."""
    import subprocess
    import sys

    from conftest import PKG_DIR, ROOT

    r = subprocess.run([sys.executable, "-c", _FRESH_PROCESS.format(root=ROOT, pkg=PKG_DIR)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    fields = r.stdout.strip().splitlines()[-1].split()
    free0, free1, free2 = (int(v) for v in fields[:3])
    dts = fields[3:]
    assert free1 == free0, (free0, free1)
    assert free2 < free1, (free1, free2)
    assert len(set(dts)) == 1, dts
