"""Face states for the drop-in HLLC tests: seeded random states (rho and p
log-uniform on [0.1, 10], velocities N(0, 1)), supersonic faces both ways,
gas at rest with equal pressures (ustar exactly 0), signed zeros, equal
states, strong pressure jumps and a spread of gamma."""
import numpy as np


def face_states(n_random=3000, seed=7, dtype=np.float64):
    rng = np.random.Generator(np.random.PCG64(seed))

    def rand(n):
        q = np.empty((n, 5))
        q[:, 0] = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))
        q[:, 1] = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))
        q[:, 2:] = rng.normal(size=(n, 3))
        return q

    qL, qR = [rand(n_random)], [rand(n_random)]
    m = 200
    # supersonic to the right and to the left
    for s in (8.0, -8.0):
        a, b = rand(m), rand(m)
        a[:, 2:] += s
        b[:, 2:] += s
        qL.append(a)
        qR.append(b)
    # gas at rest, equal pressures, different densities: ustar == 0 exactly
    a, b = rand(m), rand(m)
    a[:, 2:] = 0.0
    b[:, 2:] = 0.0
    b[:, 1] = a[:, 1]
    qL.append(a)
    qR.append(b)
    # signed zeros in the velocities
    a, b = rand(m), rand(m)
    a[:, 2:] = 0.0
    b[:, 2:] = -0.0
    qL.append(a)
    qR.append(b)
    # identical states
    a = rand(m)
    qL.append(a)
    qR.append(a.copy())
    # strong pressure jumps
    a, b = rand(m), rand(m)
    a[:, 1] *= 1e4
    b[:, 1] *= 1e-4
    qL.append(a)
    qR.append(b)
    qL = np.concatenate(qL).astype(dtype)
    qR = np.concatenate(qR).astype(dtype)
    n = qL.shape[0]
    dirs = rng.integers(0, 3, n).astype(np.int32)
    gamma = rng.uniform(1.1, 1.67, n).astype(dtype)
    gamma[: n // 2] = dtype(1.4)
    return dirs, gamma, qL, qR


def write_faces(path, dirs, gamma, qL, qR):
    with open(path, "wb") as f:
        f.write(np.int64(len(dirs)).tobytes())
        f.write(np.ascontiguousarray(dirs, dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(gamma).tobytes())
        f.write(np.ascontiguousarray(qL).tobytes())
        f.write(np.ascontiguousarray(qR).tobytes())


def read_fluxes(path, n, dtype):
    return np.fromfile(path, dtype=dtype).reshape(n, 5)


def oracle_fluxes(O, dirs, gamma, qL, qR, impl="port"):
    out = np.empty_like(qL)
    for d in range(3):
        for g in np.unique(gamma):
            sel = (dirs == d) & (gamma == g)
            if sel.any():
                out[sel] = O.hllc_faces(d, float(g), qL[sel], qR[sel], impl=impl)
    return out
