"""Seeded synthetic inputs for the benchmark configurations.

A counter-based generator (splitmix64 finaliser over seed + i * golden gamma,
then 53-bit uniforms and Box-Muller normals) so that the same seed gives the
same float64 inputs on any machine, without numpy's generator versions.
"""
import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
BASE_SEED = 0x6B3A2026


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def uniform(seed, n, offset=0):
    """n uniforms in [0, 1) for stream `seed`, starting at counter `offset`."""
    with np.errstate(over="ignore"):
        i = np.arange(offset, offset + n, dtype=np.uint64)
        z = np.uint64(seed) * _GAMMA + (i + np.uint64(1)) * _GAMMA
        return (_mix(z) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform_pm1(seed, n):
    """i.i.d. uniform[-1, 1)."""
    return 2.0 * uniform(seed, n) - 1.0


def normal(seed, n):
    """i.i.d. N(0, 1) by Box-Muller on pairs of uniforms.  Large arrays are
    generated in chunks of pairs on several threads (numpy releases the GIL in
    its element-wise kernels); every pair depends on its counter alone."""
    m = (n + 1) // 2
    out = np.empty(2 * m)

    def pairs(a, b):
        u1 = uniform(seed, b - a, a)
        u2 = uniform(seed, b - a, m + a)
        r = np.sqrt(-2.0 * np.log1p(-u1))  # 1-u1 in (0, 1]
        t = 2.0 * np.pi * u2
        out[2 * a:2 * b:2] = r * np.cos(t)
        out[2 * a + 1:2 * b:2] = r * np.sin(t)

    chunk = 1 << 21
    if m <= chunk:
        pairs(0, m)
    else:
        import concurrent.futures as cf
        import os
        with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
            list(ex.map(lambda a: pairs(a, min(m, a + chunk)), range(0, m, chunk)))
    return out[:n]


def four1_c1(seed=BASE_SEED):
    """four1 N=4096 complex, re/im uniform[-1,1)."""
    return uniform_pm1(seed, 2 * 4096)


def convlv_c2(n=1 << 20, m=257, seed=BASE_SEED + 1):
    """Real N(0,1) signal of n samples and an m-tap response (Gaussian window,
    sigma = m/6, times N(0,1)) in wrap-around order inside a length-n buffer."""
    x = normal(seed, n)
    half = (m - 1) // 2
    lags = np.arange(-half, half + 1)
    taps = np.exp(-0.5 * (lags / (m / 6.0)) ** 2) * normal(seed + 1000, m)
    r = np.zeros(n)
    r[lags % n] = taps
    return x, r


def batch_c3(count=20000, kmin=6, kmax=14, seed=BASE_SEED + 2):
    """Sizes 2^k, k uniform in [kmin, kmax]; complex N(0,1) * 10^u, u~U[-3,3]."""
    k = kmin + np.floor(uniform(seed, count) * (kmax - kmin + 1)).astype(np.int64)
    k = np.minimum(k, kmax)
    u = -3.0 + 6.0 * uniform(seed + 1, count)
    sizes = (1 << k).astype(np.int64)
    return sizes, u


def batch_c3_data(sizes, u, seed=BASE_SEED + 3):
    out = []
    for t, (nn, ut) in enumerate(zip(sizes, u)):
        out.append(normal(seed * 1000003 + t, 2 * int(nn)) * (10.0 ** ut))
    return out


def plane_waves(shape, count=32, seed=BASE_SEED + 4):
    """uniform[-1,1) plus a seeded sum of `count` unit plane waves with integer
    wave vectors and random phases (real field of the given shape)."""
    n = int(np.prod(shape))
    x = uniform_pm1(seed, n).reshape(shape)
    kv = np.floor(uniform(seed + 1, count * len(shape)).reshape(count, len(shape)) *
                  np.array(shape)).astype(np.int64)
    ph = 2 * np.pi * uniform(seed + 2, count)
    grids = np.meshgrid(*[np.arange(s) / s for s in shape], indexing="ij")
    for c in range(count):
        arg = sum(kv[c, d] * grids[d] for d in range(len(shape)))
        x = x + np.cos(2 * np.pi * arg + ph[c])
    return x


def plane_waves_torch(shape, device, seed=BASE_SEED + 4, count=32):
    """The same construction as plane_waves (uniform[-1,1) plus `count` unit
    plane waves with integer wave vectors and random phases), generated on a
    torch device with torch's seeded generator: fast enough for the 512^3
    fields of the 3-D configurations."""
    import math
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    x = torch.rand(shape, generator=g, device=device, dtype=torch.float64) * 2 - 1
    kv = (torch.rand((count, len(shape)), generator=g, device=device, dtype=torch.float64) *
          torch.tensor(shape, device=device, dtype=torch.float64)).floor()
    ph = 2 * math.pi * torch.rand(count, generator=g, device=device, dtype=torch.float64)
    grids = [torch.arange(s, device=device, dtype=torch.float64) / s for s in shape]
    for c in range(count):
        arg = None
        for d in range(len(shape)):
            view = [1] * len(shape)
            view[d] = shape[d]
            term = (kv[c, d] * grids[d]).reshape(view)
            arg = term if arg is None else arg + term
        x += torch.cos(2 * math.pi * arg + ph[c])
    return x.contiguous()
