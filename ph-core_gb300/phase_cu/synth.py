"""Seeded synthetic inputs (SplitMix64), identical bytes for every consumer.

SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014): state += 0x9E3779B97F4A7C15; z = state;
z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9; z = (z ^ (z >> 27)) * 0x94D049BB133111EB;
return z ^ (z >> 31).  Uniforms take the top 53 bits; normals use Box-Muller.
Vectorised with numpy uint64 arithmetic (wrapping).
"""
import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, n, start=0):
    """The n outputs number start..start+n-1 of the SplitMix64 stream seeded with `seed`."""
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed, n, start=0):
    """Doubles in [0, 1) from the top 53 bits."""
    return (splitmix64(seed, n, start) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform_f32(shape, seed=0, lo=-1.0, hi=1.0, start=0):
    n = int(np.prod(shape)) if len(shape) else 0
    u = uniform01(seed, n, start)
    return (lo + (hi - lo) * u).astype(np.float32).reshape(shape)


def uniform_i32(shape, seed=0, lo=-1000, hi=1000, start=0):
    """Integers uniform in [lo, hi] (inclusive)."""
    n = int(np.prod(shape)) if len(shape) else 0
    span = np.uint64(hi - lo + 1)
    z = splitmix64(seed, n, start)
    return (np.int64(lo) + (z % span).astype(np.int64)).astype(np.int32).reshape(shape)


def normal_f64(n, seed=0, start=0):
    """Box-Muller normals from consecutive uniform pairs."""
    m = (n + 1) // 2
    u1 = uniform01(seed, m, start)
    u2 = uniform01(seed, m, start + m)
    u1 = np.maximum(u1, 1e-300)
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
    return z[:n]


def lognormal_f32(shape, seed=0, mu=0.0, sigma=1.0, start=0):
    n = int(np.prod(shape)) if len(shape) else 0
    return np.exp(mu + sigma * normal_f64(n, seed, start)).astype(np.float32).reshape(shape)


def gaussian_bumps_f32(n, m, bumps=16, seed=0, wmin=20.0, wmax=200.0):
    """Heat-equation initial field: sum of `bumps` Gaussians A=1 with seeded
    centres in [0, n) x [0, m) and widths in [wmin, wmax], computed in FP64,
    rounded to FP32, boundary rows and columns set to zero."""
    z = splitmix64(seed, 3 * bumps)
    ci = (z[0::3] % np.uint64(n)).astype(np.float64)
    cj = (z[1::3] % np.uint64(m)).astype(np.float64)
    w = wmin + (wmax - wmin) * ((z[2::3] >> np.uint64(11)).astype(np.float64) / 9007199254740992.0)
    ii = np.arange(n, dtype=np.float64)[:, None]
    jj = np.arange(m, dtype=np.float64)[None, :]
    u = np.zeros((n, m), dtype=np.float64)
    for b in range(bumps):
        u += np.exp(-((ii - ci[b]) ** 2 + (jj - cj[b]) ** 2) / (2.0 * w[b] * w[b]))
    u[0, :] = 0
    u[-1, :] = 0
    u[:, 0] = 0
    u[:, -1] = 0
    return u.astype(np.float32)
