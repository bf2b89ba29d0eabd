"""The oracle's FP32 noise against an independent restatement of the published
algorithms in numpy float32 arithmetic (one rounding per operation, like the oracle):
splitmix64 (Steele, Lea, Flood 2014), a Fisher-Yates shuffle of 0..255 driven by it, and
Perlin's improved noise (SIGGRAPH 2002) with his branching gradient function. The
oracle's gradient is the dot product with Perlin's coefficient vector, which gives the
same value except for the sign of an exact zero, so values are compared with ==
(-0 == +0) and nonzero values bit for bit."""
import ctypes

import numpy as np
import pytest

F = np.float32
M64 = (1 << 64) - 1


def splitmix64(state):
    state = (state + 0x9E3779B97F4A7C15) & M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return state, z ^ (z >> 31)


def permutation(seed):
    perm = list(range(256))
    s = seed
    for i in range(255, 0, -1):
        s, r = splitmix64(s)
        j = r % (i + 1)
        perm[i], perm[j] = perm[j], perm[i]
    return perm + perm


def fade(t):
    return t * t * t * (t * (t * F(6) - F(15)) + F(10))


def lerp(t, a, b):
    return a + t * (b - a)


def grad(h, x, y, z):
    h &= 15
    u = x if h < 8 else y
    v = y if h < 4 else (x if h in (12, 14) else z)
    return (u if (h & 1) == 0 else -u) + (v if (h & 2) == 0 else -v)


def noise3(p, x, y, z):
    fx, fy, fz = F(np.floor(x)), F(np.floor(y)), F(np.floor(z))
    X, Y, Z = int(fx) & 255, int(fy) & 255, int(fz) & 255
    x, y, z = x - fx, y - fy, z - fz
    u, v, w = fade(x), fade(y), fade(z)
    A = p[X] + Y
    AA, AB = p[A] + Z, p[A + 1] + Z
    B = p[X + 1] + Y
    BA, BB = p[B] + Z, p[B + 1] + Z
    one = F(1)
    return lerp(w,
                lerp(v, lerp(u, grad(p[AA], x, y, z), grad(p[BA], x - one, y, z)),
                     lerp(u, grad(p[AB], x, y - one, z), grad(p[BB], x - one, y - one, z))),
                lerp(v, lerp(u, grad(p[AA + 1], x, y, z - one), grad(p[BA + 1], x - one, y, z - one)),
                     lerp(u, grad(p[AB + 1], x, y - one, z - one),
                          grad(p[BB + 1], x - one, y - one, z - one))))


def noise2(p, x, y):
    return noise3(p, x, y, F(0))  # the z = 0 slice


def fbm(noise, p, coords, octaves, freq, lac, gain):
    s, amp, f = F(0), F(1), F(freq)
    for _ in range(octaves):
        s = s + amp * noise(p, *[c * f for c in coords])
        f = f * F(lac)
        amp = amp * F(gain)
    return s


def same(a, b):
    a, b = F(a), F(b)
    if a == 0 and b == 0:
        return True
    return a.view(np.uint32) == b.view(np.uint32)


@pytest.mark.parametrize("seed", [0, 1, 7, 42, 1234, 2 ** 63 + 5])
def test_permutation(oracle, seed):
    assert oracle.perm(seed).tolist() == permutation(seed)


@pytest.fixture(scope="module")
def lib(oracle):
    L = oracle.load()
    L.or_fbm2_f32.restype = ctypes.c_float
    L.or_fbm2_f32.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                              ctypes.c_float, ctypes.c_float, ctypes.c_float]
    L.or_fbm3_f32.restype = ctypes.c_float
    L.or_fbm3_f32.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                              ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    return L


def points(rng, k, dim):
    # lattice points, small and large magnitudes, negative coordinates
    pts = rng.uniform(-300.0, 300.0, (k, dim)).astype(np.float32)
    pts[: k // 8] = np.round(pts[: k // 8])
    pts[k // 8: k // 4] *= np.float32(1e-3)
    return pts


def test_noise3_and_noise2(oracle, lib):
    rng = np.random.default_rng(7)
    for seed in (1234, 7):
        pp = oracle.perm(seed)
        p = permutation(seed)
        buf = np.ascontiguousarray(pp, np.uint8)
        for x, y, z in points(rng, 300, 3):
            got = lib.or_noise3_f32(buf.ctypes.data, float(x), float(y), float(z))
            assert same(got, noise3(p, x, y, z)), (seed, x, y, z)
        for x, y in points(rng, 300, 2):
            got = lib.or_noise2_f32(buf.ctypes.data, float(x), float(y))
            assert same(got, noise2(p, x, y)), (seed, x, y)


@pytest.mark.parametrize("octaves,freq,lac,gain", [(4, 1 / 128, 2.0, 0.5), (3, 1 / 96, 2.0, 0.5),
                                                   (3, 0.09, 0.5, 2.5), (1, 1 / 64, 2.0, 0.5)])
def test_fbm(oracle, lib, octaves, freq, lac, gain):
    rng = np.random.default_rng(octaves)
    pp = np.ascontiguousarray(oracle.perm(42), np.uint8)
    p = permutation(42)
    for x, y, z in points(rng, 100, 3):
        got3 = lib.or_fbm3_f32(pp.ctypes.data, float(x), float(y), float(z), octaves, freq, lac, gain)
        assert same(got3, fbm(noise3, p, (x, y, z), octaves, freq, lac, gain))
        got2 = lib.or_fbm2_f32(pp.ctypes.data, float(x), float(z), octaves, freq, lac, gain)
        assert same(got2, fbm(noise2, p, (x, z), octaves, freq, lac, gain))
