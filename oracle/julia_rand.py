"""Julia's `rand(MersenneTwister(seed), dims...)` Float64 stream -- TEST INFRASTRUCTURE ONLY.

The reference's "noisy spheres" count test (test/runtests.jl:152-172) adds
`sigma*rand(Random.MersenneTwister(0), 21, 21, 21)` to a distance field.  The
reference's CI runs Julia 1.9 (.github/workflows/CI.yml:13, Project.toml
`julia = "1.9"`), whose MersenneTwister is dSFMT-19937 (Saito & Matsumoto,
"SIMD-oriented Fast Mersenne Twister", dSFMT v2.2, the double-precision
variant; its published parameter set for MEXP 19937 is used below).  This
module restates, in plain Python integers:

* Julia 1.9 seeding: `seed!(r, n::Integer)` turns n into its little-endian
  UInt32 words (`Random.make_seed`: 0 -> UInt32[0]) and calls dSFMT's
  `dsfmt_init_by_array` on them (Random/src/RNGs.jl of Julia 1.9).  Julia 1.11
  and later hash integer seeds with SHA-256 first, so their stream differs;
  the reference's KAT is pinned to the 1.9 stream.
* dSFMT's state initialisation (init_by_array: the 0x8b fill, the two mixing
  passes with (x ^ x>>27) * 1664525 and * 1566083941, the mantissa mask to
  [1, 2), period certification) and its recursion (do_recursion with the
  128-bit "lung" word).
* Julia's `rand!(::MersenneTwister, ::Array{Float64})`: for n > 383 values
  the first (n-2)//2*2 come from dsfmt_fill_array_close_open, the rest from
  the scalar cache refilled by dsfmt_fill_array_close1_open2; both continue
  one dSFMT sequence, so the array is the sequence's first n values, each
  `x - 1.0` for x in [1, 2), in column-major order.

Only the tests import this module.
"""
import numpy as np

M64 = (1 << 64) - 1
M32 = (1 << 32) - 1

# dSFMT-params19937.h (MEXP 19937)
N = (19937 - 128) // 104 + 1      # 191 128-bit words of state (+ 1 lung word)
POS1 = 117
SL1 = 19
SR = 12
MSK1 = 0x000ffafffffffb3f
MSK2 = 0x000ffdfffc90fffd
FIX1 = 0x90014964b32f4329
FIX2 = 0x3b8d12ac548a7c7a
PCV1 = 0x3d84e1ac0dc82880
PCV2 = 0x0000000000000001
LOW_MASK = 0x000fffffffffffff
HIGH_CONST = 0x3ff0000000000000


def make_seed(n):
    """Random.make_seed(n::Integer) of Julia 1.9: little-endian UInt32 words."""
    if n < 0:
        raise ValueError('n must be non-negative')
    words = []
    while True:
        words.append(n & M32)
        n >>= 32
        if n == 0:
            return words


def _init_by_array(key):
    """dsfmt_init_by_array: returns the state as 2*(N+1) uint64 (lung last)."""
    size = (N + 1) * 4                      # 32-bit words, lung included
    lag = 11 if size >= 623 else 7 if size >= 68 else 5 if size >= 39 else 3
    mid = (size - lag) // 2
    s = [0x8b8b8b8b] * size

    def f1(x):
        return ((x ^ (x >> 27)) * 1664525) & M32

    def f2(x):
        return ((x ^ (x >> 27)) * 1566083941) & M32

    count = max(len(key) + 1, size)
    r = f1(s[0] ^ s[mid % size] ^ s[(size - 1) % size])
    s[mid % size] = (s[mid % size] + r) & M32
    r = (r + len(key)) & M32
    s[(mid + lag) % size] = (s[(mid + lag) % size] + r) & M32
    s[0] = r
    count -= 1
    i, j = 1, 0
    while j < count and j < len(key):
        r = f1(s[i] ^ s[(i + mid) % size] ^ s[(i + size - 1) % size])
        s[(i + mid) % size] = (s[(i + mid) % size] + r) & M32
        r = (r + key[j] + i) & M32
        s[(i + mid + lag) % size] = (s[(i + mid + lag) % size] + r) & M32
        s[i] = r
        i = (i + 1) % size
        j += 1
    while j < count:
        r = f1(s[i] ^ s[(i + mid) % size] ^ s[(i + size - 1) % size])
        s[(i + mid) % size] = (s[(i + mid) % size] + r) & M32
        r = (r + i) & M32
        s[(i + mid + lag) % size] = (s[(i + mid + lag) % size] + r) & M32
        s[i] = r
        i = (i + 1) % size
        j += 1
    for _ in range(size):
        r = f2((s[i] + s[(i + mid) % size] + s[(i + size - 1) % size]) & M32)
        s[(i + mid) % size] ^= r
        r = (r - i) & M32
        s[(i + mid + lag) % size] ^= r
        s[i] = r
        i = (i + 1) % size
    # 32-bit words -> 64-bit words (little endian: word 2k is the low half)
    u = [s[2 * k] | (s[2 * k + 1] << 32) for k in range(size // 2)]
    # initial_mask: the N state words (not the lung) become doubles in [1, 2)
    for k in range(2 * N):
        u[k] = (u[k] & LOW_MASK) | HIGH_CONST
    # period_certification on the lung
    t0, t1 = u[2 * N] ^ FIX1, u[2 * N + 1] ^ FIX2
    inner = (t0 & PCV1) ^ (t1 & PCV2)
    sh = 32
    while sh > 0:
        inner ^= inner >> sh
        sh >>= 1
    if (inner & 1) != 1:
        u[2 * N + 1] ^= 1
    return u


def dsfmt_doubles(seed, n):
    """The first n values of the dSFMT sequence seeded as Julia 1.9 seeds
    MersenneTwister(seed), as doubles in [1, 2)."""
    u = _init_by_array(make_seed(seed))
    hist = [(u[2 * k], u[2 * k + 1]) for k in range(N)]   # sliding window x[k-N .. k-1]
    l0, l1 = u[2 * N], u[2 * N + 1]
    out = []
    k = 0
    while len(out) < n:
        a0, a1 = hist[k]                 # x[k - N]
        b0, b1 = hist[(k + POS1) % N]    # x[k - N + POS1]
        n0 = ((a0 << SL1) & M64) ^ (l1 >> 32) ^ ((l1 << 32) & M64) ^ b0
        n1 = ((a1 << SL1) & M64) ^ (l0 >> 32) ^ ((l0 << 32) & M64) ^ b1
        l0, l1 = n0, n1
        r0 = (l0 >> SR) ^ (l0 & MSK1) ^ a0
        r1 = (l1 >> SR) ^ (l1 & MSK2) ^ a1
        hist[k] = (r0, r1)
        k = (k + 1) % N
        out.append(r0)
        out.append(r1)
    bits = np.array(out[:n], dtype=np.uint64)
    return bits.view(np.float64)


def rand_mersenne_twister(seed, *dims):
    """`rand(MersenneTwister(seed), dims...)` of Julia 1.9 (Float64, [0, 1)),
    returned as a Fortran-ordered numpy array of shape dims."""
    n = int(np.prod(dims))
    vals = dsfmt_doubles(seed, n) - 1.0
    return np.asfortranarray(vals.reshape(dims, order='F'))


def noisy_spheres(N_=10, sigma=1.0):
    """The volume of the reference's "noisy spheres" test (test/runtests.jl:158-161):
    Float32 distances sqrt(Float32(i^2+j^2+k^2)) for i, j, k in -N:N, plus
    sigma * rand(MersenneTwister(0), 2N+1, 2N+1, 2N+1); Float32 + Float64 promotes
    to a Float64 array."""
    r = np.arange(-N_, N_ + 1)
    i, j, k = np.meshgrid(r, r, r, indexing='ij')
    dist = np.sqrt((i * i + j * j + k * k).astype(np.float32))
    noise = rand_mersenne_twister(0, 2 * N_ + 1, 2 * N_ + 1, 2 * N_ + 1)
    return np.asfortranarray(dist.astype(np.float64) + sigma * noise)

