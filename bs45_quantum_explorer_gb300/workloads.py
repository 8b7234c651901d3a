"""Seeded synthetic inputs with the shapes of the reference's own workloads.

No public dataset is involved: the reference measures on streams its own DFS produces.
The Hall microbench generator is defined per pair index, so the device generator
(bs_gen_hall_pairs_dev in libbsfh.so), the oracle's C generator and the small numpy form
below produce bit-identical words from the same seed:

  mix(z)      = splitmix64 finaliser; sm(s, k) = mix(s + (k+1) * 0x9E3779B97F4A7C15)
  pair p < npairs/2 (i.i.d. half):  C = sm(seed, 2p) & mask, D = sm(seed, 2p+1) & mask
  pair p >= npairs/2 (mirror half, n even): attempt t = 0, 1, ... draws
      r = sm(seed ^ 0xA5A5A5A5A5A5A5A5, (p << 20) + t); bits 0..3 pick the depth-0 quad from
      the 16 quads, then 3 bits per depth d = 1..n/2-1 pick a positive-product quad; the
      attempt is kept when sum C = sum D = 0 (rejection sampling). n/2-1 <= 20 (n <= 42).
"""
import numpy as np

GOLDEN = 0x9E3779B97F4A7C15
MIRROR_SALT = 0xA5A5A5A5A5A5A5A5
M64 = (1 << 64) - 1


def mix64(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def sm(seed, k):
    return mix64((seed + (k + 1) * GOLDEN) & M64)


def quad_tables():
    """The Thm 2.2 quad tables in the reference's order (wz_match.cpp:534-545)."""
    allq, pos, neg = [], [], []
    for i in range(16):
        v = [1 if i & 8 else -1, 1 if i & 4 else -1, 1 if i & 2 else -1, 1 if i & 1 else -1]
        allq.append(v)
        (pos if v[0] * v[1] * v[2] * v[3] == 1 else neg).append(v)
    return allq, pos, neg


def mirror_attempt(n, r):
    """One mirror-rule attempt from the 64 random bits r -> (Cword, Dword)."""
    allq, pos, _ = quad_tables()
    C = [0] * n
    D = [0] * n
    bits = r
    for d in range(n // 2):
        if d == 0:
            q = allq[bits & 15]
            bits >>= 4
        else:
            q = pos[bits & 7]
            bits >>= 3
        C[d], D[d], C[n - 1 - d], D[n - 1 - d] = q
    cw = sum(1 << i for i in range(n) if C[i] == 1)
    dw = sum(1 << i for i in range(n) if D[i] == 1)
    return cw, dw, sum(C), sum(D)


def hall_microbench_pairs_py(n, npairs, seed=0xB545C2, first=0, count=None):
    """Pure-Python form of the generator for pairs [first, first+count) (small counts)."""
    count = npairs - first if count is None else count
    half = npairs // 2
    mask = (1 << n) - 1
    out = np.zeros((count, 2), np.uint64)
    for t, p in enumerate(range(first, first + count)):
        if p < half or n % 2 or n > 42:
            out[t] = (sm(seed, 2 * p) & mask, sm(seed, 2 * p + 1) & mask)
            continue
        a = 0
        while True:
            cw, dw, sc, sd = mirror_attempt(n, sm(seed ^ MIRROR_SALT, (p << 20) + a))
            a += 1
            if sc == 0 and sd == 0:
                out[t] = (cw, dw)
                break
    return out


def unpack_pairs(words, n):
    """uint64 [npairs, 2] -> int8 [npairs, 2, n]."""
    w = np.asarray(words, np.uint64)
    bits = (w[..., None] >> np.arange(n, dtype=np.uint64)) & np.uint64(1)
    return np.where(bits == 1, 1, -1).astype(np.int8)
