"""The arithmetic of the tensor-core setup (pfcsieve_gb300/csrc/setup_tc.cu),
emulated on the CPU with numpy: fp16 byte planes, fp32 sums of 112 products
behind a 2^23 bias read back from their bits, the word's fold T assembled from
the planes, and the one-round reduction.  Checks the bounds the kernel relies
on (every partial sum an integer below 2^24, T < 2^79 for class 64 and
< 2^47 for class 32, u < 2^48 + p) and that u = Z (mod p) for the folded word
Z, on random and extreme inputs.  The kernel's results equal the integer-pipe
setup's on the GPU (tests/test_gpu_parity.py); this pins the formulation."""
import numpy as np

BYTES = 224          # a 1792-bit word
HALF = BYTES // 2    # bytes summed into one fp32 accumulator
K = 16               # bytes per MMA step
BIAS = 2048 * 4096   # the bias MMA's product, 2^23


def positions(p, planes):
    """w_b = 2^(8 b + 32) mod p as byte planes W[a][b]."""
    w = [pow(2, 8 * b + 32, p) for b in range(BYTES)]
    W = np.array([[(x >> (8 * a)) & 0xFF for x in w] for a in range(planes)], dtype=np.float16)
    return w, W


def fold(zbytes, W):
    """fp32 sums D[a][h] = 2^23 + sum over half h of z_b W_a[b], accumulated in
    K-byte steps as the MMAs do, read back as 0x4B000000 + integer."""
    z = np.asarray(zbytes, dtype=np.float16)
    assert np.array_equal(z.astype(np.int64), np.asarray(zbytes))   # bytes are exact in fp16
    T = 0
    for a in range(W.shape[0]):
        halves = []
        for h in range(2):
            acc = np.float32(BIAS)
            for k0 in range(h * HALF, (h + 1) * HALF, K):
                acc = np.float32(acc + np.dot(z[k0:k0 + K].astype(np.float32), W[a, k0:k0 + K].astype(np.float32)))
            bits = int(np.array([acc], dtype=np.float32).view(np.uint32)[0])
            assert 0x4B000000 <= bits < 0x4B800000        # an integer in [2^23, 2^24): exact
            halves.append(bits - 0x4B000000 + BIAS)
        T += (halves[0] + halves[1] - 2 * BIAS) << (8 * a)
    return T


def reduce_round(T, p):
    """u = (T + m p) / 2^32, m = -T p^-1 mod 2^32: u = T 2^-32 (mod p)."""
    m = (-T * pow(p, -1, 2**32)) % 2**32
    assert (T + m * p) % 2**32 == 0
    return (T + m * p) >> 32


def check(p, planes, zbytes, w):
    _, W = positions(p, planes)
    T = fold(zbytes, W)
    assert T == sum(z * x for z, x in zip(zbytes, w))           # the exact contraction
    Z = sum(z << (8 * b) for b, z in enumerate(zbytes))
    assert T % p == (Z << 32) % p
    return T, Z


def test_class64_fold_and_reduction():
    rng = np.random.default_rng(0)
    lazy_end = 0x5555555555555556
    ps = [2**31 + 11, 2**40 + 15, 2**62 + 135, lazy_end - 3] + [int(x) | 1 for x in rng.integers(2**31, 2**62, 4)]
    for p in ps:
        w, _ = positions(p, 8)
        for zb in (rng.integers(0, 256, BYTES).tolist(), [255] * BYTES, [0] * BYTES):
            T, Z = check(p, 8, zb, w)
            assert T < 2**79
            u = reduce_round(T, p)
            assert u % p == Z % p and u < 2**48 + p


def test_class32_fold_and_reduction():
    rng = np.random.default_rng(1)
    ps = [3, 1000003, 2**31 - 1] + [int(x) | 1 for x in rng.integers(5, 2**31, 4)]
    for p in ps:
        w, _ = positions(p, 4)
        assert max(w) < 2**31
        for zb in (rng.integers(0, 256, BYTES).tolist(), [255] * BYTES):
            T, Z = check(p, 4, zb, w)
            assert T < 2**47
            # one 32-bit round on the high and low words: u = hi(T) - hi(m p) (+ p)
            m = (T * pow(p, -1, 2**32)) % 2**32
            u = (T >> 32) - ((m * p) >> 32)
            u = u + p if u < 0 else u
            assert 0 <= u < p + 2**15 and (u - (Z % p)) % p == 0


def test_fp16_byte_conversion():
    """A byte v becomes the fp16 v exactly as the fp16 of 1024 + v (bits 0x6400 | v)
    less 1024, the conversion the tile packing uses."""
    v = np.arange(256, dtype=np.uint16)
    x = (0x6400 | v).view(np.float16)
    assert np.array_equal((x - np.float16(1024)).astype(np.int64), v.astype(np.int64))
