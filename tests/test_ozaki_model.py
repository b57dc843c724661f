"""A NumPy model of the sliced (Ozaki) arithmetic of the tcgen05 GEMM kernel
(mbsymmetry_gb300/csrc/kernels_oz.cu), checking the error analysis its design
rests on, on the CPU:

* four fixed-point slices per value (s0 with |s0| <= 128, s1..s3 of 8 bits
  below it) are exact in BF16 and reproduce the value to 2^-31 of the row's
  scale 2^E;
* the class sums D0 (s0 t0) and D1 (s0 t1 + s1 t0) of one round of 16 complex
  K (32 real products) are exact in FP32;
* the product of two rows from the classes 0-3 differs from the exact product
  by less than K 2^-29 of (row scale x column scale).

The model mirrors the kernel's operations (round to nearest integer of the
scaled value, the two-sum of the remainder with the low word, slices times
2^-8i) in float32 with NumPy, and compares with exact rational / float64
arithmetic."""
import numpy as np


def exponent(m):
    """E with |x| < 2^E for |x| <= m (frexp: m = f 2^e, f in [0.5, 1))."""
    return np.frexp(np.float32(m))[1] if m > 0 else -100


def slices(hi, lo, E):
    """The kernel's four slices (s0, s1 2^-8, s2 2^-16, s3 2^-24) of hi + lo."""
    f = np.float32(2.0 ** (7 - E))
    h, l = np.float32(hi) * f, np.float32(lo) * f
    s0 = np.rint(h).astype(np.float32)
    r = np.float32(h - s0)
    rh = np.float32(r + l)
    bb = np.float32(rh - r)
    rl = np.float32((r - np.float32(rh - bb)) + np.float32(l - bb))
    t1 = np.float32(rh * np.float32(256.0))
    s1 = np.rint(t1).astype(np.float32)
    t2 = np.float32(np.float32(np.float32(t1 - s1) + np.float32(rl * np.float32(256.0))) * np.float32(256.0))
    s2 = np.rint(t2).astype(np.float32)
    s3 = np.rint(np.float32(np.float32(t2 - s2) * np.float32(256.0))).astype(np.float32)
    return s0, s1 * np.float32(2.0 ** -8), s2 * np.float32(2.0 ** -16), s3 * np.float32(2.0 ** -24)


def is_bf16(x):
    """Exactly representable in BF16: at most 8 significant bits."""
    x = np.asarray(x, dtype=np.float32)
    return np.array_equal(x, (x.view(np.uint32) & np.uint32(0xFFFF0000)).view(np.float32))


def ff(x):
    """float-float split of float64 values: (hi, lo) float32."""
    hi = x.astype(np.float32)
    return hi, (x - hi.astype(np.float64)).astype(np.float32)


def test_slices_are_bf16_and_reproduce_the_value():
    rng = np.random.default_rng(1)
    for _ in range(200):
        x = rng.standard_normal(16) * 10.0 ** rng.uniform(-6, 6, size=16)  # wide dynamic range in a round
        hi, lo = ff(x)
        E = exponent(np.abs(hi).max())
        s = slices(hi, lo, E)
        assert all(is_bf16(si) for si in s)
        assert np.abs(s[0]).max() <= 128 and all(np.abs(si).max() <= 128.0 * 2.0 ** (-8 * i)
                                                  for i, si in enumerate(s) if i)
        back = sum(si.astype(np.float64) for si in s) * 2.0 ** (E - 7)
        assert np.abs(back - (hi.astype(np.float64) + lo)).max() <= 2.0 ** (E - 31)


def test_class_sums_of_a_round_are_exact_in_fp32():
    rng = np.random.default_rng(2)
    for _ in range(200):
        a, b = rng.standard_normal(32), rng.standard_normal(32)  # 16 complex = 32 real per round
        ea, eb = exponent(np.abs(a).max()), exponent(np.abs(b).max())
        sa, sb = slices(*ff(a), ea), slices(*ff(b), eb)
        d0 = np.float32(0)
        d1 = np.float32(0)
        for k in range(32):  # FP32 accumulation in the kernel's order
            d0 = np.float32(d0 + np.float32(sa[0][k] * sb[0][k]))
            d1 = np.float32(d1 + np.float32(sa[0][k] * sb[1][k]))
            d1 = np.float32(d1 + np.float32(sa[1][k] * sb[0][k]))
        exact0 = sum(float(sa[0][k]) * float(sb[0][k]) for k in range(32))
        exact1 = sum(float(sa[0][k]) * float(sb[1][k]) + float(sa[1][k]) * float(sb[0][k]) for k in range(32))
        assert float(d0) == exact0 and float(d1) == exact1


def test_row_product_error_bound():
    """Classes 0-3 of the slice products: |sum - exact| < K 2^-29 2^(Ea + Eb)."""
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(200):
        K = 32
        a = rng.standard_normal(K) * 10.0 ** rng.uniform(-3, 3, size=K)
        b = rng.standard_normal(K) * 10.0 ** rng.uniform(-3, 3, size=K)
        ah, al = ff(a)
        bh, bl = ff(b)
        ea, eb = exponent(np.abs(ah).max()), exponent(np.abs(bh).max())
        sa, sb = slices(ah, al, ea), slices(bh, bl, eb)
        approx = sum(float(np.dot(sa[i].astype(np.float64), sb[j].astype(np.float64)))
                     for i in range(4) for j in range(4) if i + j <= 3) * 2.0 ** (ea + eb - 14)
        exact = float(np.dot(ah.astype(np.float64) + al, bh.astype(np.float64) + bl))
        err = abs(approx - exact) / 2.0 ** (ea + eb)
        worst = max(worst, err)
        assert err < K * 2.0 ** -29
    print(f"worst error / (row scale x column scale): {worst:.2e} (bound {32 * 2.0 ** -29:.2e})")
