"""The contraction's split-precision schemes emulated in numpy on a seeded Gram
problem, against FP64: the FP16x3 split the tensor-core kernel runs (row
scales, an integer leading plane of 8 bits and two FP16 planes, the six
products with plane(A) + plane(B) <= 2, the integer products summed exactly,
the five corrections in FP32) and the TF32-compensated form (hi + lo TF32
terms, hi.hi + hi.lo + lo.hi summed in FP32), which is not built.

The tf32 kind runs at half the FP16 rate, so its three products take the
tensor time of FP16x3's six; this test measures what they buy.  Both
emulations round to nearest in every FP32 sum (the tensor core's
accumulation is no better), so the gap is a lower bound."""
import numpy as np


def _tf32(x):
    """Round float32 values to TF32 (10 explicit mantissa bits), to nearest even."""
    b = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    lsb = (b >> 13) & 1
    b = ((b + 0xFFF + lsb) >> 13) << 13
    return b.astype(np.uint32).view(np.float32)


def _gram_tf32c(a, b):
    ah = _tf32(a)
    al = _tf32(a - ah)
    bh = _tf32(b)
    bl = _tf32(b - bh)
    # each product of two TF32 values is exact in FP32; sequential FP32 sums
    terms = (ah[:, None, :] * bh[None, :, :] + ah[:, None, :] * bl[None, :, :]
             + al[:, None, :] * bh[None, :, :]).astype(np.float32)
    return np.add.accumulate(terms, axis=2, dtype=np.float32)[:, :, -1].astype(np.float64)


def _split_fp16x3(v, scale):
    """Integer plane (|v s| <= 128) and two FP16 remainder planes, in row units."""
    s = (v * scale).astype(np.float32)
    p0 = np.rint(s).astype(np.float32)
    r = (s - p0).astype(np.float32)
    p1 = r.astype(np.float16).astype(np.float32)
    p2 = (r - p1).astype(np.float16).astype(np.float32)
    return p0, p1, p2


def _row_scale(v):
    m = np.abs(v).max(axis=1, keepdims=True)
    e = np.frexp(m)[1]
    return np.ldexp(1.0, 7 - e).astype(np.float32)


def _gram_fp16x3(a, b):
    sa, sb = _row_scale(a), _row_scale(b)
    A = _split_fp16x3(a, sa)
    B = _split_fp16x3(b, sb)
    main = (A[0].astype(np.int64)[:, None, :] * B[0].astype(np.int64)[None, :, :]).sum(axis=2)
    corr = np.zeros(main.shape + (a.shape[1],), np.float32)
    for pa, pb in ((0, 1), (0, 2), (1, 0), (1, 1), (2, 0)):
        corr += (A[pa][:, None, :] * B[pb][None, :, :]).astype(np.float32)
    c = np.add.accumulate(corr, axis=2, dtype=np.float32)[:, :, -1]
    return (main.astype(np.float64) + c.astype(np.float64)) / (sa.astype(np.float64) * sb.astype(np.float64).T)


def test_tf32_compensated_against_fp16x3():
    rng = np.random.default_rng(11)
    rows, K = 24, 1024           # one 1024-K sub-chunk, as the kernel's
    y = rng.standard_normal((rows, K)).astype(np.float32)
    w = rng.uniform(0.1, 1.0, K).astype(np.float32)          # positive weights: a diagonal-like sum
    a = (y * w).astype(np.float32)
    exact = a.astype(np.float64) @ y.astype(np.float64).T
    den = np.abs(exact).max()
    e_tf32 = np.abs(_gram_tf32c(a, y) - exact).max() / den
    e_fp16x3 = np.abs(_gram_fp16x3(a, y) - exact).max() / den
    print(f"normwise Gram error at K = {K}: TF32-compensated {e_tf32:.2e}, FP16x3 {e_fp16x3:.2e}")
    # FP16x3 keeps about 27 bits per product and sums its leading part exactly
    assert e_fp16x3 < 1e-7
    # the TF32 form keeps about 22 bits per product: several times worse at the
    # same tensor time
    assert e_tf32 > 3 * e_fp16x3
