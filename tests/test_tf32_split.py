"""Error of the tensor-core scattering's FP32 emulation (scat_tc_kernel),
checked in numpy: each FP32 value v is split into hi = v rounded to TF32
(round to nearest, ties away from zero: the rounding of cvt.rna.tf32.f32) and
lo = v - hi (exact in FP32); the MMA reads both operands as TF32 (assumed here
to truncate lo, the worse case) and the product is lo_a hi_b + hi_a lo_b +
hi_a hi_b.  Per product the relative error stays below 2^-20; dot products of
the lengths the kernel meets (up to 224 angular nodes) stay within the 2e-6
that the GPU tests allow for the FP32 apply."""
import numpy as np

TF32_MASK = np.uint32(0xFFFFE000)


def _rna_tf32(v):
    b = v.astype(np.float32).view(np.uint32)
    finite = (b & np.uint32(0x7F800000)) != np.uint32(0x7F800000)
    r = np.where(finite, (b + np.uint32(0x1000)) & TF32_MASK, b)
    return r.astype(np.uint32).view(np.float32)


def _trunc_tf32(v):
    return (v.astype(np.float32).view(np.uint32) & TF32_MASK).view(np.float32)


def _split(v):
    hi = _rna_tf32(v)
    lo = (v.astype(np.float32) - hi).astype(np.float32)
    return hi, lo


def _product3(a, b):
    ah, al = _split(a)
    bh, bl = _split(b)
    # the tensor core reads TF32 operands; products and sums in float64 here
    ah, al, bh, bl = (x.astype(np.float64) for x in (_trunc_tf32(ah), _trunc_tf32(al), _trunc_tf32(bh),
                                                      _trunc_tf32(bl)))
    return al * bh + ah * bl + ah * bh


def test_split_is_exact_in_fp32():
    rng = np.random.default_rng(0)
    v = (rng.standard_normal(200_000) * np.exp(rng.uniform(-20, 20, 200_000))).astype(np.float32)
    hi, lo = _split(v)
    assert np.array_equal((hi.astype(np.float64) + lo.astype(np.float64)), v.astype(np.float64))
    # hi is a TF32 value and lo is at most half a TF32 unit of hi
    assert np.array_equal(_trunc_tf32(hi), hi)
    assert np.all(np.abs(lo.astype(np.float64)) <= np.abs(hi.astype(np.float64)) * 2.0 ** -11 * (1 + 1e-12))


def test_product_error_below_2_pow_minus_20():
    rng = np.random.default_rng(1)
    a = (rng.standard_normal(500_000) * np.exp(rng.uniform(-10, 10, 500_000))).astype(np.float32)
    b = (rng.standard_normal(500_000) * np.exp(rng.uniform(-10, 10, 500_000))).astype(np.float32)
    exact = a.astype(np.float64) * b.astype(np.float64)
    rel = np.abs(_product3(a, b) - exact) / np.abs(exact)
    assert rel.max() < 2.0 ** -20


def test_dot_products_within_fp32_apply_tolerance():
    rng = np.random.default_rng(2)
    for n in (16, 64, 144, 224):
        W = rng.uniform(0., 1., (64, n)).astype(np.float32)       # scattering weights are positive
        X = rng.standard_normal((n, 81)).astype(np.float32)
        exact = W.astype(np.float64) @ X.astype(np.float64)
        approx = sum(_product3(np.broadcast_to(W[:, k:k + 1], (64, 81)), np.broadcast_to(X[k:k + 1, :], (64, 81)))
                     for k in range(n))
        err = np.linalg.norm(approx - exact) / np.linalg.norm(exact)
        assert err < 2e-6, (n, err)
