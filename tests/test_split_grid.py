"""The scaled-grid FP16 split of the tensor-core contractions (grid_code, grid_scales, grid_hb and split_grid_f16x2 in
sparse_wf_gb300/csrc/fire_tc.cuh; k_gemm_tca with hb = 7 for K <= 256, k_env_tc with hb = grid_hb(8 N)), restated in
numpy and checked for the properties the kernels rely on:

- a row whose largest magnitude is in [2^e, 2^(e+1)) is scaled by 2^(hb - e), so hi = rint(x) is an integer of
  magnitude <= 2^(hb+1), exact in FP16, and lo = x - hi (|lo| <= 1/2) rounds to FP16 within 2^-13;
- K products of two hi parts are integers of magnitude <= 2^(2 hb + 2) and K 2^(2 hb + 2) <= 2^24, so their sum is
  exact in an FP32 accumulator in any order (the tensor core's accumulation order and rounding do not matter);
- with the three other products added, the reconstruction errs by ~2^-(13 + hb) of the row's largest value per
  element (2^-20 for hb = 7, 2^-19 for hb = 6)."""
import numpy as np
import pytest

f16, f32, f64 = np.float16, np.float32, np.float64
GRID_ZERO, GRID_NAN = -32768, 32767


def grid_code(mx):
    if mx == 0:
        return GRID_ZERO
    if not (mx <= 3.4e38):
        return GRID_NAN
    return max(int(np.frexp(f64(mx))[1]) - 1, -120)  # ilogb


def grid_hb(K):
    l = 0
    while (1 << l) < K:
        l += 1
    return (22 - l) // 2


def split(x_row, hb):
    """(hi, lo, sc): FP16 hi and lo parts of a row and the scale the epilogue applies."""
    code = grid_code(float(np.max(np.abs(x_row))))
    if code == GRID_ZERO:
        return np.zeros_like(x_row, f16), np.zeros_like(x_row, f16), 0.0
    inv = f32(np.ldexp(1.0, hb - code))
    x = (x_row.astype(f32) * inv).astype(f32)
    hi = np.rint(x).astype(f32)
    lo = (x - hi).astype(f32)
    return hi.astype(f16), lo.astype(f16), float(np.ldexp(1.0, code - hb))


@pytest.mark.parametrize("K,hb", [(256, 7), (976, grid_hb(976)), (64, 7)])
def test_split_bounds_and_exact_hi_sums(K, hb):
    assert grid_hb(976) == 6 and grid_hb(256) == 7 and K * 2.0 ** (2 * hb + 2) <= 2.0 ** 24
    rng = np.random.default_rng(K)
    for trial in range(20):
        a = (rng.standard_normal(K) * np.exp(rng.uniform(-30, 30))).astype(f32)
        w = (rng.standard_normal(K) * np.exp(rng.uniform(-30, 30))).astype(f32)
        if trial % 5 == 0:  # a row of one dominant value and many tiny ones
            a[rng.integers(K)] *= 1e6
        ha, la, sa = split(a, hb)
        hw, lw, sw = split(w, hb)
        assert np.all(np.abs(ha.astype(f64)) <= 2.0 ** (hb + 1)) and np.all(ha.astype(f64) == np.rint(ha.astype(f64)))
        x = a.astype(f64) / sa
        assert np.all(np.abs(x - ha.astype(f64)) <= 0.5) and np.all(np.abs(x - ha - la.astype(f64)) <= 2.0 ** -13)
        # hi x hi: integer products summed in FP32 in two different orders give the exact integer sum
        p = ha.astype(f64) * hw.astype(f64)
        exact = int(np.sum(p.astype(np.int64)))
        for order in (np.arange(K), rng.permutation(K)):
            acc = f32(0)
            for k in order:
                acc = f32(acc + f32(p[k]))
            assert int(acc) == exact
        # the four products against the exact dot product: ~2^-(13 + hb) of the largest values, summed over K
        cross = np.sum(ha.astype(f64) * lw + la.astype(f64) * hw + la.astype(f64) * lw.astype(f64))
        got = (exact + cross) * sa * sw
        ref = float(np.dot(a.astype(np.longdouble), w.astype(np.longdouble)))
        bound = K * 2.0 ** -(12 + hb) * np.max(np.abs(a)) * np.max(np.abs(w))
        assert abs(got - ref) <= bound, (got, ref, bound)


def test_split_codes_of_zero_and_non_finite_rows():
    assert grid_code(0.0) == GRID_ZERO and grid_code(float("inf")) == GRID_NAN and grid_code(float("nan")) == GRID_NAN
    assert grid_code(1e-40) == -120 and grid_code(1.0) == 0 and grid_code(1.5) == 0 and grid_code(2.0) == 1
    hi, lo, sc = split(np.zeros(16, f32), 7)
    assert sc == 0.0 and not np.any(hi) and not np.any(lo)
