"""The compensated value contraction's arithmetic (k_gemm_comp in sparse_wf_gb300/csrc/fire_gemm.cuh), restated in
numpy float32 and checked against long-double sums and against Dot2 (Ogita, Rump and Oishi), the scheme it replaced.

Per 16-k tile every row of A is scaled by a power of two so that |a'| < 1, every column of B is bounded over K by
|b| < 2^eb; t = fma(a', b, 3 * 2^eb) lies in [2^(eb+1), 2^(eb+2)], where floats are evenly spaced, so the bit
patterns of t count grid steps exactly in a 32-bit integer, and fma(a', b, 3 * 2^eb - t) is the exact remainder.
An FMA is emulated in float64: the product of two floats is exact there, and so is every remainder this scheme takes
(it spans at most 48 bits); t itself may land on the neighbouring grid point in rare halfway cases, which the scheme
tolerates by construction (q = t - sigma is whatever grid point t gives, and the remainder is taken against it)."""
import numpy as np
import pytest

f32, f64 = np.float32, np.float64
KT = 16


def _fma(a, b, c):
    return (a.astype(f64) * b.astype(f64) + c.astype(f64)).astype(f32)


def _two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    return s, ((a - (s - bb)).astype(f32) + (b - bb).astype(f32)).astype(f32)


def _field(m):
    return (m.astype(f32).view(np.int32) >> 23) & 0xff


def _nanmax_abs(x, axis):
    """fmaxf semantics: NaN entries are skipped unless every entry is NaN."""
    with np.errstate(all="ignore"):
        m = np.nanmax(np.where(np.isnan(x), -np.inf, np.abs(x)), axis=axis)
    return np.where(np.all(np.isnan(x), axis=axis), np.nan, m).astype(f32)


def grid_sum(A, B):
    """hi + lo of A @ B as the kernel forms them (returned as float64 hi + lo)."""
    M, K = A.shape
    N = B.shape[1]
    mb = _nanmax_abs(B, 0)
    eb = np.maximum(_field(mb) - 126, -100)
    bad_col = (_field(mb) == 255) | (eb > 119)  # a non-finite or huge bound: the column's outputs are NaN
    eb = np.where(bad_col, 0, eb)
    sg = (f32(3) * np.ldexp(f32(1), eb)).astype(f32)[None, :]
    sg = np.where(bad_col[None, :], f32(np.nan), sg).astype(f32)
    g = np.ldexp(f32(1), eb - 22).astype(f32)[None, :]
    sb16 = (16 * sg.view(np.uint32).astype(np.uint64)) % (1 << 32)
    hi = np.zeros((M, N), f32)
    lo = np.zeros((M, N), f32)
    for k0 in range(0, K, KT):
        At = np.zeros((M, KT), f32)
        Bt = np.zeros((KT, N), f32)
        w = min(KT, K - k0)
        At[:, :w], Bt[:w] = A[:, k0:k0 + w], B[k0:k0 + w]
        m = _nanmax_abs(At, 1)
        ea = np.where(m > 0, np.maximum(_field(m) - 126, -125), 0)
        bad_row = (_field(m) == 255) | (ea > 126)
        ea = np.where(bad_row, 0, ea)
        inv = np.where(bad_row, f32(np.nan), np.ldexp(f32(1), -ea)).astype(f32)
        a_s = (At * inv[:, None]).astype(f32)
        sa = np.where(bad_row, f32(np.nan), np.ldexp(f32(1), ea)).astype(f32)[:, None]
        ti = np.zeros((M, N), np.uint64)
        rh = np.zeros((M, N), f32)
        for kk in range(KT):
            a, b = a_s[:, kk:kk + 1], Bt[kk:kk + 1]
            with np.errstate(invalid="ignore"):
                t = _fma(a, b, sg)
                fin = np.isfinite(t)
                assert np.all(((t >= 2 * sg / 3) & (t <= 4 * sg / 3))[fin])  # one binade: bits linear in the value
            t = np.where(fin, t, f32(np.nan)).astype(f32)
            ti = (ti + t.view(np.uint32).astype(np.uint64)) % (1 << 32)
            with np.errstate(invalid="ignore"):
                rh = (rh + _fma(a, b, (sg - t).astype(f32))).astype(f32)
        d = ((ti - sb16) % (1 << 32)).astype(np.int64)
        d = np.where(d >= 1 << 31, d - (1 << 32), d)
        ok = np.isfinite(rh)  # a NaN anywhere in the tile's products reaches the remainder sum
        assert np.all(np.abs(d[ok]) <= 1 << 26)
        d = np.where(ok, d, 0)
        xh = d.astype(f32)
        xl = (d - xh.astype(np.int64)).astype(f32)
        assert np.all(np.abs(xl) <= 2)
        with np.errstate(invalid="ignore"):
            uh = (xh * g * sa).astype(f32)
            ul = (_fma(xl, g, rh) * sa).astype(f32)
            hi, e = _two_sum(hi, uh)
            lo = (lo + (e + ul).astype(f32)).astype(f32)
    return hi.astype(f64) + lo.astype(f64)


def dot2(A, B):
    M, K = A.shape
    hi = np.zeros((M, B.shape[1]), f32)
    lo = np.zeros_like(hi)
    for k in range(K):
        a, b = A[:, k:k + 1], B[k:k + 1]
        pr = (a * b).astype(f32)
        hi, e = _two_sum(hi, pr)
        lo = (lo + (e + _fma(a, b, -pr)).astype(f32)).astype(f32)
    return hi.astype(f64) + lo.astype(f64)


def _operands(kind, rng, M=32, N=16):
    if kind == "envelope":  # exp(-sigma d) of 122 nuclei x 8 exponents against N(0, 0.5) weights, K = 976
        d = rng.uniform(0.3, 40, size=(M, 122))
        s = rng.uniform(0.3, 3.0, size=(122, 8))
        A = np.exp(-(d[:, :, None] * s[None])).reshape(M, -1)
        return A.astype(f32), (rng.standard_normal((976, N)) * 0.5).astype(f32)
    h = rng.standard_normal((M, 256))
    A = h / (1 + np.exp(-h))  # SiLU activations against lecun-like weights, K = 256
    B = rng.standard_normal((256, N)) / 16
    if kind == "scaled":  # rows and columns over many binades
        A = A * np.exp(rng.uniform(-8, 8, size=(M, 1)))
        B = B * np.exp(rng.uniform(-8, 8, size=(1, N)))
    return A.astype(f32), B.astype(f32)


@pytest.mark.parametrize("kind", ["envelope", "orbital", "scaled"])
def test_grid_sum_error_is_of_dot2_order(kind):
    A, B = _operands(kind, np.random.default_rng(5))
    exact = (A.astype(np.longdouble) @ B.astype(np.longdouble))
    scale = np.abs(A).astype(f64) @ np.abs(B).astype(f64)
    eg = np.abs((grid_sum(A, B) - exact).astype(f64)) / scale
    ed = np.abs((dot2(A, B) - exact).astype(f64)) / scale
    print(f"{kind}: grid max {eg.max():.2e} median {np.median(eg):.2e}; dot2 max {ed.max():.2e} median {np.median(ed):.2e}")
    assert eg.max() <= 1e-12  # ~2^-40 of sum |ab|: second order in the FP32 unit roundoff
    assert eg.max() <= 5 * ed.max() + 1e-15 and np.median(eg) <= 10 * np.median(ed) + 1e-16


def test_grid_sum_cancellation_and_zero_rows():
    """A result that cancels to ~1e-7 of its terms keeps ~2^-40 of sum |ab|; zero rows and columns give exact 0."""
    rng = np.random.default_rng(6)
    A, B = _operands("orbital", rng, M=8, N=4)
    B[-1] = 0
    A[:, -1] = 1
    c = A.astype(f64) @ B.astype(f64)
    B[-1] = (-c[0]).astype(f32)  # row 0 of the product cancels to the rounding of -c
    A[3] = 0
    B[:, 2] = 0
    exact = A.astype(np.longdouble) @ B.astype(np.longdouble)
    got = grid_sum(A, B)
    scale = np.abs(A).astype(f64) @ np.abs(B).astype(f64)
    assert np.all(got[3] == 0) and np.all(got[:, 2] == 0)
    assert np.all(np.abs((got - exact).astype(f64)) <= 1e-12 * scale)


def test_grid_sum_non_finite_operands_give_nan():
    """A NaN or an infinity in a row of A or a column of B makes every output it reaches NaN (the bound of a row or
    column that holds an infinity is non-finite, and NaN products reach the remainder sum); the other outputs are
    untouched."""
    rng = np.random.default_rng(7)
    A, B = _operands("orbital", rng, M=6, N=5)
    A[1, 17] = np.nan
    A[2, 40] = np.inf
    B[100, 3] = -np.inf
    got = grid_sum(A, B)
    bad = np.zeros(got.shape, bool)
    bad[1, :] = bad[2, :] = bad[:, 3] = True
    assert np.all(np.isnan(got[bad]))
    exact = A[~np.isin(np.arange(6), [1, 2])].astype(np.longdouble) @ B.astype(np.longdouble)
    rows = np.setdiff1d(np.arange(6), [1, 2])
    cols = np.setdiff1d(np.arange(5), [3])
    scale = np.abs(A[rows]).astype(f64) @ np.abs(B).astype(f64)
    err = np.abs((got[np.ix_(rows, cols)] - exact[:, cols]).astype(f64)) / scale[:, cols]
    assert np.all(np.isfinite(got[np.ix_(rows, cols)])) and err.max() <= 1e-12
