"""The double-FP32 (df64) arithmetic of the orbital-matrix elimination (sparse_wf_gb300/csrc/fire_df64.cuh), restated
in numpy float32 and checked against long-double results: addition and multiplication to a few units of 2^-48, the
fused a - b c (df_sub_mul) to ~2^-46, the division with two correction steps, and the compensated dot product of the
panel updates (SubDot<df64>: Dot2 extended to double-FP32 factors) to ~2^-46 of the terms' magnitude.  Every FP32
operation rounds to nearest as __fadd_rn / __fmul_rn do; an FMA is emulated in float64, where the product of two
floats is exact and so is the low part fma(a, b, -fl(a b))."""
import numpy as np
import pytest

f32, f64 = np.float32, np.float64
LD = np.longdouble
U = 2.0 ** -48


def fma(a, b, c):
    return f32(f64(a) * f64(b) + f64(c))


def quick_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def two_sum(a, b):
    s = f32(a + b)
    v = f32(s - a)
    return s, f32(f32(a - f32(s - v)) + f32(b - v))


def add(a, b):
    s, sl = two_sum(a[0], b[0])
    t, tl = two_sum(a[1], b[1])
    sl = f32(sl + t)
    s, sl = quick_two_sum(s, sl)
    sl = f32(sl + tl)
    return quick_two_sum(s, sl)


def neg(a):
    return (f32(-a[0]), f32(-a[1]))


def mul(a, b):
    p = f32(a[0] * b[0])
    e = fma(a[0], b[0], -p)
    e = fma(a[0], b[1], e)
    e = fma(a[1], b[0], e)
    return quick_two_sum(p, e)


def div(a, b):
    q1 = f32(a[0] / b[0])
    r = add(a, neg(mul(b, (q1, f32(0)))))
    q2 = f32(r[0] / b[0])
    r = add(r, neg(mul(b, (q2, f32(0)))))
    q3 = f32(r[0] / b[0])
    return add(quick_two_sum(q1, q2), (q3, f32(0)))


def sub_mul(a, b, c):
    p = f32(b[0] * c[0])
    e = fma(b[0], c[0], -p)
    e = fma(b[0], c[1], e)
    e = fma(b[1], c[0], e)
    s = f32(a[0] - p)
    v = f32(s - a[0])
    t = f32(f32(a[0] - f32(s - v)) + f32(-p - v))
    return quick_two_sum(s, f32(t + f32(a[1] - e)))


def sub_dot(a, bs, ys):
    """a - sum_t b_t y_t as SubDot<df64>::add over the terms, then finish(a)."""
    s = c = f32(0)
    for b, y in zip(bs, ys):
        p = f32(b[0] * y[0])
        e = fma(b[0], y[0], -p)
        c = fma(b[0], y[1], c)
        c = fma(b[1], y[0], c)
        s1 = f32(s + p)
        bb = f32(s1 - s)
        q = f32(f32(s - f32(s1 - bb)) + f32(p - bb))
        c = f32(c + f32(q + e))
        s = s1
    r = two_sum(a[0], f32(-s))
    return two_sum(r[0], f32(r[1] + f32(a[1] - c)))


def val(x):
    return LD(x[0]) + LD(x[1])


def rand_df(rng, scale=1.0):
    d = rng.standard_normal() * scale
    hi = f32(d)
    return (hi, f32(d - f64(hi)))


@pytest.fixture
def rng():
    return np.random.default_rng(11)


def test_df64_add_mul_div_sub_mul(rng):
    worst = {"add": 0.0, "mul": 0.0, "div": 0.0, "sub_mul": 0.0}
    for _ in range(3000):
        a, b, c = rand_df(rng, 10 ** rng.uniform(-3, 3)), rand_df(rng, 10 ** rng.uniform(-3, 3)), rand_df(rng)
        worst["add"] = max(worst["add"], float(abs(val(add(a, b)) - (val(a) + val(b))) / (abs(val(a)) + abs(val(b)))))
        worst["mul"] = max(worst["mul"], float(abs(val(mul(a, b)) - val(a) * val(b)) / abs(val(a) * val(b))))
        worst["div"] = max(worst["div"], float(abs(val(div(a, b)) - val(a) / val(b)) / abs(val(a) / val(b))))
        ex = val(a) - val(b) * val(c)
        worst["sub_mul"] = max(worst["sub_mul"], float(abs(val(sub_mul(a, b, c)) - ex)
                                                      / (abs(val(a)) + abs(val(b) * val(c)))))
    print({k: f"{v / U:.2f} u" for k, v in worst.items()})
    assert worst["add"] <= 4 * U and worst["mul"] <= 8 * U and worst["div"] <= 16 * U
    assert worst["sub_mul"] <= 8 * U  # ~2^-46 of |a| + |b c|: the low parts join without their own TwoSum


@pytest.mark.parametrize("terms", [16, 322])
def test_df64_compensated_panel_update(rng, terms):
    """a - sum b_t y_t over a panel (16 terms) and over a whole row (322 terms) against long double: within a few
    units of 2^-46 of |a| + sum |b y| even where the result cancels."""
    worst = 0.0
    for trial in range(60):
        bs = [rand_df(rng) for _ in range(terms)]
        ys = [rand_df(rng) for _ in range(terms)]
        dot = sum(val(b) * val(y) for b, y in zip(bs, ys))
        a = rand_df(rng) if trial % 2 else (f32(dot), f32(f64(dot) - f64(f32(dot))))  # odd: cancelling result
        ex = val(a) - dot
        mag = abs(val(a)) + sum(abs(val(b) * val(y)) for b, y in zip(bs, ys))
        worst = max(worst, float(abs(val(sub_dot(a, bs, ys)) - ex) / mag))
    print(f"{terms} terms: worst {worst / U:.2f} u of |a| + sum |b y|")
    assert worst <= 16 * U
