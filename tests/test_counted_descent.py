"""The counted FP16-brick form replaces the plain march's descent onto a
ground plane by a closed-form step count: from height g above the plane on a
ray of downward slope s, with step = scale x distance, heights shrink by
(1 - scale s) per step, so the first sample inside the eps shell is
n = floor(ln(eps / g) / ln(1 - scale s)) + 1 steps later.  This checks that
count, in the float32 form the kernel evaluates (plane_descent_steps: the
closed form, then a check of the heights at n - 1 and n), against a literal
float32 plain march (raymarch_hit's step rule, R:4100-4137) over random
descents: equal, or off by one step, never more."""
import numpy as np


def plain_steps(oy, dy, t0, top, eps, scale, min_step, limit):
    """Steps the float32 plain march takes from t0 until a sample lies inside
    the eps shell of the plane y = top (distance y - top), or limit."""
    oy, dy, t, top, eps = np.float32(oy), np.float32(dy), np.float32(t0), np.float32(top), np.float32(eps)
    scale, min_step = np.float32(scale), np.float32(min_step)
    for k in range(limit):
        d = (oy + dy * t) - top
        if abs(d) < eps:
            return k
        t = t + max(abs(d) * scale, min_step)
    return limit


def closed_form(g, s, eps, scale):
    f = np.float32
    g, s, eps, scale = f(g), f(s), f(eps), f(scale)
    c = scale * s
    q = f(1.0) - c
    x = np.log(eps / g) / np.log1p(-c)
    assert x.dtype == np.float32
    n = int(np.floor(x)) + 1
    if n > 1 and g * np.power(q, f(n - 1)) < eps:
        n -= 1
    elif g * np.power(q, f(n)) >= eps:
        n += 1
    return n


def test_closed_form_matches_the_plain_march():
    rng = np.random.default_rng(3)
    eps, scale = 1.0e-4, 0.7
    min_step = max(eps * 0.5, 1.0e-5)
    agree = off_by_one = 0
    for _ in range(4000):
        s = float(rng.uniform(0.02, 1.0))                   # downward slope of the ray
        oy = float(rng.uniform(0.05, 6.0))                  # height of the ray origin
        dy = -s
        g = float(np.float32((np.float32(oy) + np.float32(dy) * np.float32(0.0)) - np.float32(0.0)))
        if g < eps:
            continue
        n = closed_form(g, s, eps, scale)
        k = plain_steps(oy, dy, 0.0, 0.0, eps, scale, min_step, n + 8)
        if k == n:
            agree += 1
        elif abs(k - n) == 1:
            off_by_one += 1
        else:
            raise AssertionError((oy, s, n, k))
    # Float rounding of the march's heights moves the crossing by one step when
    # the exact crossing lies within rounding of a sample (0.6 % of these
    # descents); never by more.  So the counted form can only disagree with the
    # plain march on rays whose total count is within one step of max_steps.
    assert agree / (agree + off_by_one) >= 0.99, (agree, off_by_one)
