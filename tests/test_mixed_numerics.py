"""The numerical premises of the mixed-precision form, checked in numpy on the CPU.

Positions are held as unevaluated float sums x = hi + lo (hi = float(x), lo =
float(x - hi)); the separation of two particles is formed as (hi_j - hi_i) + (lo_j - lo_i)
in float arithmetic.  Its error is a few float ulps of the separation itself, however far
the pair sits from the origin, which is what the form's FP32 pair arithmetic relies on.
"""
import numpy as np


def split(x):
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def test_hi_lo_separation_is_accurate_to_float_ulps_of_the_separation():
    rng = np.random.default_rng(17)
    n = 200000
    xi = rng.uniform(-10.0, 10.0, n)
    sep = 10.0 ** rng.uniform(-7, 0, n) * rng.choice([-1.0, 1.0], n)   # 1e-7 .. 1
    xj = xi + sep
    hi_i, lo_i = split(xi)
    hi_j, lo_j = split(xj)
    d = (hi_j - hi_i) + (lo_j - lo_i)          # float32 throughout
    exact = xj - xi                           # the fp64 separation
    rel = np.abs(d.astype(np.float64) - exact) / np.abs(exact)
    assert rel.max() < 4 * np.finfo(np.float32).eps
    # the plain float difference loses the separation entirely at small scales
    plain = (xj.astype(np.float32) - xi.astype(np.float32)).astype(np.float64)
    assert (np.abs(plain - exact) / np.abs(exact)).max() > 0.1


def test_split_is_exact():
    rng = np.random.default_rng(3)
    x = rng.uniform(-100.0, 100.0, 100000)
    hi, lo = split(x)
    # hi + lo reproduces x to the last bits of a double-float pair (about 2^-48 relative)
    err = np.abs(hi.astype(np.float64) + lo.astype(np.float64) - x) / np.abs(x)
    assert err.max() < 2.0 ** -46


def test_float_membership_with_margin_never_contradicts_fp64():
    """The SPH-neighbour test of the mixed form (float d^2 against float max(4 h_i^2,
    4 h_j^2) with a 2^-14 relative margin, fp64 re-check inside the margin): every pair the
    float test decides gets the fp64 decision."""
    margin = 2.0 ** -14
    rng = np.random.default_rng(29)
    n = 400000
    ri = rng.uniform(-5.0, 5.0, (n, 3))
    hi_h = 10.0 ** rng.uniform(-3, -1, n)
    hj_h = hi_h * rng.uniform(0.8, 1.25, n)
    hrs_i, hrs_j = 4.0 * hi_h * hi_h, 4.0 * hj_h * hj_h
    # separations concentrated around the membership boundary
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    dist = np.sqrt(np.maximum(hrs_i, hrs_j)) * (1.0 + rng.normal(0.0, 3e-4, n))
    rj = ri + u * dist[:, None]
    d64 = rj - ri
    drsqd = np.einsum("ij,ij->i", d64, d64)
    member64 = ~((drsqd >= hrs_i) & (drsqd >= hrs_j))
    hi_a, lo_a = split(ri)
    hi_b, lo_b = split(rj)
    d32 = (hi_b - hi_a) + (lo_b - lo_a)
    d2 = np.einsum("ij,ij->i", d32, d32).astype(np.float32)
    thr = np.maximum(hrs_i.astype(np.float32), hrs_j.astype(np.float32))
    yes = d2 < thr * np.float32(1.0 - margin)
    no = d2 > thr * np.float32(1.0 + margin)
    assert not np.any(yes & ~member64)
    assert not np.any(no & member64)
    # the margin band (fp64 re-check) takes a small fraction even of these near-boundary pairs
    assert np.mean(~(yes | no)) < 0.5


def test_float_walk_decisions_with_margin_never_contradict_fp64():
    """The gravity walk's near test and MAC of the mixed form: float values with a 2^-14
    margin (fp64 re-test inside it) agree with the fp64 decisions of the reference's walk
    wherever the float test decides."""
    margin = 2.0 ** -14
    rng = np.random.default_rng(41)
    n = 300000
    rc_leaf = rng.uniform(-3.0, 3.0, (n, 3))
    rmax_leaf = 10.0 ** rng.uniform(-3, -1, n)
    rmax_c = rmax_leaf * 10.0 ** rng.uniform(0, 1.5, n)
    hmax_leaf = rmax_leaf * rng.uniform(0.5, 2.0, n)
    hmax_c = rmax_c * rng.uniform(0.1, 1.0, n)
    cdist = np.maximum(rmax_c ** 2, hmax_c ** 2) / 0.25
    # cell centres near either boundary
    target = np.where(rng.random(n) < 0.5,
                      np.maximum(rmax_c + rmax_leaf + 2.0 * hmax_leaf, rmax_leaf + rmax_c + 2.0 * hmax_c),
                      np.sqrt(cdist))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    rc_c = rc_leaf + u * (target * (1.0 + rng.normal(0.0, 3e-4, n)))[:, None]
    d64 = rc_c - rc_leaf
    drsqd = np.einsum("ij,ij->i", d64, d64)
    t1 = (rmax_c + rmax_leaf + 2.0 * hmax_leaf) ** 2
    t2 = (rmax_leaf + rmax_c + 2.0 * hmax_c) ** 2
    near64 = (drsqd <= t1) | (drsqd <= t2)
    open64 = drsqd < cdist
    hi_a, lo_a = split(rc_leaf)
    hi_b, lo_b = split(rc_c)
    d32 = (hi_b - hi_a) + (lo_b - lo_a)
    d2 = np.einsum("ij,ij->i", d32, d32).astype(np.float32)
    f = lambda a: a.astype(np.float32)
    a1 = f(rmax_c) + f(rmax_leaf) + np.float32(2.0) * f(hmax_leaf)
    a2 = f(rmax_leaf) + f(rmax_c) + np.float32(2.0) * f(hmax_c)
    thr = np.maximum(a1 * a1, a2 * a2)
    near_yes = d2 < thr * np.float32(1.0 - margin)
    near_no = d2 > thr * np.float32(1.0 + margin)
    assert not np.any(near_yes & ~near64) and not np.any(near_no & near64)
    cd = f(cdist)
    open_yes = d2 < cd * np.float32(1.0 - margin)
    open_no = d2 > cd * np.float32(1.0 + margin)
    assert not np.any(open_yes & ~open64) and not np.any(open_no & open64)
