"""The reference's double-precision computations that the device decides or evaluates in FP32 (FP64 is
slow on this GPU): CorrectFlat's +-1e-6 window (gpu_fine_contact_detection.cu:256-268), the EPA's
relative 1e-5 convergence test (.cu:439), the cell coordinate trunc(p / cs) (MWDiem.py:813-816), the
contact point's barycentric weight 1 - bw - bv (.cu:583), the tangential stiffness and damping Kt, Gt
(.cu:746-749) and the Coulomb test (.cu:774).  These restate the kernels' code (narrow.cu within_1e6,
epa_converged, one_minus_two, tangential_coeffs, coulomb_compare; broad.cu cell_coord) in numpy
float32 arithmetic, which rounds as the kernels do (no contraction; the two fused multiply-adds are
remainders that float64 holds exactly), and check that they give the double computations' answers,
bit for bit, on random and adversarial inputs."""
import numpy as np

f32 = np.float32
F = np.array([0x358637BE], np.uint32).view(np.float32)[0]


def within_1e6(v):
    return (v < F) & (v > -F)


def within_1e6_ref(v):
    d = v.astype(np.float64)
    return (d < 0.000001) & (d > -0.000001)


def epa_converged(x, p):
    x = x.astype(f32)
    p = p.astype(f32)
    ax = np.abs(x)
    with np.errstate(over="ignore", invalid="ignore"):
        hi = x * f32(1.00001)
        lo = x * f32(0.99999)
        tol = ax * f32(2.384185791015625e-7)
        fast = (ax > f32(1e-30)) & (ax < f32(1e37))
        yes = fast & (p < hi - tol) & (p > lo + tol)
        no = fast & ((p > hi + tol) | (p < lo - tol))
        ref = epa_converged_ref(x, p)
    out = np.where(yes, True, np.where(no, False, ref))
    return out, ~(yes | no)


def epa_converged_ref(x, p):
    xd, pd = x.astype(np.float64), p.astype(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        return (xd * 1.00001 > pd) & (xd * 0.99999 < pd)


def test_flat_window_matches_double():
    rng = np.random.default_rng(0)
    base = np.array([1e-6, -1e-6], np.float64)
    near = []
    for b in base:
        c = f32(b)
        for k in range(-40, 41):
            near.append(c)
            c = np.nextafter(c, f32(np.inf) if k < 0 else f32(-np.inf))
    v = np.concatenate([np.array(near, f32), rng.normal(scale=2e-6, size=100000).astype(f32),
                        np.array([0.0, -0.0, np.nan, np.inf, -np.inf], f32)])
    for b in base:  # every float within 64 ulps of each bound
        c = f32(b)
        seq = [c]
        for _ in range(64):
            seq.append(np.nextafter(seq[-1], f32(np.inf)))
            seq.insert(0, np.nextafter(seq[0], f32(-np.inf)))
        v = np.concatenate([v, np.array(seq, f32)])
    assert np.array_equal(within_1e6(v), within_1e6_ref(v))


def test_epa_convergence_filter_matches_double():
    rng = np.random.default_rng(1)
    n = 400000
    x = np.concatenate([rng.uniform(1e-3, 10, n), rng.lognormal(0, 20, n // 4), -rng.uniform(0, 5, n // 8)]).astype(f32)
    rel = rng.normal(scale=2e-5, size=x.shape)
    p = (x.astype(np.float64) * (1 + rel)).astype(f32)
    # p at and around each bound of the double test, ulp by ulp
    xb = rng.uniform(0.01, 5, 2000).astype(f32)
    edge = []
    xs = []
    for c in (1.00001, 0.99999):
        for xi in xb:
            q = f32(np.float64(xi) * c)
            for _ in range(8):
                q = np.nextafter(q, f32(-np.inf))
            for _ in range(17):
                edge.append(q)
                xs.append(xi)
                q = np.nextafter(q, f32(np.inf))
    x = np.concatenate([x, np.array(xs, f32), np.array([0, 0, 1e30, 1e38, -1e38, np.nan, 2.0, 1e-35], f32)])
    p = np.concatenate([p, np.array(edge, f32), np.array([0, 1e-40, 1e30, 3e38, -3e38, 1.0, np.nan, 1e-35], f32)])
    got, slow = epa_converged(x, p)
    assert np.array_equal(got, epa_converged_ref(x, p))
    # the FP64 fallback is rare even for p spread within a few 1e-5 of x
    assert slow[:n].mean() < 0.03


def cell_coord(p, cs):
    """broad.cu cell_coord: the float quotient away from integers, else the double division."""
    inv = f32(1.0 / cs)
    q = p.astype(f32) * inv
    aq = np.abs(q)
    with np.errstate(invalid="ignore"):
        t = np.trunc(q)
        fr = aq - np.abs(t)
        band = aq * f32(4.76837158203125e-7)
        fast = (aq < f32(8388608.0)) & (fr > band) & (fr < f32(1.0) - band)
        ref = np.trunc(p / cs)
    return np.where(fast, t.astype(np.float64), ref), fast


def test_cell_coordinate_filter_matches_double():
    rng = np.random.default_rng(3)
    for cs in (2.4444444444444446, 2.4212962962962963, 1.0, 0.3, 7.123456789):
        p = np.concatenate([rng.uniform(-300, 300, 200000), rng.normal(0, 5, 50000)])
        # centres a few ulps either side of every cell boundary in range
        k = np.arange(-120, 121)
        edge = (k * cs)[:, None] + np.array([-2, -1, 0, 1, 2])[None, :] * np.spacing(np.abs(k * cs) + 1.0)[:, None]
        p = np.concatenate([p, edge.ravel(), [0.0, -0.0, 1e-300, -1e-300]])
        got, fast = cell_coord(p, cs)
        assert np.array_equal(got, np.trunc(p / cs)), cs
        assert fast[:200000].mean() > 0.999


# ---------------------------------------------------------------- float-float evaluations (narrow.cu)

def two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def fast_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def fma_rem(a, b, c):
    """fmaf(a, b, c) where the result is a rounding remainder (exactly a float): float64 holds the
    48-bit product and the cancelling sum exactly."""
    r = a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)
    return r.astype(f32)


def rounds_to(a, b, err):
    ua = a.view(np.uint32) & np.uint32(0x7FFFFFFF)
    ok = (ua >= 0x0C800000) & (ua < 0x7F000000)
    ulp = (ua & np.uint32(0x7F800000)).view(f32) * f32(1.1920928955078125e-7)
    toward_zero = (b < 0) != (a < 0)
    half = np.where(((ua & np.uint32(0x007FFFFF)) == 0) & toward_zero, f32(0.25) * ulp, f32(0.5) * ulp)
    with np.errstate(invalid="ignore", over="ignore"):
        return ok & (np.abs(b) + err < half * f32(0.99999))


def ulp_of(x):
    ux = x.view(np.uint32) & np.uint32(0x7FFFFFFF)
    normal = (ux & np.uint32(0x7F800000)).view(f32) * f32(1.1920928955078125e-7)
    return np.where((ux == 0) | (ux >= 0x7F800000), f32(np.inf),
                    np.where(ux < 0x00800000, f32(1.401298464324817e-45), normal)).astype(f32)


def one_minus_two(bw, bv):
    with np.errstate(invalid="ignore", over="ignore"):
        s1, e1 = two_sum(f32(1.0), -bw)
        s2, e2 = two_sum(s1, -bv)
        t, r = two_sum(e2, e1)
        a, b0 = two_sum(s2, t)
        q = np.minimum(np.minimum(ulp_of(bw), ulp_of(bv)), f32(1.1920928955078125e-7))
        exact = np.maximum(np.abs(s1), np.abs(a)) < q * f32(2251799813685248.0)
        b = b0 + r
        err = np.where(exact, f32(0), (np.abs(s1) + np.abs(a)) * f32(2.220446049250313e-16)) + \
            np.abs(b) * f32(1.1920928955078125e-7)
        finite = (np.abs(bw) < f32(1e30)) & (np.abs(bv) < f32(1e30))
        fast = finite & ((exact & (r == 0)) | rounds_to(a, b, err))
        ref = (1.0 - bw.astype(np.float64) - bv.astype(np.float64)).astype(f32)
    return np.where(fast, a, ref), fast, ref


def tangential_coeffs(m, x, y):
    ih, il, kh0, kl0, L = (f32(m.inv_mu_hi), f32(m.inv_mu_lo), f32(m.KtA_hi), f32(m.KtA_lo), f32(m.ln_et))
    with np.errstate(invalid="ignore", over="ignore", divide="ignore"):
        c1, e1 = two_sum(ih, x)
        c2, e2 = two_sum(c1, y)
        ch, cl = fast_two_sum(c2, (il + e1) + e2)
        rc = f32(1.0) / ch
        q1 = kh0 / ch
        rq = ((fma_rem(-q1, ch, np.full_like(ch, kh0)) + kl0) - q1 * cl) * rc
        kh, kl = fast_two_sum(q1, rq)
        g1 = f32(-2.0) * rc
        rg = (fma_rem(-g1, ch, np.full_like(ch, f32(-2.0))) - g1 * cl) * rc
        gh, gl = fast_two_sum(g1, rg)
        p = gh * L
        Gh, Gl = fast_two_sum(p, fma_rem(gh, np.full_like(gh, L), -p) + gl * L)
        ok = (x >= 0) & (x < f32(1e30)) & (y >= 0) & (y < f32(1e30)) & (ih > 0) & (ih < f32(1e30))
        okK = ok & rounds_to(kh, kl, np.abs(kh) * f32(4.547473508864641e-13))
        okG = ok & rounds_to(Gh, Gl, np.abs(Gh) * f32(4.547473508864641e-13))
        C = m.inv_mu + x.astype(np.float64) + y.astype(np.float64)
        Kref = (m.KtA * 1 / C).astype(f32)
        Gref = ((-1) * 2 / C * np.float64(L)).astype(f32)
    return np.where(okK, kh, Kref), np.where(okG, Gh, Gref), okK & okG, Kref, Gref


def coulomb_compare(Ftn, Fnn, m):
    t = f32(m.mu_f) * Fnn
    with np.errstate(invalid="ignore", over="ignore"):
        e = t * f32(4e-7)
        rng_ok = (t >= f32(1e-30)) & (t <= f32(1e30))
        X, P = Ftn.astype(np.float64), m.mu * Fnn.astype(np.float64)
        ref = np.where(X > P, 1, np.where(X <= P, 0, -1))
        got = np.where(rng_ok & (Ftn > t + e), 1, np.where(rng_ok & (Ftn < t - e), 0, ref))
    return got, ref


def bits_eq(a, b):
    a, b = np.asarray(a, f32), np.asarray(b, f32)
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_barycentric_weight_matches_double():
    rng = np.random.default_rng(11)
    n = 400000
    bw = np.concatenate([rng.uniform(-0.2, 1.2, n), rng.normal(0, 1e-9, n // 8), rng.lognormal(0, 8, n // 8)])
    bv = np.concatenate([rng.uniform(-0.2, 1.2, n), rng.uniform(0, 1, n // 8), -rng.lognormal(0, 8, n // 8)])
    bw, bv = bw.astype(f32), bv.astype(f32)
    # 1 - bw - bv at, and a few ulps either side of, float rounding midpoints
    tgt = rng.uniform(-1, 1, 20000).astype(f32)
    mid = tgt.astype(np.float64) + np.spacing(np.abs(tgt)).astype(np.float64) / 2
    bw2 = rng.uniform(-0.5, 1.5, 20000).astype(f32)
    bv2 = (1.0 - bw2.astype(np.float64) - mid).astype(f32)
    steps = np.arange(-3, 4)
    bw = np.concatenate([bw, np.repeat(bw2, len(steps)), np.array([0, 1e-40, 1, 2, 3e38, np.nan, np.inf, 1e-30], f32)])
    bv3 = np.stack([bv2 + f32(k) * np.spacing(np.abs(bv2)).astype(f32) for k in steps], 1).ravel()
    bv = np.concatenate([bv, bv3, np.array([0, 0, 1e-40, -1, -3e38, 0, 0, 1 - 1e-30], f32)])
    got, fast, ref = one_minus_two(bw, bv)
    assert bits_eq(got, ref)
    assert fast[:n].mean() > 0.999


def _materials():
    import ctypes
    from mwdiem_gb300 import _lib
    out = []
    for Kn, en, et, mu, Knw, enw, etw, muw in ((1e5, 0.372, 0.372, 0.5, 3e4, 0.5, 0.6, 0.3),
                                               (2e5, 0.2, 0.9, 0.4, 1e7, 0.05, 0.999, 1.7),
                                               (1e3, 0.8, 0.3, 0.05, 5e5, 0.3, 0.5, 0.9)):
        p = _lib.ContactParams(Kn, en, et, mu, Knw, enw, etw, muw, 5e-5, 4, 0, 0, 0)
        m = (_lib.Material * 2)()
        _lib.check(_lib.lib().mwd_derive_material(ctypes.byref(p), m))
        out += [m[0], m[1]]
    return out


def test_tangential_coefficients_match_double():
    rng = np.random.default_rng(12)
    n = 300000
    for m in _materials():
        x = np.concatenate([rng.lognormal(-2, 4, n), np.zeros(100), rng.uniform(0, 1, 1000)]).astype(f32)
        y = np.concatenate([rng.lognormal(-2, 4, n), rng.lognormal(0, 3, 100), np.zeros(1000)]).astype(f32)
        x = np.concatenate([x, np.array([np.inf, np.nan, 1e35, 0, 1e-40], f32)])
        y = np.concatenate([y, np.array([0, 0, 0, np.inf, 1e-40], f32)])
        K, G, fast, Kref, Gref = tangential_coeffs(m, x, y)
        assert bits_eq(K, Kref) and bits_eq(G, Gref)
        assert fast[:n].mean() > 0.999


def test_coulomb_compare_matches_double():
    rng = np.random.default_rng(13)
    n = 200000
    for m in _materials():
        Fnn = np.concatenate([rng.lognormal(0, 6, n), np.array([0, 0, 1e-40, np.inf, np.nan, 3e38, 1e-31])]).astype(f32)
        base = (f32(m.mu_f) * Fnn).astype(f32)
        # Ftn at and a few ulps either side of mu Fnn, and spread around it
        k = rng.integers(-6, 7, Fnn.shape)
        Ftn = np.where(rng.uniform(size=Fnn.shape) < 0.5, base + k.astype(f32) * np.spacing(np.abs(base)).astype(f32),
                       base * rng.uniform(0.5, 1.5, Fnn.shape).astype(f32)).astype(f32)
        Ftn[-7:] = np.array([0, 1, 0, np.inf, 1, np.nan, 1e-31], f32)
        got, ref = coulomb_compare(Ftn, Fnn, m)
        assert np.array_equal(got, ref)
