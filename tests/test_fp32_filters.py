"""Three of the reference's double-precision computations are decided in FP32 on the device (FP64
is slow on this GPU): CorrectFlat's +-1e-6 window (gpu_fine_contact_detection.cu:256-268), the EPA's
relative 1e-5 convergence test (.cu:439) and the cell coordinate trunc(p / cs) (MWDiem.py:813-816).
These restate the kernels' filters (narrow.cu within_1e6, epa_converged; broad.cu cell_coord) in
numpy float32 arithmetic, which rounds as the kernels do (no fused multiply-add), and check that they
give the double computations' answers on random and adversarial inputs."""
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
