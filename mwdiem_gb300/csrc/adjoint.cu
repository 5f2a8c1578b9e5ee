// Differentiable FP64 step and its hand-written adjoint (reverse mode).
//
// The contact topology of a step -- the pairs in contact and, for each, the support vertices of the
// final EPA face (three on A, three on B) -- is detected by the FP32 broad + narrow phase and logged.
// Given it, the step is a smooth map of the state:
//
//   face vertices   a_k = c_A + R(qacc_A) r0_A[fa_k],  b_k = c_B + R(qacc_B) r0_B[fb_k],  V_k = a_k - b_k
//   normal, depth   n0 = unit((V1 - V0) x (V2 - V1)) (the stored face order faces away from the
//                   origin), depth = n0 . V0           (AddTriangle, gpu_fine_contact_detection.cu:270-325)
//   contact points  barycentric weights of depth n0 on the face; cpA = sum w_k a_k, cpB = sum w_k b_k,
//                   weights (1 - w1 - w2, w1, w2) in the face's vertex order (.cu:548-600)
//   force, torque   spring-dashpot + Coulomb with zero tangential history (.cu:647-871; the reference
//                   wipes the history every step, MWDiem.py:966): row A gets Fn and (cp - cA) x Ff,
//                   row B gets -Fn and (cp - cB) x (-Ff), cp = (cpA - cpB)/2 as in the reference
//                   (.cu:677) or, on request, the midpoint (cpA + cpB)/2
//   integrator      the leapfrog of gpu_Verlet.cu:164-323 with q_acc <- unit(q q_acc) for the vertices
//
// pair_fwd / row_fwd evaluate it; pair_rev / row_rev apply the transposed Jacobian, derived by hand,
// to an upstream gradient, reusing the forward's intermediates (recomputed in the same thread, so
// no per-pair tape is stored).  Everything is FP64.  The force kernel and the pair adjoint add into
// per-row arrays with atomics; the law's gradient is reduced over a warp before its atomics.
#include "common.cuh"
#include "integrate.cuh"

namespace mwd {
namespace {

struct d3 {
    double x, y, z;
};
struct dq {
    double w, x, y, z;
};

__device__ __forceinline__ d3 D3(double x, double y, double z) { d3 r{x, y, z}; return r; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return D3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return D3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ d3 operator-(d3 a) { return D3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ d3 operator*(d3 a, double s) { return D3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ d3& operator+=(d3& a, d3 b) { a = a + b; return a; }
__device__ __forceinline__ d3& operator-=(d3& a, d3 b) { a = a - b; return a; }
__device__ __forceinline__ double dot3(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 cross3(d3 a, d3 b)
{
    return D3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ d3 had(d3 a, d3 b) { return D3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ d3 zero3() { return D3(0.0, 0.0, 0.0); }

__device__ __forceinline__ dq Q(double w, double x, double y, double z) { dq r{w, x, y, z}; return r; }
__device__ __forceinline__ dq operator+(dq a, dq b) { return Q(a.w + b.w, a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ dq& operator+=(dq& a, dq b) { a = a + b; return a; }
__device__ __forceinline__ dq operator*(dq a, double s) { return Q(a.w * s, a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double qdot(dq a, dq b) { return a.w * b.w + a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ dq conj(dq q) { return Q(q.w, -q.x, -q.y, -q.z); }
__device__ __forceinline__ d3 vec(dq q) { return D3(q.x, q.y, q.z); }
__device__ __forceinline__ dq pure(d3 v) { return Q(0.0, v.x, v.y, v.z); }
__device__ __forceinline__ dq zeroq() { return Q(0.0, 0.0, 0.0, 0.0); }
// Hamilton product, the operand order of the device quaternion product (vector part b a0 + a b0 + a x b)
__device__ __forceinline__ dq qmul(dq a, dq b)
{
    d3 u = vec(a), v = vec(b);
    d3 s = (v * a.w + u * b.w) + cross3(u, v);
    return Q(a.w * b.w - dot3(u, v), s.x, s.y, s.z);
}
// r = a b:  <gr, da b> = <gr conj(b), da>,  <gr, a db> = <conj(a) gr, db>
__device__ __forceinline__ void qmul_rev(dq a, dq b, dq gr, dq& ga, dq& gb)
{
    ga += qmul(gr, conj(b));
    gb += qmul(conj(a), gr);
}
// vector part of q1 (0, v) q2, evaluated as q1 ((0, v) q2)
__device__ __forceinline__ d3 qtrip(dq q1, d3 v, dq q2) { return vec(qmul(q1, qmul(pure(v), q2))); }
__device__ __forceinline__ void qtrip_rev(dq q1, d3 v, dq q2, d3 g, dq& gq1, d3& gv, dq& gq2)
{
    const dq P = pure(v);
    const dq m1 = qmul(P, q2);
    const dq gm2 = pure(g);
    dq gm1 = zeroq(), gP = zeroq();
    qmul_rev(q1, m1, gm2, gq1, gm1);
    qmul_rev(P, q2, gm1, gP, gq2);
    gv += vec(gP);
}

// R(q) r with the matrix of the device vertex pass (valid for unit q; a polynomial in q)
__device__ __forceinline__ d3 rotv(dq q, d3 r)
{
    const double w = q.w, x = q.x, y = q.y, z = q.z;
    return D3((1.0 - 2.0 * (y * y + z * z)) * r.x + 2.0 * (x * y - w * z) * r.y + 2.0 * (x * z + w * y) * r.z,
              2.0 * (x * y + w * z) * r.x + (1.0 - 2.0 * (x * x + z * z)) * r.y + 2.0 * (y * z - w * x) * r.z,
              2.0 * (x * z - w * y) * r.x + 2.0 * (y * z + w * x) * r.y + (1.0 - 2.0 * (x * x + y * y)) * r.z);
}
__device__ __forceinline__ dq rotv_rev(dq q, d3 r, d3 g)
{
    const double w = q.w, x = q.x, y = q.y, z = q.z;
    dq o;
    o.w = g.x * (-2.0 * z * r.y + 2.0 * y * r.z) + g.y * (2.0 * z * r.x - 2.0 * x * r.z) +
          g.z * (-2.0 * y * r.x + 2.0 * x * r.y);
    o.x = g.x * (2.0 * y * r.y + 2.0 * z * r.z) + g.y * (2.0 * y * r.x - 4.0 * x * r.y - 2.0 * w * r.z) +
          g.z * (2.0 * z * r.x + 2.0 * w * r.y - 4.0 * x * r.z);
    o.y = g.x * (-4.0 * y * r.x + 2.0 * x * r.y + 2.0 * w * r.z) + g.y * (2.0 * x * r.x + 2.0 * z * r.z) +
          g.z * (-2.0 * w * r.x + 2.0 * z * r.y - 4.0 * y * r.z);
    o.z = g.x * (-4.0 * z * r.x - 2.0 * w * r.y + 2.0 * x * r.z) + g.y * (2.0 * w * r.x - 4.0 * z * r.y + 2.0 * y * r.z) +
          g.z * (2.0 * x * r.x + 2.0 * y * r.y);
    return o;
}

// Rotation increment (cos th, sin(th) w / |w|), th = |w| s (gpu_Verlet.cu:200-214).
// k = sin(th)/|w| and h = (dk/d|w|)/|w| by their Taylor series in th^2 below 1e-6 (truncation
// below 1e-20 relative), so the map and its derivative stay smooth through w = 0.
struct Rot {
    double c, k, h;
};
__device__ __forceinline__ Rot rot_coef(d3 w, double s)
{
    const double w2 = dot3(w, w);
    const double t2 = w2 * s * s;
    Rot r;
    if (t2 < 1e-6) {
        r.c = 1.0 - t2 * 0.5 + t2 * t2 * (1.0 / 24.0);
        r.k = s * (1.0 - t2 * (1.0 / 6.0) + t2 * t2 * (1.0 / 120.0));
        r.h = s * s * s * (-1.0 / 3.0 + t2 * (1.0 / 30.0) - t2 * t2 * (1.0 / 840.0));
    } else {
        const double wn = sqrt(w2);
        const double th = wn * s;
        double sn, cs;
        sincos(th, &sn, &cs);
        r.c = cs;
        r.k = sn / wn;
        r.h = (th * cs - sn) / (w2 * wn);
    }
    return r;
}
__device__ __forceinline__ dq rot_apply(d3 w, const Rot& r) { return Q(r.c, w.x * r.k, w.y * r.k, w.z * r.k); }
// gradient of (c, k w) with respect to w:  dc/dw = -s k w,  d(k w)/dw = k I + h w w^T
__device__ __forceinline__ d3 rot_rev(d3 w, double s, const Rot& r, dq g)
{
    const d3 gv = vec(g);
    return w * (-s * r.k * g.w) + gv * r.k + w * (r.h * dot3(w, gv));
}

constexpr double kPi = 3.141592653589793;

// ------------------------------------------------------------------ pair map
struct PairIn {
    d3 cA, cB, vA, vB, wA, wB;
    dq qA, qB;
    d3 rA[3], rB[3];  // body-frame support vertices
    double IsA, IsB;
    double Kn, en, et, mu;
    double cps;  // contact point (cpA + cps cpB) / 2: -1 the reference's, +1 the midpoint
};

struct PairTape {
    d3 a[3], b[3], V[3];
    d3 e1, e2, m, n0, Pr, u1, w2;
    double l, depth;
    double d00, d01, d11, d20, d21, den, b0, b1, b2;
    d3 cpA, cpB, cp, dA, dB;
    double C, Len, Let, Xen, S, Gn, Gt, sgn;
    d3 n, rA, rB, u, un, ut;
    double uns;
    d3 Fn, Ft, Ff;
    double Fnn, utn;
    d3 th;
    bool slip;
    bool ok;
};

struct PairOut {
    d3 F, TA, TB;
};

__device__ __forceinline__ void pair_fwd(const PairIn& p, PairTape& t, PairOut& o)
{
    for (int k = 0; k < 3; ++k) {
        t.a[k] = p.cA + rotv(p.qA, p.rA[k]);
        t.b[k] = p.cB + rotv(p.qB, p.rB[k]);
        t.V[k] = t.a[k] - t.b[k];
    }
    t.e1 = t.V[1] - t.V[0];
    t.e2 = t.V[2] - t.V[1];
    t.m = cross3(t.e1, t.e2);
    t.l = sqrt(dot3(t.m, t.m));
    t.ok = t.l > 0.0;
    if (!t.ok) return;
    t.n0 = t.m * (1.0 / t.l);
    t.depth = dot3(t.n0, t.V[0]);
    t.Pr = t.n0 * t.depth;
    t.u1 = t.V[2] - t.V[0];
    t.w2 = t.Pr - t.V[0];
    t.d00 = dot3(t.e1, t.e1);
    t.d01 = dot3(t.e1, t.u1);
    t.d11 = dot3(t.u1, t.u1);
    t.d20 = dot3(t.w2, t.e1);
    t.d21 = dot3(t.w2, t.u1);
    t.den = t.d00 * t.d11 - t.d01 * t.d01;
    t.ok = t.den > 0.0;
    if (!t.ok) return;
    t.b1 = (t.d11 * t.d20 - t.d01 * t.d21) / t.den;
    t.b2 = (t.d00 * t.d21 - t.d01 * t.d20) / t.den;
    t.b0 = 1.0 - t.b2 - t.b1;
    t.cpA = (t.a[0] * t.b0 + t.a[1] * t.b1) + t.a[2] * t.b2;
    t.cpB = (t.b[0] * t.b0 + t.b[1] * t.b1) + t.b[2] * t.b2;
    t.cp = (t.cpA + t.cpB * p.cps) * 0.5;
    t.dA = t.cp - p.cA;
    t.dB = t.cp - p.cB;
    t.C = 1.0 / p.mu + dot3(t.dA, t.dA) / p.IsA + dot3(t.dB, t.dB) / p.IsB;
    t.Len = log(p.en);
    t.Let = log(p.et);
    t.Xen = t.Len * t.Len + kPi * kPi;
    // Gn = -2 mu Len / tc with tc = sqrt(mu Xen / Kn), i.e. -2 Len sqrt(mu Kn / Xen) (.cu:676-690)
    t.S = sqrt(p.mu * p.Kn / t.Xen);
    t.Gn = -2.0 * t.Len * t.S;
    t.Gt = -2.0 * t.Let / t.C;
    t.sgn = dot3(p.cB - p.cA, t.n0) < 0.0 ? -1.0 : 1.0;
    t.n = t.n0 * t.sgn;
    t.rA = t.cpA - p.cA;
    t.rB = t.cpB - p.cB;
    t.u = ((p.vA + cross3(p.wA, t.rA)) - p.vB) - cross3(p.wB, t.rB);
    t.uns = dot3(t.u, t.n);
    t.un = t.n * t.uns;
    t.ut = t.u - t.un;
    t.Fn = t.n * (-p.Kn * t.depth) - t.un * t.Gn;
    t.Fnn = sqrt(dot3(t.Fn, t.Fn));
    const d3 Ftl = t.ut * (-t.Gt);
    const double Ftn = sqrt(dot3(Ftl, Ftl));
    t.slip = Ftn > p.mu * t.Fnn;
    if (t.slip) {
        t.utn = sqrt(dot3(t.ut, t.ut));
        t.th = t.ut * (1.0 / t.utn);
        t.Ft = t.th * (-p.mu * t.Fnn);
    } else {
        t.utn = 0.0;
        t.th = zero3();
        t.Ft = Ftl;
    }
    t.Ff = t.Ft + t.Fn;
    o.F = t.Fn;
    o.TA = cross3(t.dA, t.Ff);
    o.TB = -cross3(t.dB, t.Ff);
}

struct PairGrad {
    d3 cA, cB, vA, vB, wA, wB;
    dq qA, qB;
    double Kn, en, et, mu;
};

// gF: gradient on F (row A's force; row B's is -F), gTA, gTB: on the torques
__device__ __forceinline__ void pair_rev(const PairIn& p, const PairTape& t, d3 gF, d3 gTA, d3 gTB, PairGrad& g)
{
    g.cA = g.cB = g.vA = g.vB = g.wA = g.wB = zero3();
    g.qA = g.qB = zeroq();
    g.Kn = g.en = g.et = g.mu = 0.0;
    if (!t.ok) return;
    // TA = dA x Ff, TB = -(dB x Ff)
    d3 gdA = cross3(t.Ff, gTA);
    d3 gFf = cross3(gTA, t.dA);
    d3 gdB = -cross3(t.Ff, gTB);
    gFf -= cross3(gTB, t.dB);
    d3 gFn = gF + gFf;
    const d3 gFt = gFf;
    d3 gut;
    double gGt = 0.0, gFnn = 0.0;
    if (t.slip) {
        // Ft = th (-mu Fnn), th = ut / |ut|
        const d3 gth = gFt * (-p.mu * t.Fnn);
        const double tg = dot3(t.th, gFt);
        g.mu += -t.Fnn * tg;
        gFnn = -p.mu * tg;
        gut = (gth - t.th * dot3(t.th, gth)) * (1.0 / t.utn);
    } else {
        // Ft = ut (-Gt)
        gut = gFt * (-t.Gt);
        gGt = -dot3(t.ut, gFt);
    }
    if (t.Fnn > 0.0) gFn += t.Fn * (gFnn / t.Fnn);
    // Fn = n (-Kn depth) - un Gn
    const double ng = dot3(t.n, gFn);
    d3 gn = gFn * (-p.Kn * t.depth);
    g.Kn += -t.depth * ng;
    double gdepth = -p.Kn * ng;
    d3 gun = gFn * (-t.Gn);
    const double gGn = -dot3(t.un, gFn);
    // ut = u - un, un = n uns, uns = u . n
    d3 gu = gut;
    gun -= gut;
    gn += gun * t.uns;
    const double guns = dot3(t.n, gun);
    gu += t.n * guns;
    gn += t.u * guns;
    // u = vA + wA x rA - vB - wB x rB
    g.vA = gu;
    g.vB = -gu;
    g.wA = cross3(t.rA, gu);
    const d3 grA = cross3(gu, p.wA);
    g.wB = -cross3(t.rB, gu);
    const d3 grB = -cross3(gu, p.wB);
    d3 gcpA = grA, gcpB = grB;
    g.cA -= grA;
    g.cB -= grB;
    // n = n0 sgn
    d3 gn0 = gn * t.sgn;
    // Gt = -2 Let / C
    double gC = gGt * 2.0 * t.Let / (t.C * t.C);
    const double gLet = gGt * (-2.0 / t.C);
    // Gn = -2 Len S, S = sqrt(mu Kn / Xen), Xen = Len^2 + pi^2
    const double gS = gGn * (-2.0 * t.Len);
    double gLen = gGn * (-2.0 * t.S);
    g.mu += gS * t.S / (2.0 * p.mu);
    g.Kn += gS * t.S / (2.0 * p.Kn);
    const double gXen = -gS * t.S / (2.0 * t.Xen);
    gLen += gXen * 2.0 * t.Len;
    g.en += gLen / p.en;
    g.et += gLet / p.et;
    // C = 1/mu + dA.dA / IsA + dB.dB / IsB
    g.mu += -gC / (p.mu * p.mu);
    gdA += t.dA * (2.0 * gC / p.IsA);
    gdB += t.dB * (2.0 * gC / p.IsB);
    // dA = cp - cA, dB = cp - cB, cp = (cpA + cps cpB) / 2
    const d3 gcp = gdA + gdB;
    g.cA -= gdA;
    g.cB -= gdB;
    gcpA += gcp * 0.5;
    gcpB += gcp * (0.5 * p.cps);
    // cpA = sum w_k a_k, cpB = sum w_k b_k
    d3 ga[3], gb[3];
    double gbeta[3];
    const double beta[3] = {t.b0, t.b1, t.b2};
    for (int k = 0; k < 3; ++k) {
        ga[k] = gcpA * beta[k];
        gb[k] = gcpB * beta[k];
        gbeta[k] = dot3(t.a[k], gcpA) + dot3(t.b[k], gcpB);
    }
    // w0 = 1 - w2 - w1, w1 = N1 / den, w2 = N2 / den
    const double gb1 = gbeta[1] - gbeta[0], gb2 = gbeta[2] - gbeta[0];
    const double gN1 = gb1 / t.den, gN2 = gb2 / t.den;
    const double gden = -(t.b1 * gb1 + t.b2 * gb2) / t.den;
    const double gd00 = gN2 * t.d21 + gden * t.d11;
    const double gd11 = gN1 * t.d20 + gden * t.d00;
    const double gd01 = -gN1 * t.d21 - gN2 * t.d20 - 2.0 * gden * t.d01;
    const double gd20 = gN1 * t.d11 - gN2 * t.d01;
    const double gd21 = -gN1 * t.d01 + gN2 * t.d00;
    d3 ge1 = t.e1 * (2.0 * gd00) + t.u1 * gd01 + t.w2 * gd20;
    const d3 gu1 = t.e1 * gd01 + t.u1 * (2.0 * gd11) + t.w2 * gd21;
    const d3 gw2 = t.e1 * gd20 + t.u1 * gd21;
    d3 gV[3];
    gV[0] = -gu1 - gw2;
    gV[1] = zero3();
    gV[2] = gu1;
    // w2 = Pr - V0, Pr = n0 depth, depth = n0 . V0
    gn0 += gw2 * t.depth;
    gdepth += dot3(t.n0, gw2);
    gn0 += t.V[0] * gdepth;
    gV[0] += t.n0 * gdepth;
    // n0 = m / l, m = e1 x e2
    const d3 gm = (gn0 - t.n0 * dot3(t.n0, gn0)) * (1.0 / t.l);
    ge1 += cross3(t.e2, gm);
    const d3 ge2 = cross3(gm, t.e1);
    // e1 = V1 - V0, e2 = V2 - V1
    gV[1] += ge1;
    gV[0] -= ge1;
    gV[2] += ge2;
    gV[1] -= ge2;
    for (int k = 0; k < 3; ++k) {
        ga[k] += gV[k];
        gb[k] -= gV[k];
        g.cA += ga[k];
        g.cB += gb[k];
        g.qA += rotv_rev(p.qA, p.rA[k], ga[k]);
        g.qB += rotv_rev(p.qB, p.rB[k], gb[k]);
    }
}

// ------------------------------------------------------------------ row map (integrator)
struct RowIn {
    d3 c, vh, whbf, wbf, w, F, T;
    dq q, qh, qa;
    d3 I, Ii;
    double invm;
};

struct RowTape {
    d3 v32, tbf, p1, p2, al, w32bf, dx, w34bf, w34, wbf2, w2, v2, c2;
    dq rho1, q32, rho2, qn, qraw, qa2;
    Rot r1, r2;
    double nq;
    bool reset;
};

__device__ __forceinline__ void row_fwd(const RowIn& r, double dt, const double* box, RowTape& t)
{
    const double k = r.invm * dt;
    t.v32 = r.vh + r.F * k;
    t.tbf = qtrip(conj(r.q), r.T, r.q);
    t.p1 = had(r.I, r.wbf);
    t.p2 = t.tbf - cross3(r.wbf, t.p1);
    t.al = had(r.Ii, t.p2);
    t.w32bf = r.whbf + t.al * dt;
    t.r1 = rot_coef(r.w, dt * 0.5);
    t.rho1 = rot_apply(r.w, t.r1);
    t.q32 = qmul(t.rho1, r.qh);
    t.dx = t.v32 * dt;
    t.w34bf = t.w32bf + t.al * (dt * 0.25);
    t.w34 = qtrip(t.q32, t.w34bf, conj(t.q32));
    t.r2 = rot_coef(t.w34, dt * 0.25);
    t.rho2 = rot_apply(t.w34, t.r2);
    t.qn = qmul(t.rho2, t.q32);
    t.wbf2 = t.w32bf + t.al * (dt * 0.5);
    t.w2 = qtrip(t.qn, t.wbf2, conj(t.qn));
    t.v2 = t.v32 + r.F * k;
    t.qraw = qmul(t.qn, r.qa);
    t.nq = sqrt(qdot(t.qraw, t.qraw));
    t.qa2 = t.qraw * (1.0 / t.nq);
    t.c2 = r.c + t.dx;
    // fly-away reset (gpu_Verlet.cu:338-352): stop the particle, undo the move
    t.reset = t.c2.x > box[0] || t.c2.x < box[1] || t.c2.y > box[2] || t.c2.y < box[3] || t.c2.z > box[4] ||
              t.c2.z < box[5];
}

struct RowGrad {
    d3 c, vh, whbf, wbf, w, F, T;
    dq q, qh, qa;
};

// lam: gradient on the outputs c, v, vh, whbf, wbf, w, q, qh, qa (row layout, 32 doubles)
__device__ __forceinline__ void row_rev(const RowIn& r, double dt, const RowTape& t, const double* lam, RowGrad& g)
{
    auto L3 = [&](int o) { return D3(lam[o], lam[o + 1], lam[o + 2]); };
    auto L4 = [&](int o) { return Q(lam[o], lam[o + 1], lam[o + 2], lam[o + 3]); };
    const double k = r.invm * dt;
    d3 gc2 = L3(0), gv2 = L3(3), gvh2 = L3(6), gwhbf2 = L3(9), gwbf2o = L3(12), gw2 = L3(15);
    dq gqn = L4(18), gq32 = L4(22), gqa2 = L4(26);
    d3 gdx = gc2;
    if (t.reset) {
        gv2 = gvh2 = gwhbf2 = gwbf2o = gw2 = zero3();
        gdx = zero3();
    }
    g.c = gc2;
    // qa2 = qraw / |qraw|, qraw = qn qa
    const dq gqraw = (gqa2 + t.qa2 * (-qdot(t.qa2, gqa2))) * (1.0 / t.nq);
    g.qa = zeroq();
    qmul_rev(t.qn, r.qa, gqraw, gqn, g.qa);
    // v2 = v32 + F k
    d3 gv32 = gvh2 + gv2;
    g.F = gv2 * k;
    // w2 = qtrip(qn, wbf2, conj(qn))
    {
        dq g1 = zeroq(), g2 = zeroq();
        d3 gv = zero3();
        qtrip_rev(t.qn, t.wbf2, conj(t.qn), gw2, g1, gv, g2);
        gqn += g1 + conj(g2);
        gwbf2o += gv;
    }
    // wbf2 = w32bf + al dt/2
    d3 gw32bf = gwhbf2 + gwbf2o;
    d3 gal = gwbf2o * (dt * 0.5);
    // qn = rho2 q32
    dq grho2 = zeroq();
    qmul_rev(t.rho2, t.q32, gqn, grho2, gq32);
    const d3 gw34 = rot_rev(t.w34, dt * 0.25, t.r2, grho2);
    // w34 = qtrip(q32, w34bf, conj(q32))
    d3 gw34bf = zero3();
    {
        dq g1 = zeroq(), g2 = zeroq();
        qtrip_rev(t.q32, t.w34bf, conj(t.q32), gw34, g1, gw34bf, g2);
        gq32 += g1 + conj(g2);
    }
    // w34bf = w32bf + al dt/4
    gw32bf += gw34bf;
    gal += gw34bf * (dt * 0.25);
    // dx = v32 dt
    gv32 += gdx * dt;
    // q32 = rho1 qh
    dq grho1 = zeroq();
    g.qh = zeroq();
    qmul_rev(t.rho1, r.qh, gq32, grho1, g.qh);
    g.w = rot_rev(r.w, dt * 0.5, t.r1, grho1);
    // w32bf = whbf + al dt
    g.whbf = gw32bf;
    gal += gw32bf * dt;
    // al = Ii o p2, p2 = tbf - wbf x p1, p1 = I o wbf
    const d3 gp2 = had(r.Ii, gal);
    const d3 gtbf = gp2;
    g.wbf = -cross3(t.p1, gp2);
    const d3 gp1 = -cross3(gp2, r.wbf);
    g.wbf += had(r.I, gp1);
    // tbf = qtrip(conj(q), T, q)
    {
        dq g1 = zeroq(), g2 = zeroq();
        d3 gT = zero3();
        qtrip_rev(conj(r.q), r.T, r.q, gtbf, g1, gT, g2);
        g.q = conj(g1) + g2;
        g.T = gT;
    }
    // v32 = vh + F k
    g.vh = gv32;
    g.F += gv32 * k;
}

__device__ __forceinline__ d3 ld3(const double* p) { return D3(p[0], p[1], p[2]); }
__device__ __forceinline__ dq ld4q(const double* p) { return Q(p[0], p[1], p[2], p[3]); }
__device__ __forceinline__ void st3(double* p, d3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
__device__ __forceinline__ void st4q(double* p, dq v) { p[0] = v.w; p[1] = v.x; p[2] = v.y; p[3] = v.z; }
__device__ __forceinline__ void add3(double* p, d3 v)
{
    atomicAdd(p, v.x);
    atomicAdd(p + 1, v.y);
    atomicAdd(p + 2, v.z);
}
__device__ __forceinline__ void add4q(double* p, dq v)
{
    atomicAdd(p, v.w);
    atomicAdd(p + 1, v.x);
    atomicAdd(p + 2, v.y);
    atomicAdd(p + 3, v.z);
}

// explicit steps are offset by *t_base when given; t < 0 reads the forward's device counter
__device__ __forceinline__ int step_of(const mwd_diff& d, int t)
{
    return t >= 0 ? t + (d.t_base ? *d.t_base : 0) : *d.t_dev;
}

__device__ __forceinline__ void load_pair_in(const mwd_diff& d, const double* x, const mwd_contact_rec& rc, PairIn& p,
                                             bool& wall)
{
    const int A = rc.A, B = rc.B;
    const double* xa = x + (size_t)MWD_DIFF_ROW * A;
    const double* xb = x + (size_t)MWD_DIFF_ROW * B;
    p.cA = ld3(xa);
    p.cB = ld3(xb);
    p.vA = ld3(xa + 3);
    p.vB = ld3(xb + 3);
    p.wA = ld3(xa + 15);
    p.wB = ld3(xb + 15);
    p.qA = ld4q(xa + 26);
    p.qB = ld4q(xb + 26);
    const float4* bv = reinterpret_cast<const float4*>(d.body_verts);
    const int oa = d.vert_off[A], ob = d.vert_off[B];
    for (int k = 0; k < 3; ++k) {
        const float4 ra = bv[oa + rc.fa[k]], rb = bv[ob + rc.fb[k]];
        p.rA[k] = D3(ra.x, ra.y, ra.z);
        p.rB[k] = D3(rb.x, rb.y, rb.z);
    }
    p.IsA = d.inertia[4 * A + 3];
    p.IsB = d.inertia[4 * B + 3];
    wall = (d.info[A] & 1) || (d.info[B] & 1);
    const double* L = d.law + (wall ? 4 : 0);
    p.Kn = L[0];
    p.en = L[1];
    p.et = L[2];
    p.mu = L[3];
    p.cps = d.contact_point == 1 ? 1.0 : -1.0;
}

__device__ __forceinline__ void load_row_in(const mwd_diff& d, const double* xr, const double* F, const double* T,
                                            int r, RowIn& in)
{
    in.c = ld3(xr);
    in.vh = ld3(xr + 6);
    in.whbf = ld3(xr + 9);
    in.wbf = ld3(xr + 12);
    in.w = ld3(xr + 15);
    in.q = ld4q(xr + 18);
    in.qh = ld4q(xr + 22);
    in.qa = ld4q(xr + 26);
    in.F = ld3(F);
    in.T = ld3(T);
    in.I = ld3(d.inertia + 4 * r);
    in.Ii = ld3(d.inv_inertia + 4 * r);
    in.invm = d.inv_inertia[4 * r + 3];
}

__device__ __forceinline__ int64_t log_count(const mwd_diff& d, int t)
{
    const int64_t off = d.step_off[t];
    const int64_t c = d.step_count[t];
    const int64_t room = d.rec_cap - off;
    return c < room ? c : (room > 0 ? room : 0);
}

// FP32 copies the detection reads: centre (pos.w, the bounding radius, is kept), velocities,
// quaternions and the world-frame vertices c + R(q_acc) r0
__device__ __forceinline__ void write_mirror(const mwd_state& m, int r, const double* row)
{
    double4* pos = reinterpret_cast<double4*>(m.pos);
    double4 pw = pos[r];
    pw.x = row[0];
    pw.y = row[1];
    pw.z = row[2];
    pos[r] = pw;
    reinterpret_cast<float4*>(m.vel)[r] = make_float4((float)row[3], (float)row[4], (float)row[5], 0.f);
    reinterpret_cast<float4*>(m.w)[r] = make_float4((float)row[15], (float)row[16], (float)row[17], 0.f);
    reinterpret_cast<float4*>(m.q)[r] = make_float4((float)row[18], (float)row[19], (float)row[20], (float)row[21]);
    reinterpret_cast<float4*>(m.q_acc)[r] = make_float4((float)row[26], (float)row[27], (float)row[28], (float)row[29]);
    reinterpret_cast<float4*>(m.force)[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    reinterpret_cast<float4*>(m.torque)[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (m.xform && m.vert_owner) {
        // the row transform for the per-vertex pass (launch_world_verts): R(q_acc) from the float
        // q_acc, as the device step forms it, and the centre as float hi + lo
        const float qw = (float)row[26], qx = (float)row[27], qy = (float)row[28], qz = (float)row[29];
        float x[16];
        x[0] = 1.f - 2.f * (qy * qy + qz * qz); x[1] = 2.f * (qx * qy - qw * qz); x[2] = 2.f * (qx * qz + qw * qy);
        x[3] = 2.f * (qx * qy + qw * qz); x[4] = 1.f - 2.f * (qx * qx + qz * qz); x[5] = 2.f * (qy * qz - qw * qx);
        x[6] = 2.f * (qx * qz - qw * qy); x[7] = 2.f * (qy * qz + qw * qx); x[8] = 1.f - 2.f * (qx * qx + qy * qy);
        for (int k = 0; k < 3; ++k) {
            const float hi = (float)row[k];
            x[9 + 2 * k] = hi;
            x[10 + 2 * k] = (float)(row[k] - (double)hi);
        }
        x[15] = 0.f;
        float4* o = reinterpret_cast<float4*>(m.xform) + 4 * (size_t)r;
        o[0] = make_float4(x[0], x[1], x[2], x[3]);
        o[1] = make_float4(x[4], x[5], x[6], x[7]);
        o[2] = make_float4(x[8], x[9], x[10], x[11]);
        o[3] = make_float4(x[12], x[13], x[14], x[15]);
        return;
    }
    const dq qa = ld4q(row + 26);
    const d3 c = ld3(row);
    const float4* bv = reinterpret_cast<const float4*>(m.body_verts);
    float4* wv = reinterpret_cast<float4*>(m.world_verts);
    for (int j = m.vert_off[r]; j < m.vert_off[r + 1]; ++j) {
        const float4 b = bv[j];
        const d3 v = c + rotv(qa, D3(b.x, b.y, b.z));
        wv[j] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
    }
}

}  // namespace

// ------------------------------------------------------------------ kernels

__global__ void diff_collect_kernel(mwd_diff d, const int2* __restrict__ pairs, const int64_t* __restrict__ n_pairs,
                                    const int32_t* __restrict__ collision, const int32_t* __restrict__ face_ids)
{
    const int t = *d.t_dev;
    if (t >= d.n_steps) return;
    const int64_t np = *n_pairs;
    const int64_t base = d.step_off[t];
    const int lane = threadIdx.x & 31;
    for (int64_t P0 = (int64_t)blockIdx.x * blockDim.x; P0 < np; P0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = P0 + threadIdx.x;
        const bool hit = P < np && collision[P] == 1;
        const unsigned b = __ballot_sync(0xffffffffu, hit);
        if (!b) continue;
        int first = 0;
        if (lane == 0) first = atomicAdd(d.step_count + t, __popc(b));
        first = __shfl_sync(0xffffffffu, first, 0);
        if (hit) {
            const int64_t slot = base + first + __popc(b & ((1u << lane) - 1u));
            if (slot < d.rec_cap) {
                const int2 pr = pairs[P];
                const int32_t* f = face_ids + 6 * P;
                mwd_contact_rec rc;
                rc.A = pr.x;
                rc.B = pr.y;
                rc.fa[0] = f[0]; rc.fa[1] = f[1]; rc.fa[2] = f[2];
                rc.fb[0] = f[3]; rc.fb[1] = f[4]; rc.fb[2] = f[5];
                d.rec[slot] = rc;
            } else {
                set_status(d.status, MWD_ST_LOG_OVERFLOW);
            }
        }
    }
}

__global__ void diff_force_kernel(mwd_diff d, const double* __restrict__ x, int t_arg)
{
    const int t = step_of(d, t_arg);
    if (t >= d.n_steps) return;
    const int64_t cnt = log_count(d, t);
    const int64_t off = d.step_off[t];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
        const mwd_contact_rec rc = d.rec[off + i];
        PairIn p;
        bool wall;
        load_pair_in(d, x, rc, p, wall);
        PairTape tp;
        PairOut o;
        pair_fwd(p, tp, o);
        if (!tp.ok) {
            set_status(d.status, MWD_ST_DEGENERATE_FACE);
            continue;
        }
        if (!(d.info[rc.A] & 1)) {
            add3(d.F + 4 * rc.A, o.F);
            add3(d.T + 4 * rc.A, o.TA);
        }
        if (!(d.info[rc.B] & 1)) {
            add3(d.F + 4 * rc.B, -o.F);
            add3(d.T + 4 * rc.B, o.TB);
        }
    }
}

// FP64-heavy row kernels: small blocks spread a few thousand rows over many SMs (GB300's FP64
// pipe is narrow, so rows per SM, not occupancy, set the time)
constexpr int DIFF_RB = 32;

__global__ void __launch_bounds__(DIFF_RB) diff_integrate_kernel(mwd_diff d, const double* __restrict__ x, double* xo,
                                                                 double* FT_store, mwd_state mirror, int has_mirror,
                                                                 int t_arg)
{
    __shared__ double s_com[3][DIFF_RB / 32];
    __shared__ bool s_last;
    const int t = step_of(d, t_arg);
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    d3 cnew = zero3();
    bool particle = false;
    if (r < d.n && t < d.n_steps) {
        const double* xr = x + (size_t)MWD_DIFF_ROW * r;
        double* xw = xo + (size_t)MWD_DIFF_ROW * r;
        double row[MWD_DIFF_ROW];
        for (int k = 0; k < MWD_DIFF_ROW; ++k) row[k] = xr[k];
        if (!(d.info[r] & 1)) {
            particle = true;
            double F[3], T[3];
            for (int k = 0; k < 3; ++k) {
                F[k] = d.F[4 * r + k] + d.ext[4 * r + k];
                T[k] = d.T[4 * r + k];
            }
            RowIn in;
            load_row_in(d, row, F, T, r, in);
            RowTape tp;
            row_fwd(in, d.dt, d.box, tp);
            if (tp.reset) {
                set_status(d.status, MWD_ST_FLY_RESET);
                for (int k = 3; k < 18; ++k) row[k] = 0.0;
            } else {
                st3(row + 0, tp.c2);
                st3(row + 3, tp.v2);
                st3(row + 6, tp.v32);
                st3(row + 9, tp.w32bf);
                st3(row + 12, tp.wbf2);
                st3(row + 15, tp.w2);
            }
            st4q(row + 18, tp.qn);
            st4q(row + 22, tp.q32);
            st4q(row + 26, tp.qa2);
            if (FT_store) {
                double* o = FT_store + 8 * (size_t)r;
                o[0] = F[0]; o[1] = F[1]; o[2] = F[2]; o[3] = 0.0;
                o[4] = T[0]; o[5] = T[1]; o[6] = T[2]; o[7] = 0.0;
            }
            for (int k = 0; k < 4; ++k) {
                d.F[4 * r + k] = 0.0;
                d.T[4 * r + k] = 0.0;
            }
            cnew = ld3(row);
        }
        for (int k = 0; k < MWD_DIFF_ROW; ++k) xw[k] = row[k];
        if (t_arg < 0 && d.ckpt && d.ckpt_every > 0 && (t + 1) % d.ckpt_every == 0) {
            double* ck = d.ckpt + ((size_t)((t + 1) / d.ckpt_every) * d.n + r) * MWD_DIFF_ROW;
            for (int k = 0; k < MWD_DIFF_ROW; ++k) ck[k] = row[k];
        }
        if (has_mirror) write_mirror(mirror, r, row);
    }
    if (t_arg >= 0) return;
    // centre of mass after step t, then the step advance by the last block to finish
    if (d.com && t < d.n_steps) {
        d3 v = particle ? cnew : zero3();
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
            v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
        }
        if ((threadIdx.x & 31) == 0) {
            s_com[0][threadIdx.x >> 5] = v.x;
            s_com[1][threadIdx.x >> 5] = v.y;
            s_com[2][threadIdx.x >> 5] = v.z;
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            double s = 0.0;
            for (int w = 0; w < DIFF_RB / 32; ++w) s += s_com[threadIdx.x][w];
            atomicAdd(d.com + 4 * (size_t)t + threadIdx.x, s / d.n_particles);
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(d.sync, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        if (t < d.n_steps) {
            d.step_off[t + 1] = d.step_off[t] + log_count(d, t);
            *d.t_dev = t + 1;
        }
        *d.sync = 0u;
    }
}

__global__ void diff_mirror_kernel(mwd_diff d, const double* __restrict__ x, mwd_state mirror)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= d.n) return;
    write_mirror(mirror, r, x + (size_t)MWD_DIFF_ROW * r);
}

// lam_prev = (d step / d state)^T lam for the integrator part; gFT = gradient on the step's F, T
__global__ void __launch_bounds__(DIFF_RB) adj_integrate_kernel(mwd_diff d, const double* __restrict__ x,
                                                                const double* __restrict__ FT, int t_arg,
                                                                const double* __restrict__ lam, double* lam_prev,
                                                                const double* __restrict__ com_grad, double* gFT)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = step_of(d, t_arg);
    if (r >= d.n || t >= d.n_steps) return;
    double* lp = lam_prev + (size_t)MWD_DIFF_ROW * r;
    double* gft = gFT + 8 * (size_t)r;
    if (d.info[r] & 1) {
        for (int k = 0; k < MWD_DIFF_ROW; ++k) lp[k] = 0.0;
        for (int k = 0; k < 8; ++k) gft[k] = 0.0;
        return;
    }
    double row[MWD_DIFF_ROW], up[MWD_DIFF_ROW];
    const double* xr = x + (size_t)MWD_DIFF_ROW * r;
    const double* lr = lam + (size_t)MWD_DIFF_ROW * r;
    for (int k = 0; k < MWD_DIFF_ROW; ++k) {
        row[k] = xr[k];
        up[k] = lr[k];
    }
    if (com_grad) {
        const double s = 1.0 / d.n_particles;
        up[0] += com_grad[4 * (size_t)t + 0] * s;
        up[1] += com_grad[4 * (size_t)t + 1] * s;
        up[2] += com_grad[4 * (size_t)t + 2] * s;
    }
    const double* ft = FT + 8 * (size_t)r;
    RowIn in;
    load_row_in(d, row, ft, ft + 4, r, in);
    RowTape tp;
    row_fwd(in, d.dt, d.box, tp);
    RowGrad g;
    row_rev(in, d.dt, tp, up, g);
    st3(lp + 0, g.c);
    st3(lp + 3, zero3());
    st3(lp + 6, g.vh);
    st3(lp + 9, g.whbf);
    st3(lp + 12, g.wbf);
    st3(lp + 15, g.w);
    st4q(lp + 18, g.q);
    st4q(lp + 22, g.qh);
    st4q(lp + 26, g.qa);
    lp[30] = lp[31] = 0.0;
    st3(gft, g.F);
    gft[3] = 0.0;
    st3(gft + 4, g.T);
    gft[7] = 0.0;
}

__global__ void adj_force_kernel(mwd_diff d, const double* __restrict__ x, int t_arg, const double* __restrict__ gFT,
                                 double* lam_prev, double* glaw)
{
    const int t = step_of(d, t_arg);
    if (t >= d.n_steps) return;
    const int64_t cnt = log_count(d, t);
    const int64_t off = d.step_off[t];
    double gl[8];
    for (int k = 0; k < 8; ++k) gl[k] = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t i = i0; i < cnt; i += stride) {
        const mwd_contact_rec rc = d.rec[off + i];
        PairIn p;
        bool wall;
        load_pair_in(d, x, rc, p, wall);
        PairTape tp;
        PairOut o;
        pair_fwd(p, tp, o);
        if (!tp.ok) continue;
        const bool wa = d.info[rc.A] & 1, wb = d.info[rc.B] & 1;
        const double* ga = gFT + 8 * (size_t)rc.A;
        const double* gb = gFT + 8 * (size_t)rc.B;
        d3 gF = zero3(), gTA = zero3(), gTB = zero3();
        if (!wa) {
            gF += ld3(ga);
            gTA = ld3(ga + 4);
        }
        if (!wb) {
            gF -= ld3(gb);
            gTB = ld3(gb + 4);
        }
        PairGrad g;
        pair_rev(p, tp, gF, gTA, gTB, g);
        if (!wa) {
            double* l = lam_prev + (size_t)MWD_DIFF_ROW * rc.A;
            add3(l + 0, g.cA);
            add3(l + 3, g.vA);
            add3(l + 15, g.wA);
            add4q(l + 26, g.qA);
        }
        if (!wb) {
            double* l = lam_prev + (size_t)MWD_DIFF_ROW * rc.B;
            add3(l + 0, g.cB);
            add3(l + 3, g.vB);
            add3(l + 15, g.wB);
            add4q(l + 26, g.qB);
        }
        const int o4 = wall ? 4 : 0;
        gl[o4 + 0] += g.Kn;
        gl[o4 + 1] += g.en;
        gl[o4 + 2] += g.et;
        gl[o4 + 3] += g.mu;
    }
    // every lane of the warp reaches the reduction (the loop above has no early return)
    for (int k = 0; k < 8; ++k) {
        double v = gl[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(glaw + k, v);
    }
}

}  // namespace mwd

using namespace mwd;

static bool diff_ok(const mwd_diff* d, const char* who)
{
    if (!d || d->n < 0 || !d->inertia || !d->inv_inertia || !d->ext || !d->body_verts || !d->vert_off || !d->info ||
        !d->law || !d->F || !d->T || !d->rec || !d->step_off || !d->step_count || !d->t_dev || !d->sync ||
        d->n_particles < 1 || d->n_steps < 0 || d->rec_cap < 0 || d->contact_point < 0 || d->contact_point > 1) {
        set_error("%s: incomplete mwd_diff", who);
        return false;
    }
    return true;
}

extern "C" {

int mwd_diff_collect(const mwd_diff* d, const mwd_work* work, mwd_stream_t stream)
{
    if (!diff_ok(d, "mwd_diff_collect")) return MWD_ERR_INVALID;
    if (!work || !work->pairs || !work->n_pairs || !work->collision || !work->face_ids || work->pair_cap < 0) {
        set_error("mwd_diff_collect: work needs pairs, n_pairs, collision and face_ids");
        return MWD_ERR_INVALID;
    }
    if (work->pair_cap == 0) return MWD_OK;
    int64_t b = (work->pair_cap + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 2;
    if (b > cap) b = cap;
    diff_collect_kernel<<<(int)b, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        *d, reinterpret_cast<const int2*>(work->pairs), work->n_pairs, work->collision, work->face_ids);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

int mwd_diff_force(const mwd_diff* d, const double* x, int32_t t, mwd_stream_t stream)
{
    if (!diff_ok(d, "mwd_diff_force")) return MWD_ERR_INVALID;
    if (!x || t >= d->n_steps) {
        set_error("mwd_diff_force: bad arguments");
        return MWD_ERR_INVALID;
    }
    // the contact count lives on the device: one block per SM strides through the step's records
    diff_force_kernel<<<num_sms(), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*d, x, t);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

int mwd_diff_integrate(const mwd_diff* d, const double* x, double* x_out, double* FT_store, mwd_state* mirror,
                       int32_t t, mwd_stream_t stream)
{
    if (!diff_ok(d, "mwd_diff_integrate")) return MWD_ERR_INVALID;
    if (!x || !x_out || t >= d->n_steps) {
        set_error("mwd_diff_integrate: bad arguments");
        return MWD_ERR_INVALID;
    }
    if (d->n == 0) return MWD_OK;
    mwd_state m = {};
    if (mirror) {
        if (mirror->n != d->n || !mirror->pos || !mirror->vel || !mirror->w || !mirror->q || !mirror->q_acc ||
            !mirror->force || !mirror->torque || !mirror->body_verts || !mirror->world_verts || !mirror->vert_off) {
            set_error("mwd_diff_integrate: mirror state does not match");
            return MWD_ERR_INVALID;
        }
        m = *mirror;
    }
    const int blocks = (d->n + DIFF_RB - 1) / DIFF_RB;
    diff_integrate_kernel<<<blocks, DIFF_RB, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*d, x, x_out, FT_store, m,
                                                                                        mirror ? 1 : 0, t);
    MWD_CUDA(cudaGetLastError());
    if (mirror && m.xform && m.vert_owner) return launch_world_verts(m, reinterpret_cast<cudaStream_t>(stream));
    return MWD_OK;
}

int mwd_diff_mirror(const mwd_diff* d, const double* x, mwd_state* mirror, mwd_stream_t stream)
{
    if (!diff_ok(d, "mwd_diff_mirror")) return MWD_ERR_INVALID;
    if (!x || !mirror || mirror->n != d->n || !mirror->pos || !mirror->vel || !mirror->w || !mirror->q ||
        !mirror->q_acc || !mirror->force || !mirror->torque || !mirror->body_verts || !mirror->world_verts ||
        !mirror->vert_off) {
        set_error("mwd_diff_mirror: bad arguments");
        return MWD_ERR_INVALID;
    }
    if (d->n == 0) return MWD_OK;
    diff_mirror_kernel<<<(d->n + 127) / 128, 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*d, x, *mirror);
    MWD_CUDA(cudaGetLastError());
    if (mirror->xform && mirror->vert_owner) return launch_world_verts(*mirror, reinterpret_cast<cudaStream_t>(stream));
    return MWD_OK;
}

int mwd_diff_adjoint(const mwd_diff* d, const double* x, const double* FT, int32_t t, const double* lam,
                     double* lam_prev, const double* com_grad, double* gFT, double* glaw, mwd_stream_t stream)
{
    if (!diff_ok(d, "mwd_diff_adjoint")) return MWD_ERR_INVALID;
    if (!x || !FT || !lam || !lam_prev || !gFT || !glaw || t < 0 || t >= d->n_steps || lam == lam_prev) {
        set_error("mwd_diff_adjoint: bad arguments");
        return MWD_ERR_INVALID;
    }
    if (d->n == 0) return MWD_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    adj_integrate_kernel<<<(d->n + DIFF_RB - 1) / DIFF_RB, DIFF_RB, 0, s>>>(*d, x, FT, t, lam, lam_prev, com_grad, gFT);
    MWD_CUDA(cudaGetLastError());
    adj_force_kernel<<<num_sms(), 128, 0, s>>>(*d, x, t, gFT, lam_prev, glaw);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

}  // extern "C"
