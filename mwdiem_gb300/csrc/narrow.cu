// Narrow phase (GJK + EPA) and contact force, warp-cooperative, for sm_103a.
//
// Algorithm: LIBRARIES/gpu_fine_contact_detection.cu (GJK driver :996-1288, simplex tests :103-268,
// EPA :270-603, force :647-871).  The decisions and the floating-point operation sequence are the
// reference's, so contact flags, depths, normals and forces round exactly as the reference kernel
// evaluated without FMA contraction.  The execution model is not:
//
//  * a group of LPP lanes (4/8/16/32) works on one pair; a block holds 128/LPP groups and the grid
//    strides over the pair list.  The device step runs two passes: GJK (gjk_pass_kernel, also one
//    lane per pair) writes the pairs in contact with the simplex it stopped on to a list, and EPA
//    with the force (epa_pass_kernel) continues from that list with its own lanes per pair;
//  * a support query is a strided scan of the float4 hull vertices (staged in shared memory, or read
//    in place from the L1-cached vertex table) by the group's lanes, then a group argmax on (value
//    desc, index asc), which reproduces the reference's strict-'>' first-index tie break;
//  * the simplex logic runs redundantly (identically) on every lane of the group, so control flow
//    stays group-uniform;
//  * EPA keeps an append-only face list of MWD_EPA_FACE_CAP faces in shared memory, like the
//    reference's T[50]/n[50]/dist[50] (which overflow past 50 faces); a pair that outgrows it runs
//    again with the deleted faces removed from the list (epa_compacting); the face scan, the
//    visibility test, the horizon edge count (the reference's 50x50 delpair matrix, replaced by
//    counting over the deleted-face list) and the new faces are computed lane-parallel, with ballots
//    to keep the reference's face order;
//  * force/torque are accumulated with float atomics (skipped for wall rows in table mode, whose
//    forces the reference discards, MWDiem.py:977-978).
#include <float.h>

#include "common.cuh"
#include "narrow.cuh"

namespace mwd {

namespace {

constexpr int FCAP = MWD_EPA_FACE_CAP;
constexpr int VCAP = MWD_EPA_VERT_CAP;

// per-group shared memory (the hull staging area follows, 2 * hull_cap float4)
struct EpaMem {
    float4 fn[FCAP];       // face normal xyz, distance
    uint32_t ft[FCAP];     // T0 | T1 << 8 | T2 << 16 | (valid + 2) << 24
    float4 pv[VCAP];       // polytope vertices
    uint16_t pab[VCAP];    // support index on A | on B << 8
    uint32_t del[FCAP];    // faces deleted in this iteration, in index order: vertices T0 T1 T2 | face << 24
};

__device__ __forceinline__ int ft_v(uint32_t t, int k) { return (t >> (8 * k)) & 0xff; }
__device__ __forceinline__ int ft_valid(uint32_t t) { return (int)(t >> 24) - 2; }
__device__ __forceinline__ uint32_t ft_make(int a, int b, int c, int valid)
{
    return (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c << 16) | ((uint32_t)(valid + 2) << 24);
}

template <int LPP>
struct Group {
    int lane;
    unsigned mask;
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ unsigned ballot(bool p) const
    {
        unsigned b = __ballot_sync(mask, p);
        if (LPP < 32) b = (b & mask) >> (__ffs(mask) - 1);
        return b;
    }
    __device__ __forceinline__ unsigned lt_mask() const { return (1u << lane) - 1u; }
};

// Order-preserving key of a float (-0 and +0 share the key of +0, as they compare equal): the
// group reductions below run on these keys with redux.sync.
__device__ __forceinline__ unsigned fkey(float f)
{
    f = (f == 0.f) ? 0.f : f;
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Group-wide (largest value, then smallest index) of the lanes' (v, i), v not NaN: the sequential
// "v > best" scan's first-index result when each lane holds its own first-index best.
template <int LPP>
__device__ __forceinline__ int group_argmax(const Group<LPP>& g, float v, int i)
{
    if (LPP == 1) return i;  // one lane per pair: its own scan is the sequential one
    const unsigned k = fkey(v);
    const unsigned km = __reduce_max_sync(g.mask, k);
    return (int)__reduce_min_sync(g.mask, k == km ? (unsigned)i : 0xffffffffu);
}

// Work queue of the EPA pass: a 64-bit counter after the EPA record count in the block epa_count points
// to (MWD_EPA_COUNT_INTS ints, 8-byte aligned), ints [2..3].  Zeroed with the record count before
// each narrow phase.
__device__ __forceinline__ unsigned long long* epa_queue(const NarrowArgs& a)
{
    return reinterpret_cast<unsigned long long*>(a.epa_count + 2);
}

// EPA records whose face list overflowed, run again by epa_retry_kernel after the EPA pass: their
// count at int [4] of the block epa_count points to, the record indices from int [8]
constexpr int EPA_RETRY_CAP = MWD_EPA_COUNT_INTS - 8;
__device__ __forceinline__ int* epa_retry_count(const NarrowArgs& a) { return a.epa_count + 4; }
__device__ __forceinline__ int32_t* epa_retry_list(const NarrowArgs& a) { return a.epa_count + 8; }

// The next `amount` items of a queue for the calling group: its first lane takes them with one atomic.
template <int LPP>
__device__ __forceinline__ int64_t claim(const Group<LPP>& g, unsigned long long* next, int64_t amount)
{
    unsigned long long base = 0;
    if (g.lane == 0) base = atomicAdd(next, (unsigned long long)amount);
    return (int64_t)__shfl_sync(g.mask, base, (int)(threadIdx.x & 31) - g.lane);
}

// argmax of d.a over A and of (-d).b over B, first index on ties (.cu:55-101)
// work counted per pair when the caller asks for it: vertex dot products, EPA faces, support queries
struct Work3 {
    uint32_t dots, faces, queries;
};

template <int LPP>
__device__ __forceinline__ void support(const Group<LPP>& g, const float4* hA, int nA, const float4* hB, int nB,
                                        f3 d, f3& s, int& ia, int& ib, Work3& wk)
{
    wk.dots += (uint32_t)(nA + nB);
    wk.queries += 1;
    float bA = -1e30f, bB = -1e30f;
    int iA = 0, iB = 0;
    // unrolled so that several vertex loads are in flight (the scan order, and so the result, is
    // unchanged)
#pragma unroll 4
    for (int i = g.lane; i < nA; i += LPP) {
        float4 v = hA[i];
        float t = d.x * v.x + d.y * v.y + d.z * v.z;
        if (t > bA) { bA = t; iA = i; }
    }
    f3 nd = d * (-1.f);
#pragma unroll 4
    for (int j = g.lane; j < nB; j += LPP) {
        float4 v = hB[j];
        float t = nd.x * v.x + nd.y * v.y + nd.z * v.z;
        if (t > bB) { bB = t; iB = j; }
    }
    iA = group_argmax<LPP>(g, bA, iA);
    iB = group_argmax<LPP>(g, bB, iB);
    ia = iA;
    ib = iB;
    float4 a = hA[iA], b = hB[iB];
    s = mk3(a.x - b.x, a.y - b.y, a.z - b.z);
}

// The first two support queries of GJK, in directions d1 and d2 = -d1, in one pass over the hulls:
// the same dot products, maxima and first-index ties as two calls of support() (the A side of d2
// and the B side of d1 both use -d1 = d1 * -1, the B side of d2 uses d2 * -1 = d1), so the results
// are those two calls'.  The second query's latency overlaps the first's; the caller counts it as
// work only when GJK gets that far.
template <int LPP>
__device__ __forceinline__ void support_pair(const Group<LPP>& g, const float4* hA, int nA, const float4* hB, int nB,
                                             f3 d1, f3& S1, int& a1, int& b1, f3& S2, int& a2, int& b2)
{
    const f3 n1 = d1 * (-1.f);
    float tA = -1e30f, uA = -1e30f, tB = -1e30f, uB = -1e30f;
    int itA = 0, iuA = 0, itB = 0, iuB = 0;
#pragma unroll 4
    for (int i = g.lane; i < nA; i += LPP) {
        const float4 v = hA[i];
        const float t = d1.x * v.x + d1.y * v.y + d1.z * v.z;
        const float u = n1.x * v.x + n1.y * v.y + n1.z * v.z;
        if (t > tA) { tA = t; itA = i; }
        if (u > uA) { uA = u; iuA = i; }
    }
#pragma unroll 4
    for (int j = g.lane; j < nB; j += LPP) {
        const float4 v = hB[j];
        const float t = d1.x * v.x + d1.y * v.y + d1.z * v.z;
        const float u = n1.x * v.x + n1.y * v.y + n1.z * v.z;
        if (t > tB) { tB = t; itB = j; }
        if (u > uB) { uB = u; iuB = j; }
    }
    a1 = group_argmax<LPP>(g, tA, itA);  // support(d1): argmax d1.a, argmax (-d1).b
    b1 = group_argmax<LPP>(g, uB, iuB);
    a2 = group_argmax<LPP>(g, uA, iuA);  // support(d2): argmax (-d1).a, argmax d1.b
    b2 = group_argmax<LPP>(g, tB, itB);
    const float4 p1 = hA[a1], q1 = hB[b1], p2 = hA[a2], q2 = hB[b2];
    S1 = mk3(p1.x - q1.x, p1.y - q1.y, p1.z - q1.z);
    S2 = mk3(p2.x - q2.x, p2.y - q2.y, p2.z - q2.z);
}

// ---- simplex tests, identical on every lane (.cu:103-268) ----
__device__ __forceinline__ void seg_test(f3 P1, f3 P2, int& coll, f3& d)
{
    coll = -1;
    d = mk3(0.f, 0.f, 0.f);
    f3 e = P2 - P1;
    if (dot(e, P2) < 0.f) { coll = 0; return; }
    f3 t = cross(e, P2);
    if (t.x == 0.f && t.y == 0.f && t.z == 0.f) { coll = 1; return; }
    f3 tmp = cross(e, P2 * (-1.f));
    d = cross(tmp, e);
}

__device__ __forceinline__ void tri_test(f3 P1, f3 P2, f3 P3, int& coll, f3& d)
{
    coll = -1;
    d = mk3(0.f, 0.f, 0.f);
    int c2, c3;
    seg_test(P2, P3, c2, d);
    if (c2 == 1) { coll = 1; return; }
    seg_test(P1, P3, c3, d);
    if (c3 == 1) { coll = 1; return; }
    if (c2 + c3 > -1) { coll = 0; return; }
    f3 e32 = P3 - P2, e13 = P1 - P3;
    f3 n = cross(e32, e13);
    f3 n2 = cross(e32, n);
    f3 n3 = cross(e13, n);
    if (dot(n2, P2) < 0.f) { d = n2; return; }
    if (dot(n3, P3) < 0.f) { d = n3; return; }
    if (dot(P3, n) == 0.f) { coll = 1; return; }
    if (dot(n, P3) > 0.f) d = n * (-1.f);
    else d = n;
}

__device__ __forceinline__ void tet_test(f3 P1, f3 P2, f3 P3, f3 P4, int& coll, f3& d, int& todel)
{
    coll = -1;
    d = mk3(0.f, 0.f, 0.f);
    todel = 0;
    int c1, c2, c3;
    tri_test(P1, P2, P4, c1, d);
    if (c1 == 1) { coll = 1; return; }
    tri_test(P2, P3, P4, c2, d);
    if (c2 == 1) { coll = 1; return; }
    tri_test(P3, P1, P4, c3, d);
    if (c3 == 1) { coll = 1; return; }
    if (c1 + c2 + c3 > -2) { coll = 0; return; }
    f3 e13 = P1 - P3, e21 = P2 - P1, e32 = P3 - P2, e41 = P4 - P1;
    f3 n2 = cross(e21, e41);
    f3 e42 = P4 - P2;
    f3 n3 = cross(e32, e42);
    f3 e43 = P4 - P3;
    f3 n4 = cross(e13, e43);
    if (dot(n2, P4) < 0.f) { d = n2; todel = 3; }
    else if (dot(n3, P4) < 0.f) { d = n3; todel = 1; }
    else if (dot(n4, P4) < 0.f) { d = n4; todel = 2; }
    else coll = 1;
}

// (double)v < 1e-6 && (double)v > -1e-6 for a float v, without FP64: a float compares with the
// double 1e-6 as it compares with the smallest float not below it (0x358637be); NaN fails both
__device__ __forceinline__ bool within_1e6(float v)
{
    const float F = __uint_as_float(0x358637beu);
    return v < F && v > -F;
}

// CorrectFlat: both determinants inside a double +-1e-6 window (.cu:256-268)
__device__ __forceinline__ bool is_flat(f3 S1, f3 S2, f3 S3, f3 S4)
{
    float det1 = S1.x * (S2.y * S3.z - S3.y * S2.z) - S2.x * (S1.y * S3.z - S3.y * S1.z) + S3.x * (S1.y * S2.z - S2.y * S1.z);
    if (within_1e6(det1)) {
        float det2 = S1.x * (S2.y * S4.z - S4.y * S2.z) - S2.x * (S1.y * S4.z - S4.y * S1.z) + S4.x * (S1.y * S2.z - S2.y * S1.z);
        if (within_1e6(det2)) return true;
    }
    return false;
}

// The EPA's convergence test (.cu:439), (double)x * 1.00001 > (double)p && (double)x * 0.99999 <
// (double)p, decided in FP32 unless p lies within 2^-22 |x| of one of the two bounds.  The float
// products x * 1.00001f, x * 0.99999f are within 7.5e-8 |x| of the double ones and the shifted
// bounds round by at most 6e-8 |x| more (1.4e-7 |x| < 2^-22 |x| in all), so outside that band the
// float answer is the double one; inside it (and for |x| outside [1e-30, 1e37], NaN, or 0) the
// double test runs.
__device__ __forceinline__ bool epa_converged(float x, float p)
{
    const float ax = fabsf(x);
    if (ax > 1e-30f && ax < 1e37f) {
        const float hi = x * 1.00001f, lo = x * 0.99999f;
        const float tol = ax * 2.384185791015625e-7f;
        if (p < hi - tol && p > lo + tol) return true;
        if (p > hi + tol || p < lo - tol) return false;
    }
    return (double)x * 1.00001 > (double)p && (double)x * 0.99999 < (double)p;
}

// ---------------------------------------------------------------- the reference's double results in FP32
// A few per-contact quantities the reference computes in double and rounds to float (the barycentric
// weight of the contact point, .cu:583; the tangential stiffness and damping, .cu:746-749; the Coulomb
// test, .cu:774).  FP64 runs at a small fraction of the FP32 rate on this GPU and its long latency sat
// on every contact's path, so they are evaluated in float-float arithmetic (error-free sums, fused
// multiply-add remainders) and the float is taken when it is provably the double computation's result
// rounded to float: when the value lies farther from a float rounding boundary than the error bound of
// both computations.  Otherwise (a value within ~2^-18 of a boundary, or non-finite or extreme
// operands) the double computation runs.

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// s + e = a + b exactly, for |a| >= |b| (or a = 0) (Dekker)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    e = b - (s - a);
}

// true when every real within `err` of a + b rounds to the float a (round to nearest): |b| plus the
// error stays below half the spacing of the floats next to a on b's side (the spacing below a power
// of two, toward zero, is half the one above).  False for |a| outside [2^-102, 2^127) and non-finite a.
__device__ __forceinline__ bool rounds_to(float a, float b, float err)
{
    const uint32_t ua = __float_as_uint(a) & 0x7fffffffu;
    if (ua < 0x0c800000u || ua >= 0x7f000000u) return false;
    const float ulp = __uint_as_float(ua & 0x7f800000u) * 1.1920928955078125e-7f;  // 2^(exponent - 23)
    const bool toward_zero = (b < 0.f) != (a < 0.f);
    const float half = ((ua & 0x007fffffu) == 0u && toward_zero) ? 0.25f * ulp : 0.5f * ulp;
    return fabsf(b) + err < half * 0.99999f;
}

// spacing of the floats at x (2^-149 for subnormal x, +inf for 0 and non-finite x)
__device__ __forceinline__ float ulp_of(float x)
{
    const uint32_t ux = __float_as_uint(x) & 0x7fffffffu;
    if (ux == 0u || ux >= 0x7f800000u) return __int_as_float(0x7f800000);
    if (ux < 0x00800000u) return 1.401298464324817e-45f;
    return __uint_as_float(ux & 0x7f800000u) * 1.1920928955078125e-7f;
}

// (float)(1.0 - (double)bw - (double)bv).  The exact value is s2 + t + r (error-free sums) and a is the
// float nearest to s2 + t.  1, bw and bv are multiples of q = the smallest of their spacings, and so
// are 1 - bw and the result: below 2^53 q the double computation holds both exactly, and with r = 0 a is
// then its result rounded to float, ties included.  Otherwise a is certified against the double
// computation's error, at most 2^-53 (|1 - bw| + |result|).
__device__ __forceinline__ float one_minus_two(float bw, float bv)
{
    float s1, e1, s2, e2, t, r, a, b0;
    two_sum(1.f, -bw, s1, e1);
    two_sum(s1, -bv, s2, e2);
    two_sum(e2, e1, t, r);
    two_sum(s2, t, a, b0);
    if (fabsf(bw) < 1e30f && fabsf(bv) < 1e30f) {
        const float q = fminf(fminf(ulp_of(bw), ulp_of(bv)), 1.1920928955078125e-7f);
        const bool exact = fmaxf(fabsf(s1), fabsf(a)) < q * 2251799813685248.f;  // 2^51 q
        if (exact && r == 0.f) return a;
        const float b = b0 + r;
        const float err = (exact ? 0.f : (fabsf(s1) + fabsf(a)) * 2.220446049250313e-16f) +
                          fabsf(b) * 1.1920928955078125e-7f;
        if (rounds_to(a, b, err)) return a;
    }
    return (float)(1.0 - (double)bw - (double)bv);
}

// Kt = (float)(KtA * 1 / C) and Gt = (float)((-1) * 2 / C * (double)ln_et) with
// C = inv_mu + (double)x + (double)y (.cu:746-749; x, y the float quotients dA^2/IsA, dB^2/IsB).  C is
// formed as a float pair from non-negative terms; each quotient is a rounded float quotient (KtA_hi / ch,
// and -2 / ch as -2 RN(1 / ch), exact scaling), whose remainder a fused multiply-add gives exactly,
// corrected by that remainder times RN(1 / ch).  The pair values are within 2^-43 of the exact ones
// and the double results within 5 * 2^-53 of them: a margin of 2^-41 certifies the float.
__device__ __forceinline__ void tangential_coeffs(const mwd_material& M, float x, float y, float& Kt, float& Gt)
{
    bool okK = false, okG = false;
    if (x >= 0.f && x < 1e30f && y >= 0.f && y < 1e30f && M.inv_mu_hi > 0.f && M.inv_mu_hi < 1e30f) {
        float c1, e1, c2, e2, ch, cl;
        two_sum(M.inv_mu_hi, x, c1, e1);
        two_sum(c1, y, c2, e2);
        fast_two_sum(c2, (M.inv_mu_lo + e1) + e2, ch, cl);
        const float rc = 1.f / ch;
        // (KtA_hi + KtA_lo) / (ch + cl)
        const float q1 = M.KtA_hi / ch;
        const float rq = ((fmaf(-q1, ch, M.KtA_hi) + M.KtA_lo) - q1 * cl) * rc;
        float kh, kl;
        fast_two_sum(q1, rq, kh, kl);
        // -2 / (ch + cl), then times ln_et
        const float g1 = -2.f * rc;
        const float rg = (fmaf(-g1, ch, -2.f) - g1 * cl) * rc;
        float gh, gl;
        fast_two_sum(g1, rg, gh, gl);
        const float p = gh * M.ln_et;
        float Gh, Gl;
        fast_two_sum(p, fmaf(gh, M.ln_et, -p) + gl * M.ln_et, Gh, Gl);
        okK = rounds_to(kh, kl, fabsf(kh) * 4.547473508864641e-13f);  // 2^-41
        okG = rounds_to(Gh, Gl, fabsf(Gh) * 4.547473508864641e-13f);
        Kt = kh;
        Gt = Gh;
    }
    if (okK && okG) return;
    const double C = M.inv_mu + (double)x + (double)y;
    if (!okK) Kt = (float)(M.KtA * 1 / C);
    if (!okG) Gt = (float)((-1) * 2 / C * (double)M.ln_et);
}

// (double)Ftn > mu * (double)Fnn (.cu:774): 1 when greater, 0 when not greater, -1 when unordered (NaN).
// mu_f * Fnn is within 2.1 u of the double product (u = 2^-24): a margin of 4e-7 (~6.7 u) decides.
__device__ __forceinline__ int coulomb_compare(float Ftn, float Fnn, const mwd_material& M)
{
    const float t = M.mu_f * Fnn;
    if (t >= 1e-30f && t <= 1e30f) {
        const float e = t * 4e-7f;
        if (Ftn > t + e) return 1;
        if (Ftn < t - e) return 0;
    }
    const double X = (double)Ftn, P = M.mu * (double)Fnn;
    return X > P ? 1 : (X <= P ? 0 : -1);
}

// AddTriangle (.cu:270-325): normal and distance of the face (e0, e1, e2), its winding (t1, t2) and
// validity (1, or -2 with distance 1e30 when the origin's projection falls outside it)
__device__ __forceinline__ float4 face_geom(const EpaMem& m, int e0, int e1, int e2, int& t1, int& t2, int& valid)
{
    f3 a = xyz(m.pv[e0]), b = xyz(m.pv[e1]), c = xyz(m.pv[e2]);
    f3 n = cross(b - a, c - b);
    float len = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    n = n / len;
    float dist = dot(n, a);
    t1 = e1;
    t2 = e2;
    if (dist < 0.f) {
        t2 = e1;
        t1 = e2;
        dist = dist * (-1.f);
        n = n * (-1.f);
    }
    f3 A = xyz(m.pv[e0]), B = xyz(m.pv[t1]), C = xyz(m.pv[t2]);
    bool inside = false;
    if (dot(cross(B - A, n), A * (-1.f)) < 0.f)
        if (dot(cross(C - B, n), B * (-1.f)) < 0.f)
            if (dot(cross(A - C, n), C * (-1.f)) < 0.f) inside = true;
    valid = 1;
    if (!inside) {
        valid = -2;
        dist = 1e30f;
    }
    return f4(n, dist);
}

// AddTriangle into slot f of the face list, one face per calling lane
__device__ __forceinline__ void add_face(EpaMem& m, int e0, int e1, int e2, int f)
{
    int t1, t2, valid;
    m.fn[f] = face_geom(m, e0, e1, e2, t1, t2, valid);
    m.ft[f] = ft_make(e0, t1, t2, valid);
}

// "x < best" of the reference's array_min_finder (.cu:41-53), NaN never wins
__device__ __forceinline__ bool min_better(float v, int i, float bv, int bi)
{
    if (v != v) return false;
    if (bv != bv) return true;
    return v < bv || (v == bv && i < bi);
}

struct EpaResult {
    float depth;
    f3 n, cpA, cpB;
    int fa[3], fb[3];
    uint32_t status;
};

// EPA (.cu:328-603) with the reference's append-only face list: deleted faces stay in it at distance
// 3e20 (.cu:541-542).  A pair whose list would outgrow FCAP stops with MWD_ST_EPA_OVERFLOW and is run
// again by epa_compacting.
template <int LPP>
__device__ void epa(const Group<LPP>& g, EpaMem& m, const float4* hA, int nA, const float4* hB, int nB,
                    f3 S1, int a1, int b1, f3 S2, int a2, int b2, f3 S3, int a3, int b3, f3 S4, int a4, int b4,
                    EpaResult& r, Work3& wk)
{
    r.status = 0;
    g.sync();
    if (g.lane == 0) {
        m.pv[0] = f4(S1, 0.f); m.pv[1] = f4(S2, 0.f); m.pv[2] = f4(S3, 0.f); m.pv[3] = f4(S4, 0.f);
        m.pab[0] = (uint16_t)(a1 | (b1 << 8)); m.pab[1] = (uint16_t)(a2 | (b2 << 8));
        m.pab[2] = (uint16_t)(a3 | (b3 << 8)); m.pab[3] = (uint16_t)(a4 | (b4 << 8));
    }
    g.sync();
    if (g.lane < 4) {
        // faces (0,1,2), (1,2,3), (2,0,3), (0,1,3), packed as 4-bit vertex numbers (no local array)
        const unsigned long long e = 0x310302321210ull >> (12 * g.lane);
        add_face(m, (int)(e & 0xf), (int)((e >> 4) & 0xf), (int)((e >> 8) & 0xf), g.lane);
    }
    g.sync();
    wk.faces += 4;
    int nt = 4, nv = 4, counter = 0, indmin = 0;
    float xmin_old = 1e29f;
    float proj = 2 * xmin_old + 1;
    float xmin_new = 0.f;
    while (xmin_old < proj) {
        // first index of the minimum distance
        float bv = __int_as_float(0x7fffffff);
        int bi = 0x7fffffff;
        for (int f = g.lane; f < nt; f += LPP) {
            float v = m.fn[f].w;
            if (min_better(v, f, bv, bi)) { bv = v; bi = f; }
        }
        {
            // group minimum (NaN never wins), then the first face index holding it
            const unsigned k = (bv != bv) ? 0xffffffffu : fkey(bv);
            const unsigned km = __reduce_min_sync(g.mask, k);
            bi = (int)__reduce_min_sync(g.mask, k == km ? (unsigned)bi : 0xffffffffu);
        }
        float d0 = m.fn[0].w;
        indmin = (d0 != d0) ? 0 : bi;
        float4 fm = m.fn[indmin];
        xmin_new = fm.w;
        xmin_old = xmin_new;
        f3 n = xyz(fm);
        f3 s;
        int sa, sb;
        support<LPP>(g, hA, nA, hB, nB, n, s, sa, sb, wk);
        proj = dot(n, s);
        if (xmin_old > proj || epa_converged(xmin_old, proj)) break;
        if (counter > 49) { r.status |= MWD_ST_EPA_NOCONV; break; }
        counter = counter + 1;
        if (nv >= VCAP) { r.status |= MWD_ST_EPA_OVERFLOW; break; }
        g.sync();
        if (g.lane == 0) {
            m.pv[nv] = f4(s, 0.f);
            m.pab[nv] = (uint16_t)(sa | (sb << 8));
        }
        nv++;
        // visible faces -> deleted, collected in index order
        int ndel = 0;
        for (int base = 0; base < nt; base += LPP) {
            int f = base + g.lane;
            bool dead = false;
            uint32_t t = 0;
            if (f < nt) {
                t = m.ft[f];
                int vl = ft_valid(t);
                if ((vl == 1 || vl == -2) && dot(s - xyz(m.pv[ft_v(t, 0)]), xyz(m.fn[f])) >= 0.f) {
                    dead = true;
                    m.ft[f] = (t & 0x00ffffffu) | ((uint32_t)(-1 + 2) << 24);
                }
            }
            unsigned b = g.ballot(dead);
            if (dead) m.del[ndel + __popc(b & g.lt_mask())] = (t & 0x00ffffffu) | ((uint32_t)f << 24);
            ndel += __popc(b);
        }
        g.sync();
        // horizon edges of the deleted faces, in face order then edge order (0,1),(1,2),(2,0);
        // an edge is kept when fewer than two delpair increments land on it (.cu:482-544), i.e. when
        // its unordered vertex pair occurs once among the deleted faces' edges (a face's vertex indices
        // are distinct).  When all those edges fit the group's lanes at once, one match over the lanes'
        // vertex pairs counts them; otherwise each lane counts its edge against the deleted list.
        int nnew = 0;
        bool overflow = false;
        const bool one_trip = 3 * ndel <= LPP;
        for (int base = 0; base < 3 * ndel; base += LPP) {
            int c = base + g.lane;
            bool keep = false;
            int e0 = 0, e1 = 0;
            unsigned pair_code = 0x10000u + (unsigned)g.lane;  // distinct for lanes without an edge
            if (c < 3 * ndel) {
                uint32_t t = m.del[c / 3];
                int k = c % 3;
                e0 = ft_v(t, k);
                e1 = ft_v(t, k == 2 ? 0 : k + 1);
                pair_code = (unsigned)(min(e0, e1) * 256 + max(e0, e1));
                if (!one_trip) {
                    int cnt = 0;
                    for (int j = 0; j < ndel; ++j) {
                        uint32_t u = m.del[j];
                        int x = ft_v(u, 0), y = ft_v(u, 1), z = ft_v(u, 2);
                        cnt += (e0 == y && e1 == x) + (e0 == x && e1 == y) + (e0 == z && e1 == y) +
                               (e0 == y && e1 == z) + (e0 == x && e1 == z) + (e0 == z && e1 == x);
                    }
                    keep = cnt < 2;
                }
            }
            if (one_trip) {
                // every lane of the group takes part in the match (lanes without an edge hold a code no
                // other lane holds)
                const unsigned same = __match_any_sync(g.mask, pair_code);
                keep = c < 3 * ndel && __popc(same) == 1;
            }
            unsigned b = g.ballot(keep);
            if (keep) {
                int f = nt + nnew + __popc(b & g.lt_mask());
                if (f < FCAP) add_face(m, e0, e1, nv - 1, f);
            }
            nnew += __popc(b);
        }
        if (nt + nnew > FCAP) overflow = true;
        g.sync();
        for (int k = g.lane; k < ndel; k += LPP) {
            int f = (int)(m.del[k] >> 24);
            m.ft[f] = (m.ft[f] & 0x00ffffffu) | ((uint32_t)(0 + 2) << 24);
            m.fn[f].w = 3e20f;
        }
        g.sync();
        if (overflow) { r.status |= MWD_ST_EPA_OVERFLOW; break; }
        nt += nnew;
        wk.faces += (uint32_t)nnew;
        counter = counter + 1;
    }
    g.sync();
    r.depth = xmin_new;
    // the contact point and everything after it (the force) are needed by one lane only: the others
    // skip them, which keeps their FP64 operations (below and in contact_force) off the FP64 pipe
    if (g.lane != 0) return;
    uint32_t t = m.ft[indmin];
    int a = ft_v(t, 0), b = ft_v(t, 1), c = ft_v(t, 2);
    f3 n = xyz(m.fn[indmin]);
    f3 Pr = n * r.depth;
    f3 Va = xyz(m.pv[a]), Vb = xyz(m.pv[b]), Vc = xyz(m.pv[c]);
    f3 v0 = Vb - Va, v1 = Vc - Va, v2 = Pr - Va;
    if (dot(cross(v0, v1), n) < 0.f) {
        v0 = Vc - Va;
        v1 = Vb - Va;
    }
    float v00 = dot(v0, v0), v01 = dot(v0, v1), v11 = dot(v1, v1), v20 = dot(v2, v0), v21 = dot(v2, v1);
    float den = v00 * v11 - v01 * v01;
    float bv = (v11 * v20 - v01 * v21) / den;
    float bw = (v00 * v21 - v01 * v20) / den;
    float bu = one_minus_two(bw, bv);
    int pa = m.pab[a], pb = m.pab[b], pc = m.pab[c];
    r.fa[0] = pa & 0xff; r.fa[1] = pb & 0xff; r.fa[2] = pc & 0xff;
    r.fb[0] = pa >> 8; r.fb[1] = pb >> 8; r.fb[2] = pc >> 8;
    r.cpA = (xyz(hA[r.fa[0]]) * bu + xyz(hA[r.fa[1]]) * bv) + xyz(hA[r.fa[2]]) * bw;
    r.cpB = (xyz(hB[r.fb[0]]) * bu + xyz(hB[r.fb[1]]) * bv) + xyz(hB[r.fb[2]]) * bw;
    r.n = n;
}

// The EPA of a pair whose face list outgrew FCAP, run again from the same simplex: the same decisions
// and arithmetic with the deleted faces removed from the list (the survivors keep their order) instead
// of kept at 3e20.  Of the removed faces only the earliest created can still win the minimum search
// (.cu:41-53: all are at 3e20, the first index wins): it is kept in the list's last slot, FCAP - 1, with
// every face's creation index (its index in the reference's arrays) packed into its vertex word:
// T0 | T1 << 5 | T2 << 10 | (valid + 2) << 15 | creation << 17.  At most 2 * 30 - 4 = 56 faces are
// alive within the reference's iteration limit, so this list does not overflow.  Rarely needed: the
// two-pass narrow phase runs the records that overflowed again in a kernel of their own after its EPA
// pass, the single-pass kernel calls it out of line right after the overflow (epa_run).
__device__ __forceinline__ int fc_v(uint32_t t, int k) { return (t >> (5 * k)) & 31; }
__device__ __forceinline__ uint32_t fc_created(uint32_t t) { return t >> 17; }
__device__ __forceinline__ uint32_t fc_make(int a, int b, int c, int valid, uint32_t created)
{
    return (uint32_t)a | ((uint32_t)b << 5) | ((uint32_t)c << 10) | ((uint32_t)(valid + 2) << 15) | (created << 17);
}

// contact points of the final face (.cu:548-600): barycentric coordinates of n * depth on the face
// (winding swapped when its normal points the other way), applied to the support vertices of A and B
__device__ __forceinline__ void epa_contact(const EpaMem& m, const float4* hA, const float4* hB, f3 n, int a, int b,
                                            int c, EpaResult& r)
{
    f3 Pr = n * r.depth;
    f3 Va = xyz(m.pv[a]), Vb = xyz(m.pv[b]), Vc = xyz(m.pv[c]);
    f3 v0 = Vb - Va, v1 = Vc - Va, v2 = Pr - Va;
    if (dot(cross(v0, v1), n) < 0.f) {
        v0 = Vc - Va;
        v1 = Vb - Va;
    }
    float v00 = dot(v0, v0), v01 = dot(v0, v1), v11 = dot(v1, v1), v20 = dot(v2, v0), v21 = dot(v2, v1);
    float den = v00 * v11 - v01 * v01;
    float bv = (v11 * v20 - v01 * v21) / den;
    float bw = (v00 * v21 - v01 * v20) / den;
    float bu = one_minus_two(bw, bv);
    int pa = m.pab[a], pb = m.pab[b], pc = m.pab[c];
    r.fa[0] = pa & 0xff; r.fa[1] = pb & 0xff; r.fa[2] = pc & 0xff;
    r.fb[0] = pa >> 8; r.fb[1] = pb >> 8; r.fb[2] = pc >> 8;
    r.cpA = (xyz(hA[r.fa[0]]) * bu + xyz(hA[r.fa[1]]) * bv) + xyz(hA[r.fa[2]]) * bw;
    r.cpB = (xyz(hB[r.fb[0]]) * bu + xyz(hB[r.fb[1]]) * bv) + xyz(hB[r.fb[2]]) * bw;
    r.n = n;
}

template <int LPP>
__device__ __forceinline__ EpaResult epa_compacting(const Group<LPP>& g, EpaMem* mp, const float4* hA, int nA,
                                                    const float4* hB, int nB, f3 S1, int a1, int b1, f3 S2, int a2,
                                                    int b2, f3 S3, int a3, int b3, f3 S4, int a4, int b4, Work3* wkp)
{
    constexpr int SLOT = FCAP - 1;   // the earliest-created removed face
    constexpr int LIVE = FCAP - 1;   // capacity of the live list
    constexpr uint32_t NONE = 0xffffffffu;
    EpaMem& m = *mp;
    Work3 wk = *wkp;
    EpaResult r;
    r.status = 0;
    g.sync();
    if (g.lane == 0) {
        m.pv[0] = f4(S1, 0.f); m.pv[1] = f4(S2, 0.f); m.pv[2] = f4(S3, 0.f); m.pv[3] = f4(S4, 0.f);
        m.pab[0] = (uint16_t)(a1 | (b1 << 8)); m.pab[1] = (uint16_t)(a2 | (b2 << 8));
        m.pab[2] = (uint16_t)(a3 | (b3 << 8)); m.pab[3] = (uint16_t)(a4 | (b4 << 8));
    }
    g.sync();
    if (g.lane < 4) {
        const unsigned long long e = 0x310302321210ull >> (12 * g.lane);
        const int e0 = (int)(e & 0xf), e1 = (int)((e >> 4) & 0xf), e2 = (int)((e >> 8) & 0xf);
        int t1, t2, valid;
        m.fn[g.lane] = face_geom(m, e0, e1, e2, t1, t2, valid);
        m.ft[g.lane] = fc_make(e0, t1, t2, valid, (uint32_t)g.lane);
    }
    g.sync();
    wk.faces += 4;
    int nt = 4, nv = 4, counter = 0;
    uint32_t created = 4;
    uint32_t del_c = NONE;  // creation index of the face in the slot (NONE: none removed yet)
    const int lane0 = (int)(threadIdx.x & 31) - g.lane;
    float xmin_old = 1e29f;
    float proj = 2 * xmin_old + 1;
    float xmin_new = 0.f;
    float4 fm = make_float4(0.f, 0.f, 0.f, 0.f);  // the face chosen last, and its vertex word
    uint32_t tm = 0;
    while (xmin_old < proj) {
        float bv = __int_as_float(0x7fffffff);
        int bi = 0x7fffffff;
        for (int f = g.lane; f < nt; f += LPP) {
            float v = m.fn[f].w;
            if (min_better(v, f, bv, bi)) { bv = v; bi = f; }
        }
        {
            const unsigned k = (bv != bv) ? 0xffffffffu : fkey(bv);
            const unsigned km = __reduce_min_sync(g.mask, k);
            bi = (int)__reduce_min_sync(g.mask, k == km ? (unsigned)bi : 0xffffffffu);
        }
        // the removed faces (all at 3e20) are represented by the earliest created of them
        bool use_slot = false;
        if (del_c != NONE) {
            if (bi == 0x7fffffff) use_slot = true;
            else {
                const float lv = m.fn[bi].w;
                use_slot = lv > 3e20f || (lv == 3e20f && del_c < fc_created(m.ft[bi]));
            }
        }
        // the search starts from face 0's distance: a NaN there keeps face 0
        if (nt > 0 && fc_created(m.ft[0]) == 0 && m.fn[0].w != m.fn[0].w) {
            use_slot = false;
            bi = 0;
        }
        fm = use_slot ? m.fn[SLOT] : m.fn[bi];
        tm = use_slot ? m.ft[SLOT] : m.ft[bi];
        xmin_new = fm.w;
        xmin_old = xmin_new;
        f3 n = xyz(fm);
        f3 s;
        int sa, sb;
        support<LPP>(g, hA, nA, hB, nB, n, s, sa, sb, wk);
        proj = dot(n, s);
        if (xmin_old > proj || epa_converged(xmin_old, proj)) break;
        if (counter > 49) { r.status |= MWD_ST_EPA_NOCONV; break; }
        counter = counter + 1;
        if (nv >= VCAP) { r.status |= MWD_ST_EPA_OVERFLOW; break; }
        g.sync();
        if (g.lane == 0) {
            m.pv[nv] = f4(s, 0.f);
            m.pab[nv] = (uint16_t)(sa | (sb << 8));
        }
        nv++;
        // faces the new vertex sees are deleted, collected in list order; the others move down
        int ndel = 0, nkeep = 0;
        for (int base = 0; base < nt; base += LPP) {
            const int f = base + g.lane;
            bool dead = false, live = false;
            float4 fv = make_float4(0.f, 0.f, 0.f, 0.f);
            uint32_t t = 0;
            if (f < nt) {
                fv = m.fn[f];
                t = m.ft[f];
                dead = dot(s - xyz(m.pv[fc_v(t, 0)]), xyz(fv)) >= 0.f;
                live = !dead;
            }
            const unsigned bd = g.ballot(dead), bl = g.ballot(live);
            g.sync();
            if (dead)
                m.del[ndel + __popc(bd & g.lt_mask())] = (uint32_t)fc_v(t, 0) | ((uint32_t)fc_v(t, 1) << 8) |
                                                         ((uint32_t)fc_v(t, 2) << 16);
            if (live) {
                const int o = nkeep + __popc(bl & g.lt_mask());
                if (o != f) {
                    m.fn[o] = fv;
                    m.ft[o] = t;
                }
            }
            if (bd && ndel == 0) {
                // the first face deleted in this iteration is the earliest created of them
                const int fl = __ffs(bd) - 1;
                const uint32_t c0 = (uint32_t)__shfl_sync(g.mask, (int)fc_created(t), lane0 + fl);
                if (c0 < del_c) {
                    if (g.lane == fl) {
                        m.fn[SLOT] = make_float4(fv.x, fv.y, fv.z, 3e20f);
                        m.ft[SLOT] = (t & ~((uint32_t)3 << 15)) | ((uint32_t)(0 + 2) << 15);
                    }
                    del_c = c0;
                }
            }
            ndel += __popc(bd);
            nkeep += __popc(bl);
        }
        g.sync();
        // horizon edges, as in epa (.cu:482-544); the new faces follow the survivors
        int nnew = 0;
        for (int base = 0; base < 3 * ndel; base += LPP) {
            int c = base + g.lane;
            bool keep = false;
            int e0 = 0, e1 = 0;
            if (c < 3 * ndel) {
                uint32_t t = m.del[c / 3];
                int k = c % 3;
                e0 = ft_v(t, k);
                e1 = ft_v(t, k == 2 ? 0 : k + 1);
                int cnt = 0;
                for (int j = 0; j < ndel; ++j) {
                    uint32_t u = m.del[j];
                    int x = ft_v(u, 0), y = ft_v(u, 1), z = ft_v(u, 2);
                    cnt += (e0 == y && e1 == x) + (e0 == x && e1 == y) + (e0 == z && e1 == y) +
                           (e0 == y && e1 == z) + (e0 == x && e1 == z) + (e0 == z && e1 == x);
                }
                keep = cnt < 2;
            }
            unsigned b = g.ballot(keep);
            if (keep) {
                const int q = nnew + __popc(b & g.lt_mask());
                const int f = nkeep + q;
                if (f < LIVE) {
                    int t1, t2, valid;
                    m.fn[f] = face_geom(m, e0, e1, nv - 1, t1, t2, valid);
                    m.ft[f] = fc_make(e0, t1, t2, valid, created + (uint32_t)q);
                }
            }
            nnew += __popc(b);
        }
        g.sync();
        if (nkeep + nnew > LIVE) { r.status |= MWD_ST_EPA_OVERFLOW; break; }
        nt = nkeep + nnew;
        created += (uint32_t)nnew;
        wk.faces += (uint32_t)nnew;
        counter = counter + 1;
    }
    g.sync();
    r.depth = xmin_new;
    *wkp = wk;
    if (g.lane == 0) epa_contact(m, hA, hB, xyz(fm), fc_v(tm, 0), fc_v(tm, 1), fc_v(tm, 2), r);
    return r;
}

template <int LPP>
__device__ __noinline__ EpaResult epa_compacting_call(const Group<LPP> g, EpaMem* mp, const float4* hA, int nA,
                                                      const float4* hB, int nB, f3 S1, int a1, int b1, f3 S2, int a2,
                                                      int b2, f3 S3, int a3, int b3, f3 S4, int a4, int b4, Work3* wkp)
{
    return epa_compacting<LPP>(g, mp, hA, nA, hB, nB, S1, a1, b1, S2, a2, b2, S3, a3, b3, S4, a4, b4, wkp);
}

// EPA of one pair in the single-pass kernel: the append-only list, and for the rare pair that outgrows
// it, the compacting one (its work counted once: the first attempt's is dropped)
template <int LPP>
__device__ __forceinline__ void epa_run(const Group<LPP>& g, EpaMem& m, const float4* hA, int nA, const float4* hB,
                                        int nB, f3 S1, int a1, int b1, f3 S2, int a2, int b2, f3 S3, int a3, int b3,
                                        f3 S4, int a4, int b4, EpaResult& r, Work3& wk)
{
    const Work3 w0 = wk;
    epa<LPP>(g, m, hA, nA, hB, nB, S1, a1, b1, S2, a2, b2, S3, a3, b3, S4, a4, b4, r, wk);
    if (r.status & MWD_ST_EPA_OVERFLOW) {
        wk = w0;
        r = epa_compacting_call<LPP>(g, &m, hA, nA, hB, nB, S1, a1, b1, S2, a2, b2, S3, a3, b3, S4, a4, b4, &wk);
    }
}

struct ForceResult {
    f3 F, TA, TB, dt;
};

// Force (.cu:647-871) with the pair-independent constants taken from mwd_material
// imA, imB: inverse masses (0 for a wall side), read only by the physical law.
__device__ __forceinline__ void contact_force(f3 cA, f3 cB, float depth, f3 n, f3 cpA, f3 cpB, const mwd_material& M,
                                              f3 vA, f3 vB, f3 wA, f3 wB, f3 dt, float4 qA, float dtn, float IsA,
                                              float IsB, float imA, float imB, ForceResult& o)
{
    f3 cp;
    float Kt, Gt, Gn;
    if (!M.physical) {
        cp = (cpA - cpB) / 2.f;
        f3 dA = cp - cA, dB = cp - cB;
        float dA2 = dA.x * dA.x + dA.y * dA.y + dA.z * dA.z;
        float dB2 = dB.x * dB.x + dB.y * dB.y + dB.z * dB.z;
        tangential_coeffs(M, dA2 / IsA, dB2 / IsB, Kt, Gt);
        Gn = M.Gn;
    } else {
        // effective masses from the pair; tc and the dampings follow from them (MWD_LAW_PHYSICAL)
        cp = (cpA + cpB) / 2.f;
        f3 dA = cp - cA, dB = cp - cB;
        float dA2 = dA.x * dA.x + dA.y * dA.y + dA.z * dA.z;
        float dB2 = dB.x * dB.x + dB.y * dB.y + dB.z * dB.z;
        const float im = imA + imB;
        const float mn = 1.f / im;
        const float tc2 = mn * M.Xn / M.Kn_f;
        const float tc = sqrtf(tc2);
        Gn = (-2.f) * mn * M.ln_en / tc;
        float C = im;
        if (imA != 0.f) C = C + dA2 / IsA;
        if (imB != 0.f) C = C + dB2 / IsB;
        const float mt = 1.f / C;
        Kt = mt * M.Xt / tc2;
        Gt = (-2.f) * mt * M.ln_et / tc;
    }
    if (dot(cB - cA, n) < 0.f) n = n * (-1.f);
    float nn = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    n = n / nn;
    f3 disp_n = n * depth;
    f3 u = ((vA + cross(wA, cpA - cA)) - vB) - cross(wB, cpB - cB);
    f3 un = n * dot(u, n);
    f3 ut = u - un;
    float utn = sqrtf(ut.x * ut.x + ut.y * ut.y + ut.z * ut.z);
    f3 tij = mk3(0.f, 0.f, 0.f);
    if (utn != 0.f) tij = ut / utn;
    if (utn == 0.f && dtn != 0.f) tij = dt / dtn;
    f3 Fn = (disp_n * (-1.f)) * M.Kn_f - un * Gn;
    float Fnn = sqrtf(Fn.x * Fn.x + Fn.y * Fn.y + Fn.z * Fn.z);
    f3 Ft = dt * (-1.f) * Kt - ut * Gt;
    float Ftn = sqrtf(Ft.x * Ft.x + Ft.y * Ft.y + Ft.z * Ft.z);
    // two separate tests as in the reference, so a NaN norm takes the second (slip) branch
    const int coulomb = coulomb_compare(Ftn, Fnn, M);
    if (coulomb == 1) Ft = ((tij * Fnn) * (-1.f)) * M.mu_f;
    if (coulomb == 0) {
        float4 qi = qconj(qA);
        o.dt = qtrip(qA, dt, qi) + ut * M.dt_f;
    } else {
        f3 t = (((tij * Fnn) * M.mu_f) * (-1.f)) - ut * Gt;
        o.dt = (t * 1.f) / Kt;
    }
    f3 Ff = Ft + Fn;
    o.F = Fn;
    o.TA = cross(cp - cA, Ff);
    o.TB = cross(cp - cB, Ff * (-1.f));
}

// ------------------------------------------------------------------ pair sources

struct PairView {
    f3 cA, cB, vA, vB, wA, wB, dt;
    float4 qA;
    float IsA, IsB, dtn;
    int idA, idB, nA, nB;
    int wall;
};

template <int MODE>
__device__ __forceinline__ bool load_pair(const NarrowArgs& a, int64_t P, PairView& p, float4* hA, float4* hB,
                                          int lane, int lpp, bool stage = true)
{
    if (MODE == 0) {
        const float* c;
        c = a.A_com + 3 * P; p.cA = mk3(c[0], c[1], c[2]);
        c = a.B_com + 3 * P; p.cB = mk3(c[0], c[1], c[2]);
        c = a.A_vel + 3 * P; p.vA = mk3(c[0], c[1], c[2]);
        c = a.B_vel + 3 * P; p.vB = mk3(c[0], c[1], c[2]);
        c = a.A_w + 3 * P; p.wA = mk3(c[0], c[1], c[2]);
        c = a.B_w + 3 * P; p.wB = mk3(c[0], c[1], c[2]);
        c = a.qA + 4 * P; p.qA = make_float4(c[0], c[1], c[2], c[3]);
        p.IsA = a.IsA[P];
        p.IsB = a.IsB[P];
        p.idA = a.A_id[P];
        p.idB = a.B_id[P];
        p.nA = a.A_nv[P];
        p.nB = a.B_nv[P];
        p.wall = (p.idA < a.n_wall || p.idB < a.n_wall) ? 1 : 0;
        const int64_t hb = a.hist_mode ? 4 * P : P;
        p.dt = mk3(a.hist_in[hb], a.hist_in[hb + 1], a.hist_in[hb + 2]);
        if (p.nA < 0 || p.nB < 0 || p.nA > a.hull_cap || p.nB > a.hull_cap) return false;
        const float* va = a.A_verts + P * a.V * 3;
        const float* vb = a.B_verts + P * a.V * 3;
        for (int i = lane; i < p.nA; i += lpp) hA[i] = make_float4(va[3 * i], va[3 * i + 1], va[3 * i + 2], 0.f);
        for (int i = lane; i < p.nB; i += lpp) hB[i] = make_float4(vb[3 * i], vb[3 * i + 1], vb[3 * i + 2], 0.f);
    } else {
        int2 pr = reinterpret_cast<const int2*>(a.pairs)[P];
        p.idA = pr.x;
        p.idB = pr.y;
        const double4 pa = reinterpret_cast<const double4*>(a.st.pos)[p.idA];
        const double4 pb = reinterpret_cast<const double4*>(a.st.pos)[p.idB];
        p.cA = mk3((float)pa.x, (float)pa.y, (float)pa.z);
        p.cB = mk3((float)pb.x, (float)pb.y, (float)pb.z);
        const float4* vel = reinterpret_cast<const float4*>(a.st.vel);
        const float4* w = reinterpret_cast<const float4*>(a.st.w);
        p.vA = xyz(vel[p.idA]);
        p.vB = xyz(vel[p.idB]);
        p.wA = xyz(w[p.idA]);
        p.wB = xyz(w[p.idB]);
        p.qA = reinterpret_cast<const float4*>(a.st.q)[p.idA];
        p.IsA = reinterpret_cast<const float4*>(a.st.inertia)[p.idA].w;
        p.IsB = reinterpret_cast<const float4*>(a.st.inertia)[p.idB].w;
        p.wall = ((a.st.info[p.idA] | a.st.info[p.idB]) & 1);
        p.dt = mk3(0.f, 0.f, 0.f);
        const int oa = a.st.vert_off[p.idA], ob = a.st.vert_off[p.idB];
        p.nA = a.st.vert_off[p.idA + 1] - oa;
        p.nB = a.st.vert_off[p.idB + 1] - ob;
        if (p.nA > a.hull_cap || p.nB > a.hull_cap) return false;
        if (stage) {
            const float4* wv = reinterpret_cast<const float4*>(a.st.world_verts);
            for (int i = lane; i < p.nA; i += lpp) hA[i] = wv[oa + i];
            for (int i = lane; i < p.nB; i += lpp) hB[i] = wv[ob + i];
        }
    }
    p.dtn = sqrtf(p.dt.x * p.dt.x + p.dt.y * p.dt.y + p.dt.z * p.dt.z);
    return true;
}

// Inverse masses of a pair's two rows for the physical law (0 for a wall row); the per-pair layout
// (MODE 0) carries no masses and only runs the reference law.
template <int MODE>
__device__ __forceinline__ void pair_inv_mass(const NarrowArgs& a, const PairView& p, const mwd_material& M,
                                              float& imA, float& imB)
{
    imA = 0.f;
    imB = 0.f;
    if (MODE == 0 || !M.physical) return;
    const float4* ii = reinterpret_cast<const float4*>(a.st.inv_inertia);
    if (!(a.st.info[p.idA] & 1)) imA = ii[p.idA].w;
    if (!(a.st.info[p.idB] & 1)) imB = ii[p.idB].w;
}

template <int MODE>
__device__ __forceinline__ void write_hist(const NarrowArgs& a, int64_t P, f3 v, float flag)
{
    if (MODE != 0) return;
    if (a.hist_mode) {
        float* h = a.hist_out + 4 * P;
        h[0] = v.x; h[1] = v.y; h[2] = v.z; h[3] = flag;
    } else {
        reinterpret_cast<float4*>(a.hist_stage)[P] = make_float4(v.x, v.y, v.z, flag);
        a.hist_wrote[P] = 1;
    }
}

template <int MODE>
__device__ __forceinline__ void accumulate(const NarrowArgs& a, const PairView& p, const ForceResult& fo)
{
    if (MODE == 0) {
        atomicAdd(a.force + 3 * p.idA + 0, fo.F.x);
        atomicAdd(a.force + 3 * p.idA + 1, fo.F.y);
        atomicAdd(a.force + 3 * p.idA + 2, fo.F.z);
        atomicAdd(a.force + 3 * p.idB + 0, -1 * fo.F.x);
        atomicAdd(a.force + 3 * p.idB + 1, -1 * fo.F.y);
        atomicAdd(a.force + 3 * p.idB + 2, -1 * fo.F.z);
        atomicAdd(a.torque + 3 * p.idA + 0, fo.TA.x);
        atomicAdd(a.torque + 3 * p.idA + 1, fo.TA.y);
        atomicAdd(a.torque + 3 * p.idA + 2, fo.TA.z);
        atomicAdd(a.torque + 3 * p.idB + 0, fo.TB.x);
        atomicAdd(a.torque + 3 * p.idB + 1, fo.TB.y);
        atomicAdd(a.torque + 3 * p.idB + 2, fo.TB.z);
    } else {
        float* F = a.st.force;
        float* T = a.st.torque;
        if (!(a.st.info[p.idA] & 1)) {
            atomicAdd(F + 4 * p.idA + 0, fo.F.x);
            atomicAdd(F + 4 * p.idA + 1, fo.F.y);
            atomicAdd(F + 4 * p.idA + 2, fo.F.z);
            atomicAdd(T + 4 * p.idA + 0, fo.TA.x);
            atomicAdd(T + 4 * p.idA + 1, fo.TA.y);
            atomicAdd(T + 4 * p.idA + 2, fo.TA.z);
        }
        if (!(a.st.info[p.idB] & 1)) {
            atomicAdd(F + 4 * p.idB + 0, -1 * fo.F.x);
            atomicAdd(F + 4 * p.idB + 1, -1 * fo.F.y);
            atomicAdd(F + 4 * p.idB + 2, -1 * fo.F.z);
            atomicAdd(T + 4 * p.idB + 0, fo.TB.x);
            atomicAdd(T + 4 * p.idB + 1, fo.TB.y);
            atomicAdd(T + 4 * p.idB + 2, fo.TB.z);
        }
    }
}

template <int LPP, int MODE>
__device__ void process_pair(const NarrowArgs& a, int64_t P, const Group<LPP>& g, EpaMem& em, float4* hA, float4* hB)
{
    PairView p;
    const bool ok = load_pair<MODE>(a, P, p, hA, hB, g.lane, LPP);
    g.sync();
    const bool leader = g.lane == 0;
    if (!ok) {
        if (leader) {
            set_status(a.status, MWD_ST_BAD_SHAPE);
            if (a.collision) a.collision[P] = -1;
        }
        return;
    }
    const mwd_material& M = MODE == 0 ? a.mat[p.wall] : a.scenes[a.st.info[p.idA] >> 1].mat[p.wall];

    Work3 wk = {0u, 0u, 0u};
    f3 S1, S2, S3, S4, d3, d4;
    int a1, b1, a2, b2, a3, b3, a4 = 0, b4 = 0, todel = 0, coll = -1;
    bool early = false, resolved = false;
    f3 d1 = p.cB - p.cA;
    support<LPP>(g, hA, p.nA, hB, p.nB, d1, S1, a1, b1, wk);
    if (dot(d1, S1) < 0.f) early = true;
    if (!early) {
        f3 d2 = d1 * (-1.f);
        support<LPP>(g, hA, p.nA, hB, p.nB, d2, S2, a2, b2, wk);
        if (dot(d2, S2) < 0.f) early = true;
    }
    if (!early) {
        seg_test(S1, S2, coll, d3);
        if (coll == 0) early = true;
    }
    if (!early) {
        support<LPP>(g, hA, p.nA, hB, p.nB, d3, S3, a3, b3, wk);
        if (dot(d3, S3) < 0.f) early = true;
    }
    if (!early) {
        tri_test(S1, S2, S3, coll, d4);
        if (coll == 0) early = true;
    }
    ForceResult fo;
    fo.F = fo.TA = fo.TB = mk3(0.f, 0.f, 0.f);
    fo.dt = p.dt;
    EpaResult er;
    er.status = 0;
    uint32_t st = 0;
    if (!early) {
        int zz = 0;
        while (zz < 50) {
            support<LPP>(g, hA, p.nA, hB, p.nB, d4, S4, a4, b4, wk);
            if (dot(d4, S4) < 0.f) { early = true; break; }
            bool hit = false;
            if (S4.x == 0.f && S4.y == 0.f && S4.z == 0.f) hit = true;
            else {
                tet_test(S1, S2, S3, S4, coll, d4, todel);
                if (coll == 0) { early = true; break; }
                if (coll == 1) hit = true;
            }
            if (hit) {
                if (is_flat(S1, S2, S3, S4)) {
                    d4 = cross(S1, S2);
                    support<LPP>(g, hA, p.nA, hB, p.nB, d4, S4, a4, b4, wk);
                }
                epa_run<LPP>(g, em, hA, p.nA, hB, p.nB, S1, a1, b1, S2, a2, b2, S3, a3, b3, S4, a4, b4, er, wk);
                if (leader) {
                    float imA, imB;
                    pair_inv_mass<MODE>(a, p, M, imA, imB);
                    contact_force(p.cA, p.cB, er.depth, er.n, er.cpA, er.cpB, M, p.vA, p.vB, p.wA, p.wB, p.dt,
                                  p.qA, p.dtn, p.IsA, p.IsB, imA, imB, fo);
                }
                st |= er.status;
                resolved = true;
                break;
            }
            f3 n1, n2, n3;
            int na1, nb1, na2, nb2, na3, nb3;
            if (todel == 1) { n1 = S2; na1 = a2; nb1 = b2; n2 = S3; na2 = a3; nb2 = b3; n3 = S4; na3 = a4; nb3 = b4; }
            else if (todel == 2) { n1 = S3; na1 = a3; nb1 = b3; n2 = S1; na2 = a1; nb2 = b1; n3 = S4; na3 = a4; nb3 = b4; }
            else { n1 = S1; na1 = a1; nb1 = b1; n2 = S2; na2 = a2; nb2 = b2; n3 = S4; na3 = a4; nb3 = b4; }
            S1 = n1; a1 = na1; b1 = nb1; S2 = n2; a2 = na2; b2 = nb2; S3 = n3; a3 = na3; b3 = nb3;
            zz = zz + 1;
        }
        if (!early && !resolved) st |= MWD_ST_GJK_NOCONV;
    }
    if (!leader) return;
    set_status(a.status, st);
    if (a.work_counters) {
        atomicAdd(a.work_counters + 0, (unsigned long long)wk.dots);
        atomicAdd(a.work_counters + 1, (unsigned long long)wk.faces);
        atomicAdd(a.work_counters + 2, (unsigned long long)wk.queries);
    }
    if (early) {
        if (a.collision) a.collision[P] = 0;
        write_hist<MODE>(a, P, mk3(0.f, 0.f, 0.f), 0.f);
    } else {
        if (a.collision) a.collision[P] = resolved ? 1 : -1;
        if (resolved) write_hist<MODE>(a, P, fo.dt, 1.f);
        accumulate<MODE>(a, p, fo);
    }
    if (a.diag) {
        float* dg = a.diag + 10 * P;
        if (resolved) {
            dg[0] = er.depth;
            dg[1] = er.n.x; dg[2] = er.n.y; dg[3] = er.n.z;
            dg[4] = er.cpA.x; dg[5] = er.cpA.y; dg[6] = er.cpA.z;
            dg[7] = er.cpB.x; dg[8] = er.cpB.y; dg[9] = er.cpB.z;
        } else {
            for (int k = 0; k < 10; ++k) dg[k] = 0.f;
        }
    }
    if (a.face_ids) {
        int* fid = a.face_ids + 6 * P;
        for (int k = 0; k < 3; ++k) {
            fid[k] = resolved ? er.fa[k] : -1;
            fid[3 + k] = resolved ? er.fb[k] : -1;
        }
    }
}

template <int LPP, int MODE>
__global__ void __launch_bounds__(NARROW_THREADS) narrow_kernel(NarrowArgs a)
{
    extern __shared__ float4 smem[];
    constexpr int GPB = NARROW_THREADS / LPP;
    const int grp = threadIdx.x / LPP;
    Group<LPP> g;
    g.lane = threadIdx.x % LPP;
    g.mask = LPP == 32 ? 0xffffffffu : (((1u << LPP) - 1u) << ((threadIdx.x & 31) / LPP * LPP));
    EpaMem* em = reinterpret_cast<EpaMem*>(smem) + grp;
    float4* hull = reinterpret_cast<float4*>(reinterpret_cast<EpaMem*>(smem) + GPB) + (size_t)grp * 2 * a.hull_cap;
    float4* hA = hull;
    float4* hB = hull + a.hull_cap;
    int64_t n = a.n_pairs;
    if (MODE == 1) {
        int64_t m = *a.n_pairs_dev;
        n = m < a.pair_cap ? m : a.pair_cap;
    }
    if (MODE == 1) {
        // sphere pre-test (spheres_apart), LPP candidate pairs at a time (one per lane); pairs it
        // settles get the reference's outcome (collision 0, no force) without running GJK
        const double4* pos = reinterpret_cast<const double4*>(a.st.pos);
        const int2* pairs = reinterpret_cast<const int2*>(a.pairs);
        const int64_t stride = (int64_t)gridDim.x * GPB * LPP;
        for (int64_t base = ((int64_t)blockIdx.x * GPB + grp) * LPP; base < n; base += stride) {
            const int64_t Pl = base + g.lane;
            bool live = false;
            if (Pl < n) {
                const int2 pr = pairs[Pl];
                live = !spheres_apart(pos[pr.x], pos[pr.y]);
                if (!live && a.collision) a.collision[Pl] = 0;
            }
            unsigned m = g.ballot(live);
            while (m) {
                const int l = __ffs(m) - 1;
                m &= m - 1;
                process_pair<LPP, MODE>(a, base + l, g, *em, hA, hB);
                g.sync();
            }
        }
        return;
    }
    for (int64_t P = (int64_t)blockIdx.x * GPB + grp; P < n; P += (int64_t)gridDim.x * GPB) {
        process_pair<LPP, MODE>(a, P, g, *em, hA, hB);
        g.sync();
    }
}

// ------------------------------------------------------------------ two-pass narrow phase (table mode)
//
// Pass 1 (gjk_pass_kernel) runs the sphere pre-test and GJK on every candidate pair with the hulls
// read straight from the world-vertex table (no shared memory, few registers, many resident warps);
// separated and undecided pairs are finished there.  Pairs GJK finds in contact append the simplex
// it stopped on to a compact list.  Pass 2 (epa_pass_kernel) continues exactly where pass 1
// stopped -- CorrectFlat, EPA, force -- for the listed pairs only, with the shared-memory polytope.
// The operation sequence per pair is the single-pass kernel's.

// GJK up to the decision (.cu:996-1288): 0 separated, 1 in contact (simplex in rec), -1 undecided
// after 50 tetrahedron iterations.
template <int LPP>
__device__ int gjk_decide(const Group<LPP>& g, const float4* hA, int nA, const float4* hB, int nB, f3 cA, f3 cB,
                          SimplexRec& rec, Work3& wk)
{
    f3 S1, S2, S3, S4, d3, d4;
    int a1, b1, a2, b2, a3, b3, a4 = 0, b4 = 0, todel = 0, coll = -1;
    f3 d1 = cB - cA;
    f3 d2 = d1 * (-1.f);
    support_pair<LPP>(g, hA, nA, hB, nB, d1, S1, a1, b1, S2, a2, b2);
    wk.dots += (uint32_t)(nA + nB);
    wk.queries += 1;
    if (dot(d1, S1) < 0.f) return 0;
    wk.dots += (uint32_t)(nA + nB);
    wk.queries += 1;
    if (dot(d2, S2) < 0.f) return 0;
    seg_test(S1, S2, coll, d3);
    if (coll == 0) return 0;
    support<LPP>(g, hA, nA, hB, nB, d3, S3, a3, b3, wk);
    if (dot(d3, S3) < 0.f) return 0;
    tri_test(S1, S2, S3, coll, d4);
    if (coll == 0) return 0;
    for (int zz = 0; zz < 50; ++zz) {
        support<LPP>(g, hA, nA, hB, nB, d4, S4, a4, b4, wk);
        if (dot(d4, S4) < 0.f) return 0;
        bool hit = false;
        if (S4.x == 0.f && S4.y == 0.f && S4.z == 0.f) hit = true;
        else {
            tet_test(S1, S2, S3, S4, coll, d4, todel);
            if (coll == 0) return 0;
            if (coll == 1) hit = true;
        }
        if (hit) {
            rec.S[0] = f4(S1, 0.f); rec.S[1] = f4(S2, 0.f); rec.S[2] = f4(S3, 0.f); rec.S[3] = f4(S4, 0.f);
            rec.ia = (uint32_t)a1 | ((uint32_t)a2 << 8) | ((uint32_t)a3 << 16) | ((uint32_t)a4 << 24);
            rec.ib = (uint32_t)b1 | ((uint32_t)b2 << 8) | ((uint32_t)b3 << 16) | ((uint32_t)b4 << 24);
            return 1;
        }
        f3 n1, n2, n3;
        int na1, nb1, na2, nb2, na3, nb3;
        if (todel == 1) { n1 = S2; na1 = a2; nb1 = b2; n2 = S3; na2 = a3; nb2 = b3; n3 = S4; na3 = a4; nb3 = b4; }
        else if (todel == 2) { n1 = S3; na1 = a3; nb1 = b3; n2 = S1; na2 = a1; nb2 = b1; n3 = S4; na3 = a4; nb3 = b4; }
        else { n1 = S1; na1 = a1; nb1 = b1; n2 = S2; na2 = a2; nb2 = b2; n3 = S4; na3 = a4; nb3 = b4; }
        S1 = n1; a1 = na1; b1 = nb1; S2 = n2; a2 = na2; b2 = nb2; S3 = n3; a3 = na3; b3 = nb3;
    }
    return -1;
}

// GJK on pair P by the group; lane 0 records the outcome (status, contact flag, and for a pair in
// contact its simplex in the EPA list, whose slot it also appends to *list when list is given)
template <int LPP>
__device__ __forceinline__ void gjk_pair(const NarrowArgs& a, const Group<LPP>& g, int64_t P, int* list, int* list_n)
{
    const double4* pos = reinterpret_cast<const double4*>(a.st.pos);
    const int2* pairs = reinterpret_cast<const int2*>(a.pairs);
    const float4* wv = reinterpret_cast<const float4*>(a.st.world_verts);
    SimplexRec* recs = reinterpret_cast<SimplexRec*>(a.epa_rec);
    const int2 pr = pairs[P];
    const double4 pa = pos[pr.x], pb = pos[pr.y];
    const f3 cA = mk3((float)pa.x, (float)pa.y, (float)pa.z);
    const f3 cB = mk3((float)pb.x, (float)pb.y, (float)pb.z);
    const int oa = a.st.vert_off[pr.x], ob = a.st.vert_off[pr.y];
    const int nA = a.st.vert_off[pr.x + 1] - oa, nB = a.st.vert_off[pr.y + 1] - ob;
    Work3 wk = {0u, 0u, 0u};
    SimplexRec rec;
    int out = 0;
    const bool ok = nA <= a.hull_cap && nB <= a.hull_cap;
    if (ok) out = gjk_decide<LPP>(g, wv + oa, nA, wv + ob, nB, cA, cB, rec, wk);
    if (g.lane == 0) {
        if (!ok) {
            set_status(a.status, MWD_ST_BAD_SHAPE);
            if (a.collision) a.collision[P] = -1;
        } else if (out == 1) {
            const int slot = atomicAdd(a.epa_count, 1);
            if (slot < a.epa_cap) {
                rec.P = P;
                recs[slot] = rec;
                if (list) list[atomicAdd(list_n, 1)] = slot;
            } else {
                set_status(a.status, MWD_ST_PAIR_OVERFLOW);
            }
            if (a.collision) a.collision[P] = 1;
        } else {
            // undecided pairs add zero force in the reference (.cu:1304-1319): nothing to add
            if (out == -1) set_status(a.status, MWD_ST_GJK_NOCONV);
            if (a.collision) a.collision[P] = out;
        }
        if (a.work_counters) {
            atomicAdd(a.work_counters + 0, (unsigned long long)wk.dots);
            atomicAdd(a.work_counters + 2, (unsigned long long)wk.queries);
        }
    }
    g.sync();
}

// GJK on the candidates [base, base + chunk), clipped to hi, by one group (chunk = gjk_chunk(a, LPP)).
// pre_culled: the broad phase already dropped the pairs whose spheres are apart, so each chunk is one
// pair and it runs GJK; otherwise the chunk's LPP candidates are sphere-tested at once (one per lane)
// and the survivors run GJK one after another.
__device__ __forceinline__ int gjk_chunk(const NarrowArgs& a, int lpp) { return a.pre_culled ? 1 : lpp; }

template <int LPP>
__device__ __forceinline__ void gjk_candidates(const NarrowArgs& a, const Group<LPP>& g, int64_t base, int64_t hi,
                                               int* list, int* list_n)
{
    unsigned msk;
    if (a.pre_culled) {
        msk = 1u;
    } else {
        const double4* pos = reinterpret_cast<const double4*>(a.st.pos);
        const int2* pairs = reinterpret_cast<const int2*>(a.pairs);
        const int64_t Pl = base + g.lane;
        bool live = false;
        if (Pl < hi) {
            const int2 pr = pairs[Pl];
            live = !spheres_apart(pos[pr.x], pos[pr.y]);
            if (!live && a.collision) a.collision[Pl] = 0;
        }
        msk = g.ballot(live);
    }
    while (msk) {
        const int l = __ffs(msk) - 1;
        msk &= msk - 1;
        gjk_pair<LPP>(a, g, base + l, list, list_n);
    }
}

// BT threads per block (64, 128 or 256: the autotuner's block-size knob), registers capped so that
// 896 threads per SM stay resident with one lane per pair (the 256-scene step measured 0.716 ms at
// 7 blocks of 128, 0.720 at 8 and 0.726 at 6) and 768 with lane groups
template <int LPP, int BT>
__global__ void __launch_bounds__(BT, (LPP == 1 ? 896 : 768) / BT) gjk_pass_kernel(NarrowArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    constexpr int GPB = BT / LPP;
    const int grp = threadIdx.x / LPP;
    Group<LPP> g;
    g.lane = threadIdx.x % LPP;
    g.mask = LPP == 32 ? 0xffffffffu : (((1u << LPP) - 1u) << ((threadIdx.x & 31) / LPP * LPP));
    const int64_t m = *a.n_pairs_dev;
    const int64_t n = m < a.pair_cap ? m : a.pair_cap;
    const int chunk = gjk_chunk(a, LPP);
    const int64_t stride = (int64_t)gridDim.x * GPB * chunk;
    for (int64_t base = ((int64_t)blockIdx.x * GPB + grp) * chunk; base < n; base += stride)
        gjk_candidates<LPP>(a, g, base, n, nullptr, nullptr);
}

// ------------------------------------------------------------------ persistent tangential history
// Open-addressing table keyed by the unordered pair (lower id << 32 | higher id; 0 = empty), linear
// probing, the MurmurHash3 64-bit finaliser as the hash.  Values are stored in the (lower, higher)
// orientation: a pair listed the other way round reads and writes the negated displacement.
__device__ __forceinline__ unsigned long long hist_key(int a, int b)
{
    const unsigned lo = (unsigned)(a < b ? a : b), hi = (unsigned)(a < b ? b : a);
    return ((unsigned long long)lo << 32) | hi;
}
__device__ __forceinline__ unsigned long long hist_hash(unsigned long long k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}
__device__ __forceinline__ f3 hist_get(const NarrowArgs& a, int A, int B)
{
    const int par = *a.hist_parity & 1;
    const unsigned long long* K = a.hist_keys + (size_t)par * a.hist_cap;
    const float4* V = a.hist_vals + (size_t)par * a.hist_cap;
    const unsigned long long key = hist_key(A, B);
    const unsigned long long m = (unsigned long long)a.hist_cap - 1;
    unsigned long long slot = hist_hash(key) & m;
    for (int64_t probe = 0; probe < a.hist_cap; ++probe) {
        const unsigned long long k = K[slot];
        if (k == key) {
            const f3 v = xyz(V[slot]);
            return A < B ? v : v * (-1.f);
        }
        if (k == 0ull) break;
        slot = (slot + 1) & m;
    }
    return mk3(0.f, 0.f, 0.f);
}
__device__ __forceinline__ void hist_put(const NarrowArgs& a, int A, int B, f3 dt)
{
    const int par = (*a.hist_parity & 1) ^ 1;
    unsigned long long* K = a.hist_keys + (size_t)par * a.hist_cap;
    float4* V = a.hist_vals + (size_t)par * a.hist_cap;
    const unsigned long long key = hist_key(A, B);
    const unsigned long long m = (unsigned long long)a.hist_cap - 1;
    unsigned long long slot = hist_hash(key) & m;
    for (int64_t probe = 0; probe < a.hist_cap; ++probe) {
        const unsigned long long prev = atomicCAS(K + slot, 0ull, key);
        if (prev == 0ull || prev == key) {
            V[slot] = f4(A < B ? dt : dt * (-1.f), 0.f);
            return;
        }
        slot = (slot + 1) & m;
    }
    set_status(a.status, MWD_ST_HIST_OVERFLOW);
}

// empties the table this narrow phase writes
__global__ void hist_clear_kernel(NarrowArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    const int par = (*a.hist_parity & 1) ^ 1;
    unsigned long long* K = a.hist_keys + (size_t)par * a.hist_cap;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.hist_cap; i += (int64_t)gridDim.x * blockDim.x)
        K[i] = 0ull;
}

// the table just written is read by the next narrow phase
__global__ void hist_flip_kernel(NarrowArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    if (threadIdx.x == 0 && blockIdx.x == 0) *a.hist_parity ^= 1;
}

// CorrectFlat, EPA, force and the outputs for EPA record i, by one group (em: its polytope; hull: its
// staging area when the hulls are staged).  RETRY: the record's face list overflowed in the EPA pass,
// run it with the compacting EPA.
template <int LPP, bool RETRY>
__device__ __forceinline__ void epa_record(const NarrowArgs& a, const Group<LPP>& g, EpaMem* em, float4* hull,
                                           int64_t i)
{
    const float4* wv = reinterpret_cast<const float4*>(a.st.world_verts);
    const SimplexRec* recs = reinterpret_cast<const SimplexRec*>(a.epa_rec);
    const SimplexRec rec = recs[i];
    const int64_t P = rec.P;
    // Only the hulls before the EPA: the pair's other inputs are loaded after it, by the lane that
    // evaluates the force, so that the EPA loop holds fewer registers.  The hulls are staged in shared
    // memory, or read in place from the (L1-cached) vertex table.  (GJK recorded the pair, so both
    // hulls fit the staging area.)
    const int2 pr = reinterpret_cast<const int2*>(a.pairs)[P];
    const int oa = a.st.vert_off[pr.x], ob = a.st.vert_off[pr.y];
    const int nA = a.st.vert_off[pr.x + 1] - oa, nB = a.st.vert_off[pr.y + 1] - ob;
    const float4* hA = hull;
    const float4* hB = hull + a.hull_cap;
    if (a.epa_global) {
        hA = wv + oa;
        hB = wv + ob;
    } else {
        for (int k = g.lane; k < nA; k += LPP) hull[k] = wv[oa + k];
        for (int k = g.lane; k < nB; k += LPP) hull[a.hull_cap + k] = wv[ob + k];
    }
    g.sync();
    Work3 wk = {0u, 0u, 0u};
    f3 S1 = xyz(rec.S[0]), S2 = xyz(rec.S[1]), S3 = xyz(rec.S[2]), S4 = xyz(rec.S[3]);
    int a1 = rec.ia & 0xff, a2 = (rec.ia >> 8) & 0xff, a3 = (rec.ia >> 16) & 0xff, a4 = rec.ia >> 24;
    int b1 = rec.ib & 0xff, b2 = (rec.ib >> 8) & 0xff, b3 = (rec.ib >> 16) & 0xff, b4 = rec.ib >> 24;
    if (is_flat(S1, S2, S3, S4)) {
        f3 d4 = cross(S1, S2);
        support<LPP>(g, hA, nA, hB, nB, d4, S4, a4, b4, wk);
    }
    EpaResult er;
    if (!RETRY)
        epa<LPP>(g, *em, hA, nA, hB, nB, S1, a1, b1, S2, a2, b2, S3, a3, b3, S4, a4, b4, er, wk);
    else
        er = epa_compacting<LPP>(g, em, hA, nA, hB, nB, S1, a1, b1, S2, a2, b2, S3, a3, b3, S4, a4, b4, &wk);
    if (g.lane == 0) {
        bool retry = false;
        if (!RETRY && (er.status & MWD_ST_EPA_OVERFLOW)) {
            // the face list outgrew FCAP: the record runs again with the compacting EPA after this
            // pass (the list of such records permitting; otherwise the truncated result stands, flagged)
            const int slot = atomicAdd(epa_retry_count(a), 1);
            if (slot < EPA_RETRY_CAP) {
                epa_retry_list(a)[slot] = (int32_t)i;
                retry = true;
            }
        }
        if (!retry) {
            PairView p;
            load_pair<1>(a, P, p, nullptr, nullptr, 0, 1, false);
            if (a.hist_keys) {
                p.dt = hist_get(a, p.idA, p.idB);
                p.dtn = sqrtf(p.dt.x * p.dt.x + p.dt.y * p.dt.y + p.dt.z * p.dt.z);
            }
            const mwd_material& M = a.scenes[a.st.info[p.idA] >> 1].mat[p.wall];
            ForceResult fo;
            float imA, imB;
            pair_inv_mass<1>(a, p, M, imA, imB);
            contact_force(p.cA, p.cB, er.depth, er.n, er.cpA, er.cpB, M, p.vA, p.vB, p.wA, p.wB, p.dt, p.qA, p.dtn,
                          p.IsA, p.IsB, imA, imB, fo);
            set_status(a.status, er.status);
            if (a.hist_keys) hist_put(a, p.idA, p.idB, fo.dt);
            if (a.det_out) {
                float4* o = a.det_out + 3 * i;
                o[0] = f4(fo.F, 0.f);
                o[1] = f4(fo.TA, 0.f);
                o[2] = f4(fo.TB, 0.f);
            } else {
                accumulate<1>(a, p, fo);
            }
            if (a.face_ids) {
                int* fid = a.face_ids + 6 * P;
                for (int k = 0; k < 3; ++k) {
                    fid[k] = er.fa[k];
                    fid[3 + k] = er.fb[k];
                }
            }
            if (a.work_counters) {
                atomicAdd(a.work_counters + 0, (unsigned long long)wk.dots);
                atomicAdd(a.work_counters + 1, (unsigned long long)wk.faces);
                atomicAdd(a.work_counters + 2, (unsigned long long)wk.queries);
            }
        }
    }
    g.sync();
}

// the EPA queue's smallest claim, and the fraction of the remaining records per group a claim takes
constexpr int EPA_CLAIM = 2;
constexpr int EPA_GUIDE = 4;

// BT threads per block, registers capped so that 640 threads per SM stay resident (5 blocks of 128)
template <int LPP, int BT>
__global__ void __launch_bounds__(BT, 640 / BT) epa_pass_kernel(NarrowArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    extern __shared__ float4 smem[];
    constexpr int GPB = BT / LPP;
    const int grp = threadIdx.x / LPP;
    Group<LPP> g;
    g.lane = threadIdx.x % LPP;
    g.mask = LPP == 32 ? 0xffffffffu : (((1u << LPP) - 1u) << ((threadIdx.x & 31) / LPP * LPP));
    EpaMem* em = reinterpret_cast<EpaMem*>(smem) + grp;
    float4* hull = reinterpret_cast<float4*>(reinterpret_cast<EpaMem*>(smem) + GPB) + (size_t)grp * 2 * a.hull_cap;
    const int cnt = *a.epa_count;
    const int m = (int64_t)cnt < a.epa_cap ? cnt : (int)a.epa_cap;
    // Persistent over a work queue (guided self-scheduling): every group first takes a fixed share of
    // the records, interleaved with the others' (all of them when there are no more records than
    // groups: no atomic at all); the rest are claimed from the queue in pieces of a quarter of what is
    // left per group, so that the groups that finish early take over the work of the others and the
    // pass ends with its last record rather than with the unluckiest fixed share.  (Record counts are
    // int32.)
    const int G = (int)gridDim.x * GPB;
    const int share = m <= G ? 1 : (m / (2 * G) > 1 ? m / (2 * G) : 1);
    const int fixed = m <= G ? m : G * share;
    unsigned long long* next = epa_queue(a);
    // records i, i + step, ... below e: first the fixed share (step G), then each claimed piece (step 1)
    int i = (int)blockIdx.x * GPB + grp, step = G, e = fixed;
    int seen = 0;  // queue position after this group's last claim
    for (;;) {
        if (i >= e) {
            if (fixed >= m) break;
            int size = (m - fixed - seen) / (EPA_GUIDE * G);
            if (size < EPA_CLAIM) size = EPA_CLAIM;
            const int64_t b = (int64_t)fixed + claim<LPP>(g, next, size);
            if (b >= m) break;
            i = (int)b;
            step = 1;
            e = b + size < m ? (int)b + size : m;
            seen = i - fixed + size;
        }
        epa_record<LPP, false>(a, g, em, hull, i);
        i += step;
    }
}

// The records whose face list overflowed in the EPA pass, run again with the compacting EPA (a
// separate kernel, so that the EPA pass itself carries none of that code; it finds an empty list almost
// always and ends at once)
template <int LPP, int BT>
__global__ void __launch_bounds__(BT, 1) epa_retry_kernel(NarrowArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    extern __shared__ float4 smem[];
    constexpr int GPB = BT / LPP;
    const int grp = threadIdx.x / LPP;
    Group<LPP> g;
    g.lane = threadIdx.x % LPP;
    g.mask = LPP == 32 ? 0xffffffffu : (((1u << LPP) - 1u) << ((threadIdx.x & 31) / LPP * LPP));
    EpaMem* em = reinterpret_cast<EpaMem*>(smem) + grp;
    float4* hull = reinterpret_cast<float4*>(reinterpret_cast<EpaMem*>(smem) + GPB) + (size_t)grp * 2 * a.hull_cap;
    const int c = *epa_retry_count(a);
    const int nr = c < EPA_RETRY_CAP ? c : EPA_RETRY_CAP;
    for (int k = (int)blockIdx.x * GPB + grp; k < nr; k += (int)gridDim.x * GPB)
        epa_record<LPP, true>(a, g, em, hull, epa_retry_list(a)[k]);
}

// threads per block of a block-size code of the lanes word (0: 128, 1: 64, 2: 256)
inline int block_threads(int code) { return code == 1 ? 64 : code == 2 ? 256 : 128; }

template <int LPP, int BT>
int launch_gjk_bt(const NarrowArgs& a, cudaStream_t s)
{
    static LaunchSetup setup;
    int per_sm = 0;
    int rc = launch_setup(setup, gjk_pass_kernel<LPP, BT>, BT, 0, 0, &per_sm);
    if (rc) return rc;
    MWD_CUDA(launch_pdl(gjk_pass_kernel<LPP, BT>, (unsigned)(num_sms() * per_sm), BT, 0, s, a));
    return MWD_OK;
}

template <int LPP>
int launch_gjk(const NarrowArgs& a, int code, cudaStream_t s)
{
    if (code == 1) return launch_gjk_bt<LPP, 64>(a, s);
    if (code == 2) return launch_gjk_bt<LPP, 256>(a, s);
    return launch_gjk_bt<LPP, 128>(a, s);
}

template <int LPP, int BT>
int launch_epa_bt(const NarrowArgs& a, cudaStream_t s)
{
    constexpr int GPB = BT / LPP;
    static LaunchSetup setup;
    int per_sm = 0;
    const size_t shm = (size_t)GPB * sizeof(EpaMem) + (a.epa_global ? 0 : (size_t)GPB * 2 * a.hull_cap * sizeof(float4));
    int rc = launch_setup(setup, epa_pass_kernel<LPP, BT>, BT, shm, 200 * 1024, &per_sm);
    if (rc) return rc;
    MWD_CUDA(launch_pdl(epa_pass_kernel<LPP, BT>, (unsigned)(num_sms() * per_sm), BT, shm, s, a));
    static LaunchSetup retry_setup;
    int retry_per_sm = 0;
    rc = launch_setup(retry_setup, epa_retry_kernel<LPP, BT>, BT, shm, 200 * 1024, &retry_per_sm);
    if (rc) return rc;
    MWD_CUDA(launch_pdl(epa_retry_kernel<LPP, BT>, (unsigned)num_sms(), BT, shm, s, a));
    return MWD_OK;
}

template <int LPP>
int launch_epa(const NarrowArgs& a, int code, cudaStream_t s)
{
    if (code == 1) return launch_epa_bt<LPP, 64>(a, s);
    if (code == 2) return launch_epa_bt<LPP, 256>(a, s);
    return launch_epa_bt<LPP, 128>(a, s);
}

// Resolve the reference's overlapping stride-1 history writes (.cu:1018-1021, :1158-1161): the
// value left at hist[k] is the one written by the highest pair index P' in [k-3, k] that wrote.
__global__ void hist_resolve_kernel(float* hist, const float4* stage, const uint8_t* wrote, int64_t n)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n + 3) return;
    for (int64_t P = (k < n - 1 ? k : n - 1); P >= 0 && P >= k - 3; --P) {
        if (wrote[P]) {
            float4 v = stage[P];
            int j = (int)(k - P);
            hist[k] = j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w;
            return;
        }
    }
}

template <int LPP, int MODE>
int launch_lpp(const NarrowArgs& a, int64_t n_hint, cudaStream_t s)
{
    constexpr int GPB = NARROW_THREADS / LPP;
    size_t shm = (size_t)GPB * sizeof(EpaMem) + (size_t)GPB * 2 * a.hull_cap * sizeof(float4);
    static LaunchSetup setup;
    int per_sm = 0;
    int rc = launch_setup(setup, narrow_kernel<LPP, MODE>, NARROW_THREADS, shm, 200 * 1024, &per_sm);
    if (rc) return rc;
    int64_t grid = (int64_t)num_sms() * per_sm;
    int64_t need = (n_hint + GPB - 1) / GPB;
    if (n_hint >= 0 && need < grid) grid = need > 0 ? need : 1;
    narrow_kernel<LPP, MODE><<<(unsigned)grid, NARROW_THREADS, shm, s>>>(a);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

}  // namespace

size_t narrow_smem_bytes(int lpp, int hull_cap)
{
    int gpb = NARROW_THREADS / lpp;
    return (size_t)gpb * sizeof(EpaMem) + (size_t)gpb * 2 * hull_cap * sizeof(float4);
}

int launch_narrow(const NarrowArgs& a, int mode, int lanes, int64_t n_hint, cudaStream_t s)
{
    if (mode == 0) {
        switch (lanes) {
            case 4: return launch_lpp<4, 0>(a, n_hint, s);
            case 8: return launch_lpp<8, 0>(a, n_hint, s);
            case 16: return launch_lpp<16, 0>(a, n_hint, s);
            case 32: return launch_lpp<32, 0>(a, n_hint, s);
        }
    } else {
        switch (lanes) {
            case 4: return launch_lpp<4, 1>(a, n_hint, s);
            case 8: return launch_lpp<8, 1>(a, n_hint, s);
            case 16: return launch_lpp<16, 1>(a, n_hint, s);
            case 32: return launch_lpp<32, 1>(a, n_hint, s);
        }
    }
    set_error("lanes per pair must be 4, 8, 16 or 32 (got %d)", lanes);
    return MWD_ERR_INVALID;
}

// lanes = GJK-pass lanes per pair | EPA-pass lanes per pair << 8 (EPA lanes 0: same as GJK) | the two
// passes' block-size codes (MWD_LANES_*_BLOCK_SHIFT); whether the EPA pass reads the hulls in place
// comes in NarrowArgs (epa_global)
int launch_narrow_two_pass(const NarrowArgs& a, int lanes, cudaStream_t s)
{
    const int gl = lanes & 0xff;
    int el = (lanes >> 8) & 0xff;
    if (!el) el = gl;
    const int gb = (lanes >> MWD_LANES_GJK_BLOCK_SHIFT) & 3, eb = (lanes >> MWD_LANES_EPA_BLOCK_SHIFT) & 3;
    const bool gl_ok = gl == 1 || gl == 4 || gl == 8 || gl == 16 || gl == 32;
    const bool el_ok = el == 4 || el == 8 || el == 16 || el == 32;
    if (!gl_ok || !el_ok) {
        set_error("lanes per pair must be 1 (GJK pass only), 4, 8, 16 or 32 (got GJK %d, EPA %d)", gl, el);
        return MWD_ERR_INVALID;
    }
    if (gb == 3 || eb == 3) {
        set_error("block-size code must be 0 (128 threads), 1 (64) or 2 (256) (got GJK %d, EPA %d)", gb, eb);
        return MWD_ERR_INVALID;
    }
    if (!a.epa_zeroed) MWD_CUDA(cudaMemsetAsync(a.epa_count, 0, 8 * sizeof(int32_t), s));
    if (a.hist_keys) MWD_CUDA(launch_pdl(hist_clear_kernel, (unsigned)(num_sms() * 4), 256, 0, s, a));
    int rc = MWD_OK;
    switch (gl) {
        case 1: rc = launch_gjk<1>(a, gb, s); break;
        case 4: rc = launch_gjk<4>(a, gb, s); break;
        case 8: rc = launch_gjk<8>(a, gb, s); break;
        case 16: rc = launch_gjk<16>(a, gb, s); break;
        default: rc = launch_gjk<32>(a, gb, s); break;
    }
    if (rc) return rc;
    switch (el) {
        case 4: rc = launch_epa<4>(a, eb, s); break;
        case 8: rc = launch_epa<8>(a, eb, s); break;
        case 16: rc = launch_epa<16>(a, eb, s); break;
        default: rc = launch_epa<32>(a, eb, s); break;
    }
    if (rc) return rc;
    if (a.hist_keys) MWD_CUDA(launch_pdl(hist_flip_kernel, 1, 32, 0, s, a));
    return MWD_OK;
}

int launch_hist_resolve(float* hist, const float* stage, const uint8_t* wrote, int64_t n, cudaStream_t s)
{
    if (n <= 0) return MWD_OK;
    int64_t total = n + 3;
    unsigned grid = (unsigned)((total + 255) / 256);
    hist_resolve_kernel<<<grid, 256, 0, s>>>(hist, reinterpret_cast<const float4*>(stage), wrote, n);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

}  // namespace mwd
