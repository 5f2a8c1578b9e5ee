/* CPU restatement of the MWDiEM narrow phase (GJK + EPA + contact force), one pair at a time.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle the CUDA kernels are checked against.  The product
 * library never links or calls it.
 *
 * Included twice by mwdem_oracle.c, once with ORC_REAL=float and once with ORC_REAL=double, to give
 * the FP32 restatement (the bit-exact target for contact flags) and the FP64 restatement (the
 * tolerance target for depth, normal and force).  Every arithmetic expression keeps the operand
 * types and the evaluation order of the reference kernel, including the places where a double
 * literal promotes a float expression to double (e.g. CorrectFlat's +-1e-6 window, the EPA stop
 * test's 1.00001/0.99999 factors, u = 1.0 - w - v).  Reference: LIBRARIES/gpu_fine_contact_detection.cu.
 *
 * Differences from the reference, all deliberate and mirrored by the CUDA kernel:
 *  - EPA keeps an append-only face list of ORC_FCAP faces and a vertex list of ORC_VCAP entries
 *    instead of T[50]/V[50]; the reference writes past T[50] when more than 50 faces are created
 *    (gpu_fine_contact_detection.cu:359-362,519-539).  More than face_cap faces created (50 selects
 *    the reference's own limit), or more than ORC_LIVE_CAP faces alive at the end of an iteration
 *    (the CUDA kernel keeps only the live faces), stops the EPA and raises ORC_ST_EPA_OVERFLOW.
 *  - the horizon is found by counting, for each edge of each deleted face, how many increments the
 *    reference's delpair[50][50] matrix would have received (gpu_fine_contact_detection.cu:482-493),
 *    without the matrix.
 *  - every pair reads the history array as it was on entry ("snapshot" semantics, what a warp of the
 *    GPU kernel sees); writes are applied in pair order, so overlapping stride-1 writes resolve as
 *    in a serial loop (gpu_fine_contact_detection.cu:974-976,1018-1021).
 */
#ifndef ORC_REAL
#error "define ORC_REAL before including narrow_impl.h"
#endif

#define RT ORC_REAL
typedef struct { RT x, y, z; } ORC_N(v3);
#define V3 ORC_N(v3)

static inline V3 ORC_N(mk)(RT x, RT y, RT z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline V3 ORC_N(add)(V3 a, V3 b) { return ORC_N(mk)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 ORC_N(sub)(V3 a, V3 b) { return ORC_N(mk)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 ORC_N(mul)(V3 a, RT s) { return ORC_N(mk)(a.x * s, a.y * s, a.z * s); }
static inline V3 ORC_N(div)(V3 a, RT s) { return ORC_N(mk)(a.x / s, a.y / s, a.z / s); }
static inline RT ORC_N(dot)(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 ORC_N(cross)(V3 a, V3 b)
{
    return ORC_N(mk)(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

/* Shape access: the vertices of one side of a pair, world frame, stride 3 scalars. */
typedef struct { const RT* p; int n; } ORC_N(hull);

static inline V3 ORC_N(vert)(ORC_N(hull) h, int i) { return ORC_N(mk)(h.p[3 * i], h.p[3 * i + 1], h.p[3 * i + 2]); }

/* argmax over the vertices of A of d.a and over B of (-d).b, strict '>' from -1e30 so the first
 * index wins ties (gpu_fine_contact_detection.cu:55-101). */
static void ORC_N(support)(ORC_N(hull) A, ORC_N(hull) B, V3 d, V3* s, int* ia, int* ib, int* counter)
{
    RT best = (RT)-1e30;
    int bi = 0;
    for (int i = 0; i < A.n; ++i) {
        RT t = ORC_N(dot)(d, ORC_N(vert)(A, i));
        if (t > best) { best = t; bi = i; }
    }
    V3 nd = ORC_N(mul)(d, (RT)-1);
    RT best2 = (RT)-1e30;
    int bj = 0;
    for (int j = 0; j < B.n; ++j) {
        RT t = ORC_N(dot)(nd, ORC_N(vert)(B, j));
        if (t > best2) { best2 = t; bj = j; }
    }
    *ia = bi;
    *ib = bj;
    V3 a = ORC_N(vert)(A, bi), b = ORC_N(vert)(B, bj);
    *s = ORC_N(mk)(a.x - b.x, a.y - b.y, a.z - b.z);
    if (counter) ++*counter;
}

/* Line-segment Voronoi test (gpu_fine_contact_detection.cu:103-124).  coll: -1 keep going, 0
 * separated, 1 origin on the segment line. */
static void ORC_N(seg)(V3 P1, V3 P2, int* coll, V3* d)
{
    *coll = -1;
    *d = ORC_N(mk)(0, 0, 0);
    V3 e = ORC_N(sub)(P2, P1);
    if (ORC_N(dot)(e, P2) < 0.0) { *coll = 0; return; }
    V3 t = ORC_N(cross)(e, P2);
    if (t.x == 0.0 && t.y == 0.0 && t.z == 0.0) { *coll = 1; return; }
    V3 tmp = ORC_N(cross)(e, ORC_N(mul)(P2, (RT)-1));
    *d = ORC_N(cross)(tmp, e);
}

/* Triangle Voronoi test (gpu_fine_contact_detection.cu:127-186).  The direction output is shared
 * with the nested segment tests, exactly as the reference passes its pointer down. */
static void ORC_N(tri)(V3 P1, V3 P2, V3 P3, int* coll, V3* d)
{
    *coll = -1;
    *d = ORC_N(mk)(0, 0, 0);
    int c2, c3;
    ORC_N(seg)(P2, P3, &c2, d);
    if (c2 == 1) { *coll = 1; return; }
    ORC_N(seg)(P1, P3, &c3, d);
    if (c3 == 1) { *coll = 1; return; }
    if (c2 + c3 > -1.0) { *coll = 0; return; }
    V3 e32 = ORC_N(sub)(P3, P2);
    V3 e13 = ORC_N(sub)(P1, P3);
    V3 n = ORC_N(cross)(e32, e13);
    V3 n2 = ORC_N(cross)(e32, n);
    V3 n3 = ORC_N(cross)(e13, n);
    if (ORC_N(dot)(n2, P2) < 0.0) { *d = n2; return; }
    if (ORC_N(dot)(n3, P3) < 0.0) { *d = n3; return; }
    if (ORC_N(dot)(P3, n) == 0.0) { *coll = 1; return; }
    if (ORC_N(dot)(n, P3) > 0.0) *d = ORC_N(mul)(n, (RT)-1.0);
    else *d = n;
}

/* Tetrahedron test (gpu_fine_contact_detection.cu:188-254); todel names the simplex point the
 * driver drops: 3 -> keep (S1,S2,S4), 1 -> (S2,S3,S4), 2 -> (S3,S1,S4). */
static void ORC_N(tet)(V3 P1, V3 P2, V3 P3, V3 P4, int* coll, V3* d, int* todel)
{
    *coll = -1;
    *d = ORC_N(mk)(0, 0, 0);
    *todel = 0;
    int c1, c2, c3;
    ORC_N(tri)(P1, P2, P4, &c1, d);
    if (c1 == 1) { *coll = 1; return; }
    ORC_N(tri)(P2, P3, P4, &c2, d);
    if (c2 == 1) { *coll = 1; return; }
    ORC_N(tri)(P3, P1, P4, &c3, d);
    if (c3 == 1) { *coll = 1; return; }
    if (c1 + c2 + c3 > -2) { *coll = 0; return; }
    V3 e13 = ORC_N(sub)(P1, P3);
    V3 e21 = ORC_N(sub)(P2, P1);
    V3 e32 = ORC_N(sub)(P3, P2);
    V3 e41 = ORC_N(sub)(P4, P1);
    V3 n2 = ORC_N(cross)(e21, e41);
    V3 e42 = ORC_N(sub)(P4, P2);
    V3 n3 = ORC_N(cross)(e32, e42);
    V3 e43 = ORC_N(sub)(P4, P3);
    V3 n4 = ORC_N(cross)(e13, e43);
    if (ORC_N(dot)(n2, P4) < 0.0) { *d = n2; *todel = 3; }
    else if (ORC_N(dot)(n3, P4) < 0.0) { *d = n3; *todel = 1; }
    else if (ORC_N(dot)(n4, P4) < 0.0) { *d = n4; *todel = 2; }
    else *coll = 1;
}

/* Degenerate-simplex check before EPA (gpu_fine_contact_detection.cu:256-268): two 3x3
 * determinants compared with a double +-1e-6 window. */
static int ORC_N(flat)(V3 S1, V3 S2, V3 S3, V3 S4)
{
    RT det1 = S1.x * (S2.y * S3.z - S3.y * S2.z) - S2.x * (S1.y * S3.z - S3.y * S1.z) + S3.x * (S1.y * S2.z - S2.y * S1.z);
    if (det1 < 0.000001 && det1 > -0.000001) {
        RT det2 = S1.x * (S2.y * S4.z - S4.y * S2.z) - S2.x * (S1.y * S4.z - S4.y * S1.z) + S4.x * (S1.y * S2.z - S2.y * S1.z);
        if (det2 < 0.000001 && det2 > -0.000001) return 1;
    }
    return 0;
}

typedef struct {
    V3 V[ORC_VCAP];
    int ia[ORC_VCAP], ib[ORC_VCAP];
    int T[ORC_FCAP][3];
    V3 n[ORC_FCAP];
    RT dist[ORC_FCAP];
    int valid[ORC_FCAP];
    int nv, nt;
} ORC_N(poly);

/* One polytope face from three vertex ids (gpu_fine_contact_detection.cu:270-325): unit normal,
 * flipped (with the winding) to point away from the origin; the face is kept only when the
 * origin's projection falls inside it, otherwise dist = 1e30 and valid = -2. */
static void ORC_N(face)(ORC_N(poly)* p, int e0, int e1, int e2, int f)
{
    p->T[f][0] = e0; p->T[f][1] = e1; p->T[f][2] = e2;
    V3 a = p->V[e0], b = p->V[e1], c = p->V[e2];
    V3 n = ORC_N(cross)(ORC_N(sub)(b, a), ORC_N(sub)(c, b));
    RT len = ORC_SQRT(n.x * n.x + n.y * n.y + n.z * n.z);
    n = ORC_N(div)(n, len);
    RT dist = ORC_N(dot)(n, a);
    p->valid[f] = 1;
    if (dist < 0.0) {
        p->T[f][2] = e1;
        p->T[f][1] = e2;
        dist = dist * (RT)-1.0;
        n = ORC_N(mul)(n, (RT)-1.0);
    }
    V3 A = p->V[p->T[f][0]], B = p->V[p->T[f][1]], C = p->V[p->T[f][2]];
    int inside = 0;
    if (ORC_N(dot)(ORC_N(cross)(ORC_N(sub)(B, A), n), ORC_N(mul)(A, (RT)-1.0)) < 0.0)
        if (ORC_N(dot)(ORC_N(cross)(ORC_N(sub)(C, B), n), ORC_N(mul)(B, (RT)-1.0)) < 0.0)
            if (ORC_N(dot)(ORC_N(cross)(ORC_N(sub)(A, C), n), ORC_N(mul)(C, (RT)-1.0)) < 0.0)
                inside = 1;
    if (!inside) { p->valid[f] = -2; dist = (RT)1e30; }
    p->n[f] = n;
    p->dist[f] = dist;
}

/* number of delpair increments the ordered edge (a,b) receives from the deleted faces */
static int ORC_N(edge_count)(const ORC_N(poly)* p, const int* del, int ndel, int a, int b)
{
    int c = 0;
    for (int k = 0; k < ndel; ++k) {
        const int* t = p->T[del[k]];
        int x = t[0], y = t[1], z = t[2];
        c += (a == y && b == x) + (a == x && b == y) + (a == z && b == y) + (a == y && b == z) +
             (a == x && b == z) + (a == z && b == x);
    }
    return c;
}

typedef struct {
    RT depth;
    V3 normal, cpA, cpB;
    int fa[3], fb[3]; /* support indices of the final face, A side and B side */
    int iters;
    int faces;
    int status;
} ORC_N(epa_out);

/* Expanding polytope (gpu_fine_contact_detection.cu:328-603). */
static void ORC_N(epa)(V3 S1, int a1, int b1, V3 S2, int a2, int b2, V3 S3, int a3, int b3, V3 S4,
                       int a4, int b4, ORC_N(hull) A, ORC_N(hull) B, ORC_N(epa_out)* out, int* nsupport, int fcap)
{
    static ORC_THREAD ORC_N(poly) P;
    ORC_N(poly)* p = &P;
    RT xmin_old = (RT)1e29;
    RT proj = 2 * xmin_old + 1;
    RT xmin_new = 0;
    int counter = 0, indmin = 0;
    out->status = 0;
    out->iters = 0;
    p->nv = 4;
    p->nt = 0;
    p->V[0] = S1; p->V[1] = S2; p->V[2] = S3; p->V[3] = S4;
    p->ia[0] = a1; p->ib[0] = b1; p->ia[1] = a2; p->ib[1] = b2;
    p->ia[2] = a3; p->ib[2] = b3; p->ia[3] = a4; p->ib[3] = b4;
    ORC_N(face)(p, 0, 1, 2, p->nt++);
    ORC_N(face)(p, 1, 2, 3, p->nt++);
    ORC_N(face)(p, 2, 0, 3, p->nt++);
    ORC_N(face)(p, 0, 1, 3, p->nt++);
    int live = 4;
    static ORC_THREAD int del[ORC_FCAP];
    while (xmin_old < proj) {
        /* first index of the minimum, strict '<' from dist[0] */
        indmin = 0;
        RT xm = p->dist[0];
        for (int k = 0; k < p->nt; ++k)
            if (p->dist[k] < xm) { xm = p->dist[k]; indmin = k; }
        xmin_new = p->dist[indmin];
        xmin_old = xmin_new;
        V3 s;
        int sa, sb;
        ORC_N(support)(A, B, p->n[indmin], &s, &sa, &sb, nsupport);
        proj = ORC_N(dot)(p->n[indmin], s);
        if (p->nv < ORC_VCAP) { p->ia[p->nv] = sa; p->ib[p->nv] = sb; }
        out->iters++;
        if (xmin_old > proj || (xmin_old * 1.00001 > proj && xmin_old * 0.99999 < proj)) break;
        if (counter > 49) { out->status |= ORC_ST_EPA_NOCONV; break; }
        counter = counter + 1;
        if (p->nv >= ORC_VCAP) { out->status |= ORC_ST_EPA_OVERFLOW; break; }
        p->V[p->nv] = s;
        p->nv++;
        V3 vn = p->V[p->nv - 1];
        int ndel = 0;
        for (int i = 0; i < p->nt; ++i)
            if ((p->valid[i] == 1 || p->valid[i] == -2) && ORC_N(dot)(ORC_N(sub)(vn, p->V[p->T[i][0]]), p->n[i]) >= (RT)0) {
                p->valid[i] = -1;
                del[ndel++] = i;
            }
        int overflow = 0;
        const int nt_before = p->nt;
        for (int k = 0; k < ndel && !overflow; ++k) {
            int i = del[k];
            int t0 = p->T[i][0], t1 = p->T[i][1], t2 = p->T[i][2];
            int e[3][2] = {{t0, t1}, {t1, t2}, {t2, t0}};
            for (int m = 0; m < 3; ++m) {
                if (ORC_N(edge_count)(p, del, ndel, e[m][0], e[m][1]) < 2) {
                    if (p->nt >= fcap) { overflow = 1; break; }
                    ORC_N(face)(p, e[m][0], e[m][1], p->nv - 1, p->nt);
                    p->nt++;
                }
            }
            p->valid[i] = 0;
            p->dist[i] = (RT)3e20;
        }
        if (overflow) { out->status |= ORC_ST_EPA_OVERFLOW; break; }
        live = live - ndel + (p->nt - nt_before);
        if (live > ORC_LIVE_CAP) { out->status |= ORC_ST_EPA_OVERFLOW; break; }
        counter = counter + 1;
    }
    out->faces = p->nt;
    out->depth = xmin_new;
    int a = p->T[indmin][0], b = p->T[indmin][1], c = p->T[indmin][2];
    V3 n = p->n[indmin];
    V3 Pr = ORC_N(mul)(n, out->depth);
    V3 Va = p->V[a], Vb = p->V[b], Vc = p->V[c];
    V3 v0 = ORC_N(sub)(Vb, Va), v1 = ORC_N(sub)(Vc, Va), v2 = ORC_N(sub)(Pr, Va);
    if (ORC_N(dot)(ORC_N(cross)(v0, v1), n) < 0) { v0 = ORC_N(sub)(Vc, Va); v1 = ORC_N(sub)(Vb, Va); }
    RT v00 = ORC_N(dot)(v0, v0), v01 = ORC_N(dot)(v0, v1), v11 = ORC_N(dot)(v1, v1);
    RT v20 = ORC_N(dot)(v2, v0), v21 = ORC_N(dot)(v2, v1);
    RT den = v00 * v11 - v01 * v01;
    RT bv = (v11 * v20 - v01 * v21) / den;
    RT bw = (v00 * v21 - v01 * v20) / den;
    RT bu = 1.0 - bw - bv;
    out->cpA = ORC_N(add)(ORC_N(add)(ORC_N(mul)(ORC_N(vert)(A, p->ia[a]), bu), ORC_N(mul)(ORC_N(vert)(A, p->ia[b]), bv)),
                          ORC_N(mul)(ORC_N(vert)(A, p->ia[c]), bw));
    out->cpB = ORC_N(add)(ORC_N(add)(ORC_N(mul)(ORC_N(vert)(B, p->ib[a]), bu), ORC_N(mul)(ORC_N(vert)(B, p->ib[b]), bv)),
                          ORC_N(mul)(ORC_N(vert)(B, p->ib[c]), bw));
    out->normal = n;
    out->fa[0] = p->ia[a]; out->fa[1] = p->ia[b]; out->fa[2] = p->ia[c];
    out->fb[0] = p->ib[a]; out->fb[1] = p->ib[b]; out->fb[2] = p->ib[c];
}

/* Hamilton product and q v q2 (gpu_fine_contact_detection.cu:605-643) */
static void ORC_N(qmul)(const RT* q1, const RT* q2, RT* r)
{
    V3 a = ORC_N(mk)(q1[1], q1[2], q1[3]);
    V3 b = ORC_N(mk)(q2[1], q2[2], q2[3]);
    V3 s = ORC_N(add)(ORC_N(add)(ORC_N(mul)(b, q1[0]), ORC_N(mul)(a, q2[0])), ORC_N(cross)(a, b));
    RT f = q1[0] * q2[0] - ORC_N(dot)(a, b);
    r[0] = f; r[1] = s.x; r[2] = s.y; r[3] = s.z;
}

static V3 ORC_N(qtrip)(const RT* q1, V3 v, const RT* q2)
{
    RT vq[4] = {0, v.x, v.y, v.z};
    RT m1[4], m2[4];
    ORC_N(qmul)(vq, q2, m1);
    ORC_N(qmul)(q1, m1, m2);
    return ORC_N(mk)(m2[1], m2[2], m2[3]);
}

typedef struct { V3 F, TA, TB; } ORC_N(force_out);

/* Linear spring-dashpot normal force, tangential spring-dashpot with a Coulomb cap, torques
 * (gpu_fine_contact_detection.cu:647-871).  mu doubles as the effective mass and as the friction
 * coefficient, as in the reference.  dt (the history) is updated in place.
 *
 * prm->physical selects the physical-mass variant of the same law (not in the reference): normal
 * effective mass mn = 1/(imA + imB), tangential mt = 1/(imA + imB + dA^2/IsA + dB^2/IsB) (a wall
 * side, im = 0, adds no term), tc = sqrt(mn (pi^2 + ln^2 en)/Kn), Gn = -2 mn ln en / tc,
 * Kt = mt (pi^2 + ln^2 et)/tc^2, Gt = -2 mt ln et / tc, contact point (cpA + cpB)/2. */
static void ORC_N(force)(V3 cA, V3 cB, RT depth, V3 n, V3 cpA, V3 cpB, const orc_contact_params* prm,
                         V3 vA, V3 vB, V3 wA, V3 wB, V3* dt, const RT* qA, RT dtn, RT IsA, RT IsB,
                         int wall, RT imA, RT imB, ORC_N(force_out)* o)
{
    double Kn = wall ? prm->Kn_wall : prm->Kn;
    double mu = wall ? prm->mu_wall : prm->mu;
    RT en = (RT)(wall ? prm->en_wall : prm->en);
    RT et = (RT)(wall ? prm->et_wall : prm->et);
    RT pii = (RT)3.141592653589793;
    RT Len = ORC_LOG(en), Let = ORC_LOG(et);
    V3 cp;
    RT Gn, Kt, Gt;
    if (!prm->physical) {
        cp = ORC_N(div)(ORC_N(sub)(cpA, cpB), (RT)2);
        V3 dA = ORC_N(sub)(cp, cA), dB = ORC_N(sub)(cp, cB);
        RT dA2 = dA.x * dA.x + dA.y * dA.y + dA.z * dA.z;
        RT dB2 = dB.x * dB.x + dB.y * dB.y + dB.z * dB.z;
        RT tc = ORC_SQRT_D(mu * (pii * pii + Len * Len) / Kn);
        Gn = (-1) * 2 * mu / tc * Len;
        Kt = Kn * (pii * pii + Let * Let) / (pii * pii + Len * Len) * 1 / (1 / mu + dA2 / IsA + dB2 / IsB);
        Gt = (-1) * 2 / (1 / mu + dA2 / IsA + dB2 / IsB) * Let;
    } else {
        cp = ORC_N(div)(ORC_N(add)(cpA, cpB), (RT)2);
        V3 dA = ORC_N(sub)(cp, cA), dB = ORC_N(sub)(cp, cB);
        RT dA2 = dA.x * dA.x + dA.y * dA.y + dA.z * dA.z;
        RT dB2 = dB.x * dB.x + dB.y * dB.y + dB.z * dB.z;
        RT Xn = pii * pii + Len * Len, Xt = pii * pii + Let * Let;
        RT im = imA + imB;
        RT mn = (RT)1 / im;
        RT tc2 = mn * Xn / (RT)Kn;
        RT tc = ORC_SQRT(tc2);
        Gn = (RT)-2 * mn * Len / tc;
        RT Cm = im;
        if (imA != 0) Cm = Cm + dA2 / IsA;
        if (imB != 0) Cm = Cm + dB2 / IsB;
        RT mt = (RT)1 / Cm;
        Kt = mt * Xt / tc2;
        Gt = (RT)-2 * mt * Let / tc;
    }
    if (ORC_N(dot)(ORC_N(sub)(cB, cA), n) < 0.0) n = ORC_N(mul)(n, (RT)-1.0);
    RT nn = ORC_SQRT(n.x * n.x + n.y * n.y + n.z * n.z);
    n = ORC_N(div)(n, nn);
    V3 disp_n = ORC_N(mul)(n, depth);
    V3 u = ORC_N(sub)(ORC_N(sub)(ORC_N(add)(vA, ORC_N(cross)(wA, ORC_N(sub)(cpA, cA))), vB),
                      ORC_N(cross)(wB, ORC_N(sub)(cpB, cB)));
    V3 un = ORC_N(mul)(n, ORC_N(dot)(u, n));
    V3 ut = ORC_N(sub)(u, un);
    RT utn = ORC_SQRT(ut.x * ut.x + ut.y * ut.y + ut.z * ut.z);
    V3 tij = ORC_N(mk)(0, 0, 0);
    if (utn != 0) tij = ORC_N(div)(ut, utn);
    if (utn == 0 && dtn != 0) tij = ORC_N(div)(*dt, dtn);
    V3 Fn = ORC_N(sub)(ORC_N(mul)(ORC_N(mul)(disp_n, (RT)-1), (RT)Kn), ORC_N(mul)(un, Gn));
    RT Fnn = ORC_SQRT(Fn.x * Fn.x + Fn.y * Fn.y + Fn.z * Fn.z);
    V3 Ft = ORC_N(sub)(ORC_N(mul)(ORC_N(mul)(*dt, (RT)-1), Kt), ORC_N(mul)(ut, Gt));
    RT Ftn = ORC_SQRT(Ft.x * Ft.x + Ft.y * Ft.y + Ft.z * Ft.z);
    V3 dt_new;
    if (Ftn > mu * Fnn) Ft = ORC_N(mul)(ORC_N(mul)(ORC_N(mul)(tij, Fnn), (RT)-1), (RT)mu);
    if (Ftn <= mu * Fnn) {
        RT qi[4] = {qA[0], qA[1] * (-1), qA[2] * (-1), qA[3] * (-1)};
        V3 rot = ORC_N(qtrip)(qA, *dt, qi);
        dt_new = ORC_N(add)(rot, ORC_N(mul)(ut, (RT)prm->dt));
    } else {
        V3 t = ORC_N(sub)(ORC_N(mul)(ORC_N(mul)(ORC_N(mul)(tij, Fnn), (RT)mu), (RT)-1), ORC_N(mul)(ut, Gt));
        dt_new = ORC_N(div)(ORC_N(mul)(t, (RT)1), Kt);
    }
    *dt = dt_new;
    V3 Ff = ORC_N(add)(Ft, Fn);
    o->F = Fn;
    o->TA = ORC_N(cross)(ORC_N(sub)(cp, cA), Ff);
    o->TB = ORC_N(cross)(ORC_N(sub)(cp, cB), ORC_N(mul)(Ff, (RT)-1));
}

/* Full pair pipeline over arrays in the reference's per-pair layout
 * (gpu_fine_contact_detection.cu:874-1322).  Pairs run in index order; force/torque accumulate in
 * that order.  Diagnostics (depth, normal, contact points, status, counters) are optional. */
void ORC_N(orc_contact)(int npairs, int V, const RT* Acom, const RT* Bcom, const RT* Av, const RT* Bv,
                        const RT* Avel, const RT* Bvel, const RT* Aw, const RT* Bw, const int* Anv,
                        const int* Bnv, const int* Aid, const int* Bid, RT* hist, RT* force, RT* torque,
                        const RT* qA, const RT* qB, const RT* IsA, const RT* IsB, int* collision,
                        const orc_contact_params* prm, RT* diag, int* status, int* counters, const RT* imA,
                        const RT* imB)
{
    int stride4 = prm->hist_stride4;
    int fcap = (prm->face_cap > 4 && prm->face_cap < ORC_FCAP) ? prm->face_cap : ORC_FCAP;
    /* snapshot of the history as every pair sees it on entry */
    RT* hin = NULL;
    if (!stride4) {
        size_t nh = (size_t)npairs * 4;
        hin = (RT*)malloc(nh * sizeof(RT) + 4 * sizeof(RT));
        memcpy(hin, hist, nh * sizeof(RT));
    }
    for (int P = 0; P < npairs; ++P) {
        V3 cA = ORC_N(mk)(Acom[3 * P], Acom[3 * P + 1], Acom[3 * P + 2]);
        V3 cB = ORC_N(mk)(Bcom[3 * P], Bcom[3 * P + 1], Bcom[3 * P + 2]);
        V3 vA = ORC_N(mk)(Avel[3 * P], Avel[3 * P + 1], Avel[3 * P + 2]);
        V3 vB = ORC_N(mk)(Bvel[3 * P], Bvel[3 * P + 1], Bvel[3 * P + 2]);
        V3 wA = ORC_N(mk)(Aw[3 * P], Aw[3 * P + 1], Aw[3 * P + 2]);
        V3 wB = ORC_N(mk)(Bw[3 * P], Bw[3 * P + 1], Bw[3 * P + 2]);
        int idA = Aid[P], idB = Bid[P];
        const RT* qa = qA + 4 * P;
        ORC_N(hull) HA = {Av + (size_t)P * V * 3, Anv[P]};
        ORC_N(hull) HB = {Bv + (size_t)P * V * 3, Bnv[P]};
        size_t hb = stride4 ? (size_t)4 * P : (size_t)P;
        const RT* hr = stride4 ? hist : hin;
        V3 dt = ORC_N(mk)(hr[hb], hr[hb + 1], hr[hb + 2]);
        RT dtn = ORC_SQRT(dt.x * dt.x + dt.y * dt.y + dt.z * dt.z);
        RT IA = IsA[P], IB = IsB[P];
        int wall = (idA < prm->n_wall || idB < prm->n_wall) ? 1 : 0;
        int nsup = 0, iters = 0, st = 0, coll = -1, resolved = 0;
        V3 F = ORC_N(mk)(0, 0, 0), TA = F, TB = F;
        ORC_N(epa_out) eo;
        memset(&eo, 0, sizeof(eo));
        collision[P] = -1;
        V3 S1, S2, S3, S4, d3, d4;
        int a1, b1, a2, b2, a3, b3, a4, b4, todel;
        int early = 0;
        V3 d1 = ORC_N(sub)(cB, cA);
        ORC_N(support)(HA, HB, d1, &S1, &a1, &b1, &nsup);
        if (ORC_N(dot)(d1, S1) < 0.0) early = 1;
        if (!early) {
            V3 d2 = ORC_N(mul)(d1, (RT)-1);
            ORC_N(support)(HA, HB, d2, &S2, &a2, &b2, &nsup);
            if (ORC_N(dot)(d2, S2) < 0.0) early = 1;
        }
        if (!early) {
            ORC_N(seg)(S1, S2, &coll, &d3);
            if (coll == 0) early = 1;
        }
        if (!early) {
            ORC_N(support)(HA, HB, d3, &S3, &a3, &b3, &nsup);
            if (ORC_N(dot)(d3, S3) < 0.0) early = 1;
        }
        if (!early) {
            ORC_N(tri)(S1, S2, S3, &coll, &d4);
            if (coll == 0) early = 1;
        }
        if (!early) {
            int zz = 0;
            while (zz < 50) {
                ORC_N(support)(HA, HB, d4, &S4, &a4, &b4, &nsup);
                iters++;
                if (ORC_N(dot)(d4, S4) < 0.0) { early = 1; break; }
                int hit = 0;
                if (S4.x == 0.0 && S4.y == 0.0 && S4.z == 0.0) hit = 1;
                else {
                    ORC_N(tet)(S1, S2, S3, S4, &coll, &d4, &todel);
                    if (coll == 0) { early = 1; break; }
                    if (coll == 1) hit = 1;
                }
                if (hit) {
                    coll = 1;
                    if (ORC_N(flat)(S1, S2, S3, S4)) {
                        d4 = ORC_N(cross)(S1, S2);
                        ORC_N(support)(HA, HB, d4, &S4, &a4, &b4, &nsup);
                    }
                    collision[P] = 1;
                    ORC_N(epa)(S1, a1, b1, S2, a2, b2, S3, a3, b3, S4, a4, b4, HA, HB, &eo, &nsup, fcap);
                    ORC_N(force_out) fo;
                    ORC_N(force)(cA, cB, eo.depth, eo.normal, eo.cpA, eo.cpB, prm, vA, vB, wA, wB, &dt, qa,
                                 dtn, IA, IB, wall, imA ? imA[P] : (RT)0, imB ? imB[P] : (RT)0, &fo);
                    F = fo.F; TA = fo.TA; TB = fo.TB;
                    st |= eo.status;
                    resolved = 1;
                    break;
                }
                V3 n1, n2, n3;
                int na1, nb1, na2, nb2, na3, nb3;
                if (todel == 1) { n1 = S2; na1 = a2; nb1 = b2; n2 = S3; na2 = a3; nb2 = b3; n3 = S4; na3 = a4; nb3 = b4; }
                else if (todel == 2) { n1 = S3; na1 = a3; nb1 = b3; n2 = S1; na2 = a1; nb2 = b1; n3 = S4; na3 = a4; nb3 = b4; }
                else { n1 = S1; na1 = a1; nb1 = b1; n2 = S2; na2 = a2; nb2 = b2; n3 = S4; na3 = a4; nb3 = b4; }
                S1 = n1; a1 = na1; b1 = nb1; S2 = n2; a2 = na2; b2 = nb2; S3 = n3; a3 = na3; b3 = nb3;
                zz = zz + 1;
            }
            if (!early && !resolved) st |= ORC_ST_GJK_NOCONV;
        }
        size_t wb = stride4 ? (size_t)4 * P : (size_t)P;
        if (early) {
            collision[P] = 0;
            hist[wb] = 0; hist[wb + 1] = 0; hist[wb + 2] = 0; hist[wb + 3] = 0;
        } else {
            if (resolved) {
                hist[wb] = dt.x; hist[wb + 1] = dt.y; hist[wb + 2] = dt.z; hist[wb + 3] = 1;
            }
            force[3 * idA] += F.x; force[3 * idA + 1] += F.y; force[3 * idA + 2] += F.z;
            force[3 * idB] += -1 * F.x; force[3 * idB + 1] += -1 * F.y; force[3 * idB + 2] += -1 * F.z;
            torque[3 * idA] += TA.x; torque[3 * idA + 1] += TA.y; torque[3 * idA + 2] += TA.z;
            torque[3 * idB] += TB.x; torque[3 * idB + 1] += TB.y; torque[3 * idB + 2] += TB.z;
        }
        if (diag) {
            RT* dg = diag + (size_t)ORC_DIAG * P;
            dg[0] = eo.depth;
            dg[1] = eo.normal.x; dg[2] = eo.normal.y; dg[3] = eo.normal.z;
            dg[4] = eo.cpA.x; dg[5] = eo.cpA.y; dg[6] = eo.cpA.z;
            dg[7] = eo.cpB.x; dg[8] = eo.cpB.y; dg[9] = eo.cpB.z;
            dg[10] = F.x; dg[11] = F.y; dg[12] = F.z;
            dg[13] = TA.x; dg[14] = TA.y; dg[15] = TA.z;
            dg[16] = TB.x; dg[17] = TB.y; dg[18] = TB.z;
        }
        if (status) status[P] = st;
        if (counters) {
            int* c = counters + ORC_NCOUNT * P;
            c[0] = nsup; c[1] = iters; c[2] = eo.iters;
            c[3] = eo.fa[0]; c[4] = eo.fa[1]; c[5] = eo.fa[2];
            c[6] = eo.fb[0]; c[7] = eo.fb[1]; c[8] = eo.fb[2]; c[9] = eo.faces;
        }
    }
    free(hin);
}

#undef V3
#undef RT
