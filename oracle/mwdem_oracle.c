/* MWDiEM hot-path oracle: plain-C restatement of the reference's per-step algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA library under mwdiem_gb300/ never links, loads or calls this
 * code; it is loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU reference arm, as
 * the checker and as the timed CPU baseline.
 *
 * Contents (each function cites the reference file:line it restates):
 *   orc_contact_f32 / orc_contact_f64   narrow phase + contact force   (narrow_impl.h)
 *   orc_verlet_f64                      quaternion leapfrog integrator  (gpu_Verlet.cu:85-431)
 *   orc_cell_keys                       cell hash of the centres        (MWDiem.py:813-816)
 *   orc_wall_pairs                      wall-particle candidates        (MWDiem.py:808-811)
 *   orc_linked_cell_hash                cell-pair candidates            (LIBRARY_Coarse_contact_detection.py:84-155)
 *   orc_pyset_order                     CPython 3.12 set iteration order of small int sets
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fno-fast-math -fopenmp -shared -fPIC (oracle/build.py).
 * -ffp-contract=off matters: GCC on aarch64 fuses a*b+c into FMA by default, which changes FP32
 * rounding.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_VCAP 64
#define ORC_FCAP 4096      /* faces an EPA may create (storage; the reference's T[50] overflows at 50) */
#define ORC_LIVE_CAP 127   /* faces alive at once in the CUDA kernel's compacting EPA (MWD_EPA_FACE_CAP - 1) */
#define ORC_DIAG 19
#define ORC_NCOUNT 10
#define ORC_ST_EPA_NOCONV 1
#define ORC_ST_EPA_OVERFLOW 2
#define ORC_ST_GJK_NOCONV 4
#define ORC_THREAD _Thread_local

typedef struct {
    double Kn, en, et, mu;
    double Kn_wall, en_wall, et_wall, mu_wall;
    double dt;
    int n_wall;
    int hist_stride4; /* 0: reference stride-1 history indexing, 1: stride 4 */
    int face_cap;     /* faces an EPA may create (<= ORC_FCAP; 50 is the reference's T[50]); 0 -> ORC_FCAP */
    int physical;     /* 1: the physical-mass contact law (effective masses, midpoint contact point) */
} orc_contact_params;

/* ---------------- narrow phase, FP32 ---------------- */
#define ORC_REAL float
#define ORC_N(x) x##_f32
#define ORC_SQRT(x) sqrtf(x)
#define ORC_SQRT_D(x) sqrt(x)
#define ORC_LOG(x) logf(x)
#include "narrow_impl.h"
#undef ORC_REAL
#undef ORC_N
#undef ORC_SQRT
#undef ORC_SQRT_D
#undef ORC_LOG

/* ---------------- narrow phase, FP64 ---------------- */
#define ORC_REAL double
#define ORC_N(x) x##_f64
#define ORC_SQRT(x) sqrt(x)
#define ORC_SQRT_D(x) sqrt(x)
#define ORC_LOG(x) log(x)
#include "narrow_impl.h"
#undef ORC_REAL
#undef ORC_N
#undef ORC_SQRT
#undef ORC_SQRT_D
#undef ORC_LOG

int orc_face_capacity(void) { return ORC_FCAP; }

/* ---------------- integrator, FP64 (gpu_Verlet.cu:85-431) ---------------- */
typedef struct { double x, y, z; } d3;
static inline d3 d3m(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 d3add(d3 a, d3 b) { return d3m(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 d3sub(d3 a, d3 b) { return d3m(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 d3mul(d3 a, double s) { return d3m(a.x * s, a.y * s, a.z * s); }
static inline d3 d3div(d3 a, double s) { return d3m(a.x / s, a.y / s, a.z / s); }
static inline double d3dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 d3cross(d3 a, d3 b) { return d3m(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline d3 d3ld(const double* p) { return d3m(p[0], p[1], p[2]); }
static inline void d3st(double* p, d3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

static void qmul_d(const double* a, const double* b, double* r)
{
    d3 u = d3m(a[1], a[2], a[3]), v = d3m(b[1], b[2], b[3]);
    d3 s = d3add(d3add(d3mul(v, a[0]), d3mul(u, b[0])), d3cross(u, v));
    double f = a[0] * b[0] - d3dot(u, v);
    r[0] = f; r[1] = s.x; r[2] = s.y; r[3] = s.z;
}
static void qinv_d(const double* q, double* r) { r[0] = q[0]; r[1] = q[1] * (-1); r[2] = q[2] * (-1); r[3] = q[3] * (-1); }
static d3 qtrip_d(const double* q1, d3 v, const double* q2)
{
    double vq[4] = {0, v.x, v.y, v.z}, m1[4], m2[4];
    qmul_d(vq, q2, m1);
    qmul_d(q1, m1, m2);
    return d3m(m2[1], m2[2], m2[3]);
}
static d3 matvec_d(const double* M, d3 v)
{
    return d3m(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z,
               M[6] * v.x + M[7] * v.y + M[8] * v.z);
}

typedef struct {
    double dt;
    double box[6]; /* xmax, xmin, ymax, ymin, zmax, zmin */
    int n_min, n_max, V;
    int physical; /* 1: rotate the vertices by this step's rotation q_new q_old^-1 instead of by q */
} orc_verlet_params;

/* Arrays in the reference's layout (MWDiem.py:603-631): v, v12, w12bf, wbf, w, F, T, com, dxall
 * (N,3); q12, q, qall (N,4); verts (N,V,3); mass (N,); Iinv, I (N,3,3).  Returns the number of
 * particles reset by the fly-away box. */
int orc_verlet_f64(int N, double* v, double* v12, double* w12bf, double* q12, double* q, double* qall,
                   double* wbf, double* w, const double* F, const double* T, double* verts, double* com,
                   const double* mass, const double* Iinv, const double* I, double* dxall,
                   const orc_verlet_params* prm)
{
    const double dt = prm->dt;
    const int V = prm->V;
    int nreset = 0;
    for (int P = 0; P < N; ++P) {
        if (!(P >= prm->n_min && P < prm->n_max)) continue;
        d3 vel = d3ld(v + 3 * P), vel12 = d3ld(v12 + 3 * P), om12bf = d3ld(w12bf + 3 * P);
        d3 ombf = d3ld(wbf + 3 * P), om = d3ld(w + 3 * P), c = d3ld(com + 3 * P);
        d3 f = d3ld(F + 3 * P), t = d3ld(T + 3 * P);
        double m = mass[P];
        const double* Mi = Iinv + 9 * P;
        const double* Mm = I + 9 * P;
        double qq[4], qa[4], qh[4];
        for (int i = 0; i < 4; ++i) { qq[i] = q[4 * P + i]; qa[i] = qall[4 * P + i]; qh[i] = q12[4 * P + i]; }
        d3 dxa = d3ld(dxall + 3 * P);

        d3 v32 = d3add(vel12, d3mul(d3div(d3mul(f, 1), m), dt));
        double qi[4];
        qinv_d(qq, qi);
        d3 tbf = qtrip_d(qi, t, qq);
        d3 p1 = matvec_d(Mm, ombf);
        d3 p2 = d3sub(tbf, d3cross(ombf, p1));
        d3 alpha = matvec_d(Mi, p2);
        d3 om32bf = d3add(om12bf, d3mul(alpha, dt));
        double wn = sqrt(om.x * om.x + om.y * om.y + om.z * om.z);
        d3 h = d3m(0, 0, 0);
        if (wn != 0) h = d3mul(d3div(om, wn), sin(wn * dt / 2));
        double rq[4] = {cos(wn * dt / 2), h.x, h.y, h.z};
        double q32[4];
        qmul_d(rq, qh, q32);
        vel12 = v32;
        for (int i = 0; i < 4; ++i) qh[i] = q32[i];
        om12bf = om32bf;
        d3 dx = d3mul(vel12, dt);
        dxa = d3add(dxa, dx);
        d3 om34bf = d3add(om12bf, d3div(d3mul(d3mul(alpha, dt), 1), 4));
        double qhi[4];
        qinv_d(qh, qhi);
        d3 om34 = qtrip_d(qh, om34bf, qhi);
        double wn34 = sqrt(om34.x * om34.x + om34.y * om34.y + om34.z * om34.z);
        d3 h2 = d3m(0, 0, 0);
        if (wn34 != 0) h2 = d3mul(d3div(om34, wn34), sin(wn34 * dt / 4));
        double rq2[4] = {cos(wn34 * dt / 4), h2.x, h2.y, h2.z};
        double qold[4] = {qq[0], qq[1], qq[2], qq[3]};
        qmul_d(rq2, qh, qq);
        qmul_d(qq, qold, qa);
        ombf = d3add(om12bf, d3div(d3mul(d3mul(alpha, dt), 1), 2));
        double qqi[4];
        qinv_d(qq, qqi);
        om = qtrip_d(qq, ombf, qqi);
        vel = d3add(vel12, d3div(d3mul(f, dt), m));
        double* vp = verts + (size_t)P * V * 3;
        double qr[4], qri[4];
        if (prm->physical) {  /* the vertices follow the orientation: rotate by q_new q_old^-1 */
            double qoi[4];
            qinv_d(qold, qoi);
            qmul_d(qq, qoi, qr);
        } else {              /* the reference rotates them by the whole orientation q every step */
            for (int i = 0; i < 4; ++i) qr[i] = qq[i];
        }
        qinv_d(qr, qri);
        for (int i = 0; i < V; ++i) {
            d3 r = d3sub(d3ld(vp + 3 * i), c);
            d3st(vp + 3 * i, d3add(qtrip_d(qr, r, qri), c));
        }
        c = d3add(c, dx);
        for (int i = 0; i < V; ++i) d3st(vp + 3 * i, d3add(d3ld(vp + 3 * i), dx));
        if (c.x > prm->box[0] || c.x < prm->box[1] || c.y > prm->box[2] || c.y < prm->box[3] ||
            c.z > prm->box[4] || c.z < prm->box[5]) {
            nreset++;
            vel = d3m(0, 0, 0); vel12 = vel; om12bf = vel; ombf = vel; om = vel;
            d3 back = d3mul(dx, -1);
            c = d3add(c, back);
            for (int i = 0; i < V; ++i) d3st(vp + 3 * i, d3add(d3ld(vp + 3 * i), back));
        }
        d3st(v + 3 * P, vel); d3st(v12 + 3 * P, vel12); d3st(w12bf + 3 * P, om12bf);
        d3st(com + 3 * P, c); d3st(dxall + 3 * P, dxa); d3st(wbf + 3 * P, ombf); d3st(w + 3 * P, om);
        for (int i = 0; i < 4; ++i) { q12[4 * P + i] = qh[i]; q[4 * P + i] = qq[i]; qall[4 * P + i] = qa[i]; }
    }
    return nreset;
}

/* ---------------- broad phase ---------------- */

/* Cell key of every centre (MWDiem.py:813-816): numpy's astype(int) truncates toward zero. */
void orc_cell_keys(int N, const double* com, double csx, double csy, double csz, int64_t nx, int64_t ny,
                   int64_t* keys)
{
    for (int i = 0; i < N; ++i) {
        int64_t xc = (int64_t)(com[3 * i] / csx);
        int64_t yc = (int64_t)(com[3 * i + 1] / csy);
        int64_t zc = (int64_t)(com[3 * i + 2] / csz);
        keys[i] = xc + yc * nx + zc * nx * ny;
    }
}

/* Wall candidates (MWDiem.py:808-811): wall k outer, particle j inner, pair [j, k] when
 * |n_k . (c_j - c_k)| < range.  Returns the number of pairs (written up to cap). */
int64_t orc_wall_pairs(int n_wall, int n_lo, int n_hi, const double* com, const double* wall_n,
                       const double* wall_c, double range, int32_t* out, int64_t cap)
{
    int64_t n = 0;
    for (int k = 0; k < n_wall; ++k)
        for (int j = n_lo; j < n_hi; ++j) {
            double dx = com[3 * j] - wall_c[3 * k], dy = com[3 * j + 1] - wall_c[3 * k + 1], dz = com[3 * j + 2] - wall_c[3 * k + 2];
            double s = wall_n[3 * k] * dx + wall_n[3 * k + 1] * dy + wall_n[3 * k + 2] * dz;
            if (fabs(s) < range) {
                if (n < cap) { out[2 * n] = j; out[2 * n + 1] = k; }
                n++;
            }
        }
    return n;
}

/* Iteration order of a CPython 3.12 set of small non-negative ints, built by .add() in the given
 * order (hash(i) == i).  Open addressing: slot = hash & mask, up to LINEAR_PROBES=9 adjacent slots
 * when they fit below mask, then perturb >>= 5; i = (5 i + 1 + perturb) & mask; the table (8
 * slots at first) is rebuilt at used*4 when fill*5 >= mask*3, re-inserting in old slot order.
 * Writes the members in iteration order to out; returns 0, or -1 when n exceeds the supported
 * size. */
#define PYSET_MAXTAB 1024
int orc_pyset_order(int n, const int64_t* ids, int64_t* out)
{
    int64_t tab[PYSET_MAXTAB], tmp[PYSET_MAXTAB];
    uint8_t used[PYSET_MAXTAB], used2[PYSET_MAXTAB];
    size_t mask = 7;
    int fill = 0;
    memset(used, 0, sizeof(used));
    for (int e = 0; e < n; ++e) {
        uint64_t h = (uint64_t)ids[e];
        size_t i = (size_t)(h & mask);
        uint64_t perturb = h;
        int dup = 0;
        for (;;) {
            size_t j = i;
            int probes = (i + 9 <= mask) ? 9 : 0;
            int found = 0;
            for (;;) {
                if (!used[j]) { found = 1; break; }
                if (tab[j] == ids[e]) { dup = 1; found = 1; break; }
                if (probes-- == 0) break;
                j++;
            }
            if (found) { i = j; break; }
            perturb >>= 5;
            i = (size_t)((i * 5 + 1 + perturb) & mask);
        }
        if (dup) continue;
        used[i] = 1;
        tab[i] = ids[e];
        fill++;
        if ((size_t)fill * 5 >= mask * 3) {
            size_t newsize = 8;
            size_t minused = (size_t)fill * 4;
            while (newsize <= minused) newsize <<= 1;
            if (newsize > PYSET_MAXTAB) return -1;
            size_t newmask = newsize - 1;
            memset(used2, 0, newsize);
            for (size_t s = 0; s <= mask; ++s) {
                if (!used[s]) continue;
                uint64_t hh = (uint64_t)tab[s];
                size_t ii = (size_t)(hh & newmask);
                uint64_t pp = hh;
                for (;;) {
                    if (!used2[ii]) break;
                    int placed = 0;
                    if (ii + 9 <= newmask) {
                        for (int q = 1; q <= 9; ++q)
                            if (!used2[ii + q]) { ii = ii + q; placed = 1; break; }
                    }
                    if (placed) break;
                    pp >>= 5;
                    ii = (size_t)((ii * 5 + 1 + pp) & newmask);
                }
                used2[ii] = 1;
                tmp[ii] = tab[s];
            }
            mask = newmask;
            memcpy(used, used2, newsize);
            memcpy(tab, tmp, newsize * sizeof(int64_t));
        }
    }
    int k = 0;
    for (size_t s = 0; s <= mask; ++s)
        if (used[s]) out[k++] = tab[s];
    return 0;
}

typedef struct { int64_t key; int32_t id; int32_t pad; } keyid;
static int keyid_cmp(const void* a, const void* b)
{
    const keyid* x = (const keyid*)a;
    const keyid* y = (const keyid*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->id < y->id ? -1 : (x->id > y->id);
}

static int64_t find_group(const int64_t* gkey, int ng, int64_t key)
{
    int lo = 0, hi = ng - 1;
    while (lo <= hi) {
        int mid = (lo + hi) / 2;
        if (gkey[mid] == key) return mid;
        if (gkey[mid] < key) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

/* Cell candidates (LIBRARY_Coarse_contact_detection.py:84-155).  Ids in [n_lo, n_hi) are grouped
 * by keys[id]; for each cell (in order of first appearance by id) emit the same-cell pairs (j<k in
 * CPython set order), then pairs with the cells key+1, key+nx, key+nx*ny, key+nx*ny+1,
 * key+nx*ny+1+nx, key+nx*ny+nx, key+nx+1 (A from the cell, B from the neighbour), members in set
 * order.  The output is the reference's list exactly.  Returns the number of pairs. */
int64_t orc_linked_cell_hash(int n_lo, int n_hi, const int64_t* keys, int64_t nx, int64_t ny,
                             int32_t* out, int64_t cap)
{
    int n = n_hi - n_lo;
    if (n <= 0) return 0;
    keyid* kv = (keyid*)malloc(sizeof(keyid) * n);
    for (int i = 0; i < n; ++i) { kv[i].key = keys[n_lo + i]; kv[i].id = n_lo + i; kv[i].pad = 0; }
    qsort(kv, n, sizeof(keyid), keyid_cmp);
    int64_t* gkey = (int64_t*)malloc(sizeof(int64_t) * n);
    int* gstart = (int*)malloc(sizeof(int) * (n + 1));
    int* gfirst = (int*)malloc(sizeof(int) * n);
    int ng = 0;
    for (int i = 0; i < n; ++i) {
        if (i == 0 || kv[i].key != kv[i - 1].key) { gkey[ng] = kv[i].key; gstart[ng] = i; gfirst[ng] = kv[i].id; ng++; }
    }
    gstart[ng] = n;
    /* members of each group in CPython set order */
    int64_t* mem = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* buf = (int64_t*)malloc(sizeof(int64_t) * n);
    for (int g = 0; g < ng; ++g) {
        int s = gstart[g], e = gstart[g + 1];
        for (int i = s; i < e; ++i) buf[i - s] = kv[i].id;
        if (orc_pyset_order(e - s, buf, mem + s) != 0)
            for (int i = s; i < e; ++i) mem[i] = buf[i - s];
    }
    /* groups in order of first appearance: ids are inserted ascending, so order by first id */
    int* order = (int*)malloc(sizeof(int) * ng);
    {
        /* counting by first id */
        int* pos = (int*)malloc(sizeof(int) * n);
        for (int i = 0; i < n; ++i) pos[i] = -1;
        for (int g = 0; g < ng; ++g) pos[gfirst[g] - n_lo] = g;
        int k = 0;
        for (int i = 0; i < n; ++i) if (pos[i] >= 0) order[k++] = pos[i];
        free(pos);
    }
    const int64_t offs[7] = {1, nx, nx * ny, nx * ny + 1, nx * ny + 1 + nx, nx * ny + nx, nx + 1};
    int64_t np = 0;
    for (int oi = 0; oi < ng; ++oi) {
        int g = order[oi];
        int s = gstart[g], e = gstart[g + 1];
        for (int j = s; j < e; ++j)
            for (int k = j + 1; k < e; ++k) {
                if (np < cap) { out[2 * np] = (int32_t)mem[j]; out[2 * np + 1] = (int32_t)mem[k]; }
                np++;
            }
        for (int o = 0; o < 7; ++o) {
            int64_t h = find_group(gkey, ng, gkey[g] + offs[o]);
            if (h < 0) continue;
            int s2 = gstart[h], e2 = gstart[h + 1];
            for (int j = s; j < e; ++j)
                for (int k = s2; k < e2; ++k) {
                    if (np < cap) { out[2 * np] = (int32_t)mem[j]; out[2 * np + 1] = (int32_t)mem[k]; }
                    np++;
                }
        }
    }
    free(kv); free(gkey); free(gstart); free(gfirst); free(mem); free(buf); free(order);
    return np;
}
