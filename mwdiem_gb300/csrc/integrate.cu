// Quaternion leapfrog integrator (gpu_Verlet.cu:85-431), two variants:
//
//  * verlet_ref_kernel -- FP64 over the reference's own arrays (the drop-in for gpu_Verlet.Verlet_GPU).
//    Same operation sequence as the reference; the per-vertex rotation of the world-frame vertex
//    table (gpu_Verlet.cu:279-323) is done block-cooperatively so the (N,V,3) array is read and
//    written with coalesced accesses instead of one thread walking V vertices.
//
//  * integrate_kernel -- FP32 state in float4 structure-of-arrays with FP64 centres (the
//    device-resident step).  Instead of rotating every world vertex by q each step (which compounds
//    the rotation, gpu_Verlet.cu:279-305), it keeps q_acc = q_k (x) q_acc, the product of those
//    rotations, and regenerates world = pos + R(q_acc) r0 from the body-frame table: the same
//    vertices, without accumulating rounding in the vertex coordinates.  Walls are not integrated
//    (rows below num_part_min, gpu_Verlet.cu:110).  The force/torque accumulators are consumed and
//    zeroed for the next step.
#include "common.cuh"
#include "integrate.cuh"

namespace mwd {

namespace {

struct d3 {
    double x, y, z;
};
__device__ __forceinline__ d3 dm(double x, double y, double z)
{
    d3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return dm(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return dm(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ d3 operator*(d3 a, double s) { return dm(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ d3 operator/(d3 a, double s) { return dm(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 dcross(d3 a, d3 b) { return dm(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ d3 dld(const double* p) { return dm(p[0], p[1], p[2]); }
__device__ __forceinline__ void dst(double* p, d3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

struct dq {
    double w, x, y, z;
};
// Hamilton product, operand order of gpu_Verlet.cu:43-54
__device__ __forceinline__ dq dqmul(dq a, dq b)
{
    d3 u = dm(a.x, a.y, a.z), v = dm(b.x, b.y, b.z);
    d3 s = (v * a.w + u * b.w) + dcross(u, v);
    dq r;
    r.w = a.w * b.w - ddot(u, v);
    r.x = s.x;
    r.y = s.y;
    r.z = s.z;
    return r;
}
__device__ __forceinline__ dq dqinv(dq q)
{
    dq r;
    r.w = q.w;
    r.x = q.x * (-1);
    r.y = q.y * (-1);
    r.z = q.z * (-1);
    return r;
}
__device__ __forceinline__ d3 dqtrip(dq q1, d3 v, dq q2)
{
    dq vq;
    vq.w = 0;
    vq.x = v.x;
    vq.y = v.y;
    vq.z = v.z;
    dq m = dqmul(q1, dqmul(vq, q2));
    return dm(m.x, m.y, m.z);
}
__device__ __forceinline__ dq dqld(const double* p)
{
    dq q;
    q.w = p[0];
    q.x = p[1];
    q.y = p[2];
    q.z = p[3];
    return q;
}
__device__ __forceinline__ void dqst(double* p, dq q)
{
    p[0] = q.w;
    p[1] = q.x;
    p[2] = q.y;
    p[3] = q.z;
}
__device__ __forceinline__ d3 matvec(const double* M, d3 v)
{
    return dm(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z, M[6] * v.x + M[7] * v.y + M[8] * v.z);
}

constexpr int RB = 128;  // rows per block

__global__ void __launch_bounds__(RB) verlet_ref_kernel(VerletRefArgs a)
{
    __shared__ dq s_q[RB];
    __shared__ d3 s_c[RB];
    __shared__ d3 s_dx[RB];
    __shared__ int s_mode[RB];  // 0 inactive, 1 active, 2 active + fly-away reset
    const int P = blockIdx.x * RB + threadIdx.x;
    const double dt = a.p.dt;
    int mode = 0;
    if (P < a.N && P >= a.p.n_min && P < a.p.n_max) {
        d3 vel12 = dld(a.v12 + 3 * P), om12bf = dld(a.w12bf + 3 * P), ombf = dld(a.wbf + 3 * P);
        d3 om = dld(a.w + 3 * P), c = dld(a.com + 3 * P);
        d3 f = dld(a.F + 3 * P), t = dld(a.T + 3 * P);
        const double m = a.mass[P];
        const double* Mi = a.Iinv + 9 * P;
        const double* Mm = a.I + 9 * P;
        dq qq = dqld(a.q + 4 * P), qh = dqld(a.q12 + 4 * P);
        d3 dxa = dld(a.dxall + 3 * P);

        d3 v32 = vel12 + ((f * 1) / m) * dt;
        dq qi = dqinv(qq);
        d3 tbf = dqtrip(qi, t, qq);
        d3 p1 = matvec(Mm, ombf);
        d3 p2 = tbf - dcross(ombf, p1);
        d3 alpha = matvec(Mi, p2);
        d3 om32bf = om12bf + alpha * dt;
        double wn = sqrt(om.x * om.x + om.y * om.y + om.z * om.z);
        d3 h = dm(0, 0, 0);
        if (wn != 0) h = (om / wn) * sin(wn * dt / 2);
        dq rq;
        rq.w = cos(wn * dt / 2);
        rq.x = h.x;
        rq.y = h.y;
        rq.z = h.z;
        dq q32 = dqmul(rq, qh);
        vel12 = v32;
        qh = q32;
        om12bf = om32bf;
        d3 dx = vel12 * dt;
        dxa = dxa + dx;
        d3 om34bf = om12bf + ((alpha * dt) * 1) / 4;
        d3 om34 = dqtrip(qh, om34bf, dqinv(qh));
        double wn34 = sqrt(om34.x * om34.x + om34.y * om34.y + om34.z * om34.z);
        d3 h2 = dm(0, 0, 0);
        if (wn34 != 0) h2 = (om34 / wn34) * sin(wn34 * dt / 4);
        dq rq2;
        rq2.w = cos(wn34 * dt / 4);
        rq2.x = h2.x;
        rq2.y = h2.y;
        rq2.z = h2.z;
        dq qold = qq;
        qq = dqmul(rq2, qh);
        dq qa = dqmul(qq, qold);
        ombf = om12bf + ((alpha * dt) * 1) / 2;
        om = dqtrip(qq, ombf, dqinv(qq));
        d3 vel = vel12 + (f * dt) / m;
        const d3 c_old = c;
        c = c + dx;
        mode = 1;
        const double* box = a.p.box;
        if (c.x > box[0] || c.x < box[1] || c.y > box[2] || c.y < box[3] || c.z > box[4] || c.z < box[5]) {
            mode = 2;
            vel = dm(0, 0, 0);
            vel12 = vel;
            om12bf = vel;
            ombf = vel;
            om = vel;
            c = c + dx * (-1);
            if (a.n_reset) atomicAdd(a.n_reset, 1);
        }
        dst(a.v + 3 * P, vel);
        dst(a.v12 + 3 * P, vel12);
        dst(a.w12bf + 3 * P, om12bf);
        dst(a.com + 3 * P, c);
        dst(a.dxall + 3 * P, dxa);
        dst(a.wbf + 3 * P, ombf);
        dst(a.w + 3 * P, om);
        dqst(a.q12 + 4 * P, qh);
        dqst(a.q + 4 * P, qq);
        dqst(a.qall + 4 * P, qa);
        s_q[threadIdx.x] = qq;
        s_c[threadIdx.x] = c_old;
        s_dx[threadIdx.x] = dx;
    }
    s_mode[threadIdx.x] = mode;
    __syncthreads();
    // vertices of this block's rows: rotate about the old centre, then translate (gpu_Verlet.cu:279-352)
    const int V = a.p.V;
    const int p0 = blockIdx.x * RB;
    const int rows = min(RB, a.N - p0);
    for (int j = threadIdx.x; j < rows * V; j += RB) {
        const int r = j / V;
        const int md = s_mode[r];
        if (!md) continue;
        double* vp = a.verts + ((size_t)(p0 + r) * V + (j - r * V)) * 3;
        const dq q = s_q[r];
        const d3 c = s_c[r], dx = s_dx[r];
        d3 v = dqtrip(q, dld(vp) - c, dqinv(q)) + c;
        v = v + dx;
        if (md == 2) v = v + dx * (-1);
        dst(vp, v);
    }
}

// ------------------------------------------------------------------ FP32 device-resident step

__device__ __forceinline__ float4 ld4(const float* p, int i) { return reinterpret_cast<const float4*>(p)[i]; }
__device__ __forceinline__ void st4(float* p, int i, float4 v) { reinterpret_cast<float4*>(p)[i] = v; }

struct alignas(32) dpos {
    double x, y, z, w;
};

// rotation increment [cos(|w| s), sin(|w| s) w/|w|]
__device__ __forceinline__ float4 rot_increment(f3 w, float s)
{
    float wn = sqrtf(w.x * w.x + w.y * w.y + w.z * w.z);
    float sn, cs;
    sincosf(wn * s, &sn, &cs);
    f3 h = mk3(0.f, 0.f, 0.f);
    if (wn != 0.f) h = (w / wn) * sn;
    return make_float4(cs, h.x, h.y, h.z);
}

// one row's update (walls: unchanged); returns the centre and q_acc the vertex pass uses
// MIRROR: every state array written here is also written `mirror` bytes further on, into a copy of the
// state block that lives in host memory the GPU can reach (the force/torque accumulators excepted)
template <bool MIRROR = false>
__device__ __forceinline__ void row_update(const mwd_state& st, const mwd_scene* __restrict__ scenes, int P,
                                           dpos& pos_out, float4& qacc_out, int64_t mirror = 0)
{
    const int info = st.info[P];
    dpos pos = reinterpret_cast<const dpos*>(st.pos)[P];
    float4 qacc = ld4(st.q_acc, P);
    if (!(info & (1 | MWD_INFO_INACTIVE))) {  // walls and rows waiting at an inlet stay as they are
        const mwd_scene& sc = scenes[info >> 1];
        const float dt = (float)sc.dt;
        float4 Fa = ld4(st.force, P), Ta = ld4(st.torque, P);
        float4 Fe = ld4(st.ext_force, P), Te = ld4(st.ext_torque, P);
        f3 F = mk3(Fa.x + Fe.x, Fa.y + Fe.y, Fa.z + Fe.z);
        f3 T = mk3(Ta.x + Te.x, Ta.y + Te.y, Ta.z + Te.z);
        float4 I = ld4(st.inertia, P), Ii = ld4(st.inv_inertia, P);
        const float invm = Ii.w;
        f3 vh = xyz(ld4(st.vel_half, P));
        f3 whbf = xyz(ld4(st.w_half_bf, P));
        f3 wbf = xyz(ld4(st.w_bf, P));
        f3 w = xyz(ld4(st.w, P));
        float4 q = ld4(st.q, P), qh = ld4(st.q_half, P), qall = ld4(st.q_all, P);
        dpos dxall = reinterpret_cast<const dpos*>(st.dx_all)[P];

        f3 v32 = vh + F * (invm * dt);
        f3 tbf = qtrip(qconj(q), T, q);
        f3 p1 = mk3(I.x * wbf.x, I.y * wbf.y, I.z * wbf.z);
        f3 p2 = tbf - cross(wbf, p1);
        f3 alpha = mk3(Ii.x * p2.x, Ii.y * p2.y, Ii.z * p2.z);
        f3 w32bf = whbf + alpha * dt;
        float4 q32 = qmul(rot_increment(w, dt * 0.5f), qh);
        vh = v32;
        qh = q32;
        whbf = w32bf;
        f3 dx = vh * dt;
        dxall.x += (double)dx.x;
        dxall.y += (double)dx.y;
        dxall.z += (double)dx.z;
        f3 w34bf = whbf + alpha * (dt * 0.25f);
        f3 w34 = qtrip(qh, w34bf, qconj(qh));
        float4 qold = q;
        q = qmul(rot_increment(w34, dt * 0.25f), qh);
        qall = qmul(q, qold);
        wbf = whbf + alpha * (dt * 0.5f);
        w = qtrip(q, wbf, qconj(q));
        f3 v = vh + F * (invm * dt);
        // vertices compound the rotation q every step (gpu_Verlet.cu:279-305): q_acc <- q q_acc;
        // under the physical law the vertices follow the orientation itself: q_acc <- q
        qacc = sc.mat[0].physical ? q : qmul(q, qacc);
        float qn = rsqrtf(qacc.x * qacc.x + qacc.y * qacc.y + qacc.z * qacc.z + qacc.w * qacc.w);
        qacc = make_float4(qacc.x * qn, qacc.y * qn, qacc.z * qn, qacc.w * qn);
        dpos np;
        np.x = pos.x + (double)dx.x;
        np.y = pos.y + (double)dx.y;
        np.z = pos.z + (double)dx.z;
        np.w = pos.w;
        if (np.x > sc.box[0] || np.x < sc.box[1] || np.y > sc.box[2] || np.y < sc.box[3] || np.z > sc.box[4] ||
            np.z < sc.box[5]) {
            // fly-away reset (gpu_Verlet.cu:338-352): stop the particle, undo the move
            v = vh = whbf = wbf = w = mk3(0.f, 0.f, 0.f);
            np = pos;
        }
        pos = np;
        auto putd = [&](double* a, const dpos& x) {
            reinterpret_cast<dpos*>(a)[P] = x;
            if (MIRROR) reinterpret_cast<dpos*>(reinterpret_cast<char*>(a) + mirror)[P] = x;
        };
        auto put4 = [&](float* a, float4 x) {
            st4(a, P, x);
            if (MIRROR) st4(reinterpret_cast<float*>(reinterpret_cast<char*>(a) + mirror), P, x);
        };
        putd(st.pos, pos);
        putd(st.dx_all, dxall);
        put4(st.vel, f4(v, 0.f));
        put4(st.vel_half, f4(vh, 0.f));
        put4(st.w_half_bf, f4(whbf, 0.f));
        put4(st.w_bf, f4(wbf, 0.f));
        put4(st.w, f4(w, 0.f));
        put4(st.q, q);
        put4(st.q_half, qh);
        put4(st.q_all, qall);
        put4(st.q_acc, qacc);
        st4(st.force, P, make_float4(0.f, 0.f, 0.f, 0.f));
        st4(st.torque, P, make_float4(0.f, 0.f, 0.f, 0.f));
    }
    pos_out = pos;
    qacc_out = qacc;
}

// R(q_acc) row-major and the centre as hi + lo floats per axis
__device__ __forceinline__ void row_xform(float4 qacc, dpos pos, float* R, float* c)
{
    const float qw = qacc.x, qx = qacc.y, qy = qacc.z, qz = qacc.w;
    R[0] = 1.f - 2.f * (qy * qy + qz * qz); R[1] = 2.f * (qx * qy - qw * qz); R[2] = 2.f * (qx * qz + qw * qy);
    R[3] = 2.f * (qx * qy + qw * qz); R[4] = 1.f - 2.f * (qx * qx + qz * qz); R[5] = 2.f * (qy * qz - qw * qx);
    R[6] = 2.f * (qx * qz - qw * qy); R[7] = 2.f * (qy * qz + qw * qx); R[8] = 1.f - 2.f * (qx * qx + qy * qy);
    const float hx = (float)pos.x, hy = (float)pos.y, hz = (float)pos.z;
    c[0] = hx; c[1] = (float)(pos.x - (double)hx);
    c[2] = hy; c[3] = (float)(pos.y - (double)hy);
    c[4] = hz; c[5] = (float)(pos.z - (double)hz);
}

__device__ __forceinline__ float4 world_vertex(const float* R, const float* c, float4 r0)
{
    const float rx = R[0] * r0.x + R[1] * r0.y + R[2] * r0.z;
    const float ry = R[3] * r0.x + R[4] * r0.y + R[5] * r0.z;
    const float rz = R[6] * r0.x + R[7] * r0.y + R[8] * r0.z;
    return make_float4(c[0] + (rx + c[1]), c[2] + (ry + c[3]), c[4] + (rz + c[5]), 0.f);
}

__global__ void __launch_bounds__(RB) integrate_kernel(mwd_state st, const mwd_scene* __restrict__ scenes,
                                                       uint32_t* status)
{
    pdl_wait();
    pdl_launch_dependents();
    __shared__ float s_R[RB][9];
    __shared__ float s_c[RB][6];  // centre split hi/lo per axis
    __shared__ int s_off[RB + 1];
    const int P = blockIdx.x * RB + threadIdx.x;
    const int p0 = blockIdx.x * RB;
    const int rows = min(RB, st.n - p0);
    if (P < st.n) {
        dpos pos;
        float4 qacc;
        row_update(st, scenes, P, pos, qacc);
        row_xform(qacc, pos, s_R[threadIdx.x], s_c[threadIdx.x]);
        s_off[threadIdx.x] = st.vert_off[P];
    }
    if (threadIdx.x == 0) s_off[rows] = st.vert_off[p0 + rows];
    __syncthreads();
    const int v0 = s_off[0], v1 = s_off[rows];
    const float4* bv = reinterpret_cast<const float4*>(st.body_verts);
    float4* wv = reinterpret_cast<float4*>(st.world_verts);
    constexpr int U = 4;  // vertices in flight per thread: loads first, then the stores
    for (int j0 = v0 + threadIdx.x; j0 < v1; j0 += U * RB) {
        float4 r0[U];
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const int j = j0 + k * RB;
            r0[k] = j < v1 ? __ldg(bv + j) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const int j = j0 + k * RB;
            if (j >= v1) break;
            // owner row: last r with s_off[r] <= j
            int lo = 0, hi = rows - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (s_off[mid] <= j) lo = mid; else hi = mid - 1;
            }
            wv[j] = world_vertex(s_R[lo], s_c[lo], r0[k]);
        }
    }
}

// the row pass of the split integrator: one thread per row, the transform to st.xform (MIRROR: the
// state also written into its copy in GPU-reachable host memory, `mirror` bytes further on)
template <bool MIRROR>
__global__ void __launch_bounds__(RB) integrate_rows_kernel(mwd_state st, const mwd_scene* __restrict__ scenes,
                                                            uint32_t* status, int64_t mirror)
{
    pdl_wait();
    pdl_launch_dependents();
    const int P = blockIdx.x * RB + threadIdx.x;
    if (P >= st.n) return;
    dpos pos;
    float4 qacc;
    row_update<MIRROR>(st, scenes, P, pos, qacc, mirror);
    float x[16];
    row_xform(qacc, pos, x, x + 9);
    x[15] = 0.f;
    float4* o = reinterpret_cast<float4*>(st.xform) + 4 * (size_t)P;
    o[0] = make_float4(x[0], x[1], x[2], x[3]);
    o[1] = make_float4(x[4], x[5], x[6], x[7]);
    o[2] = make_float4(x[8], x[9], x[10], x[11]);
    o[3] = make_float4(x[12], x[13], x[14], x[15]);
}

// the row transforms alone, from the current centres and orientations (no integration)
__global__ void __launch_bounds__(RB) xform_rows_kernel(mwd_state st)
{
    pdl_wait();
    pdl_launch_dependents();
    const int P = blockIdx.x * RB + threadIdx.x;
    if (P >= st.n) return;
    const dpos pos = reinterpret_cast<const dpos*>(st.pos)[P];
    float x[16];
    row_xform(ld4(st.q_acc, P), pos, x, x + 9);
    x[15] = 0.f;
    float4* o = reinterpret_cast<float4*>(st.xform) + 4 * (size_t)P;
    o[0] = make_float4(x[0], x[1], x[2], x[3]);
    o[1] = make_float4(x[4], x[5], x[6], x[7]);
    o[2] = make_float4(x[8], x[9], x[10], x[11]);
    o[3] = make_float4(x[12], x[13], x[14], x[15]);
}

// the vertex pass of the split integrator: one thread per vertex
__global__ void __launch_bounds__(256) world_verts_kernel(mwd_state st)
{
    pdl_wait();
    pdl_launch_dependents();
    const int j = blockIdx.x * 256 + threadIdx.x;
    if (j >= st.n_verts) return;
    const int o = st.vert_owner[j];
    const float4* xf = reinterpret_cast<const float4*>(st.xform) + 4 * (size_t)o;
    const float4 a = xf[0], b = xf[1], c = xf[2], d = xf[3];
    const float R[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
    const float cc[6] = {c.y, c.z, c.w, d.x, d.y, d.z};
    const float4 r0 = __ldg(reinterpret_cast<const float4*>(st.body_verts) + j);
    reinterpret_cast<float4*>(st.world_verts)[j] = world_vertex(R, cc, r0);
}
}  // namespace

int launch_verlet_ref(const VerletRefArgs& a, cudaStream_t s)
{
    if (a.N <= 0) return MWD_OK;
    verlet_ref_kernel<<<(a.N + RB - 1) / RB, RB, 0, s>>>(a);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

int launch_world_verts(const mwd_state& st, cudaStream_t s)
{
    if (st.n_verts <= 0) return MWD_OK;
    MWD_CUDA(launch_pdl(world_verts_kernel, (st.n_verts + 255) / 256, 256, 0, s, st));
    return MWD_OK;
}

int launch_refresh_vertices(const mwd_state& st, cudaStream_t s)
{
    if (st.n <= 0) return MWD_OK;
    MWD_CUDA(launch_pdl(xform_rows_kernel, (st.n + RB - 1) / RB, RB, 0, s, st));
    return launch_world_verts(st, s);
}

int launch_integrate_rows_mirror(const mwd_state& st, const mwd_scene* scenes, uint32_t* status, int64_t mirror,
                                 cudaStream_t s)
{
    if (st.n <= 0) return MWD_OK;
    MWD_CUDA(launch_pdl(integrate_rows_kernel<true>, (st.n + RB - 1) / RB, RB, 0, s, st, scenes, status, mirror));
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

// Rows and vertices in one kernel (integrate_kernel: each block's rows, then their vertices) once its
// grid spans at least two full waves of the GPU; below that the row pass and the one-thread-per-vertex
// pass spread the vertex work better.  On 256 batched scenes (2.0M rows) one kernel per step measured
// 0.676 ms per step against 0.699 ms for the two passes with the vertex pass overlapped with the next
// step's broad phase: it moves neither the row transforms nor the vertex owners through memory.
bool integrate_in_one_kernel(int64_t n)
{
    static LaunchSetup setup;
    int per_sm = 0;
    if (launch_setup(setup, integrate_kernel, RB, 0, 0, &per_sm) != MWD_OK || per_sm <= 0) return false;
    return (n + RB - 1) / RB >= 2 * (int64_t)num_sms() * per_sm;
}

int launch_integrate(const mwd_state& st, const mwd_scene* scenes, uint32_t* status, cudaStream_t s,
                     bool with_verts)
{
    if (st.n <= 0) return MWD_OK;
    if (st.vert_owner && st.xform && !(with_verts && integrate_in_one_kernel(st.n))) {
        MWD_CUDA(launch_pdl(integrate_rows_kernel<false>, (st.n + RB - 1) / RB, RB, 0, s, st, scenes, status,
                            (int64_t)0));
        if (with_verts && st.n_verts > 0)
            MWD_CUDA(launch_pdl(world_verts_kernel, (st.n_verts + 255) / 256, 256, 0, s, st));
    } else {
        MWD_CUDA(launch_pdl(integrate_kernel, (st.n + RB - 1) / RB, RB, 0, s, st, scenes, status));
    }
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

}  // namespace mwd
