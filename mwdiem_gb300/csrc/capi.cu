// extern "C" entry points of libmwdem.so (declared in include/mwdem.h).
//
// Host-side responsibilities: argument checks, the per-device scratch the reference-layout entry
// points need, the pair-independent contact-law constants, and error strings.  No entry point
// synchronises the device except mwd_linked_cell_hash, which must read the key range before it
// can size its cell table.
#include <math.h>
#include <stdlib.h>
#include <stdarg.h>
#include <stdio.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "broad.cuh"
#include "common.cuh"
#include "integrate.cuh"
#include "reduce.cuh"
#include "narrow.cuh"

namespace mwd {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_check(cudaError_t e, const char* what)
{
    set_error("%s: %s", what, cudaGetErrorString(e));
    return MWD_ERR_CUDA;
}

int num_sms()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (!v) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        v = n > 0 ? n : 152;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

namespace {

// Library-owned scratch of the reference-layout entry points: one grow-only buffer per device.
// Calls that use it must not overlap on the GPU (the reference itself is single-stream).
struct ScratchBuf {
    void* p = nullptr;
    size_t bytes = 0;
};
std::mutex g_scratch_mu;
ScratchBuf g_scratch[64];

int scratch(size_t bytes, void** out)
{
    int dev = 0;
    MWD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return MWD_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    ScratchBuf& b = g_scratch[dev];
    if (b.bytes < bytes) {
        if (b.p) {
            // cudaFree waits for work already queued that may still use the old buffer
            MWD_CUDA(cudaFree(b.p));
            b.p = nullptr;
            b.bytes = 0;
        }
        size_t want = bytes + bytes / 2 + 4096;
        if (cudaMalloc(&b.p, want) != cudaSuccess) {
            cudaGetLastError();
            set_error("cudaMalloc of %zu bytes of scratch failed", want);
            return MWD_ERR_NOMEM;
        }
        b.bytes = want;
    }
    *out = b.p;
    return MWD_OK;
}

// carve aligned sub-buffers out of one allocation
int check_lanes(int lanes, int* out)
{
    if (lanes == 0) lanes = 8;
    if (lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32) {
        set_error("lanes per pair must be 4, 8, 16 or 32 (got %d)", lanes);
        return MWD_ERR_INVALID;
    }
    *out = lanes;
    return MWD_OK;
}

}  // namespace

// Pair-independent constants, with the reference's operand types (gpu_fine_contact_detection.cu:685-701):
// log of a float argument in float, pi^2 + ln^2 in float, the products with the double literals
// mu and Kn in double.  Evaluated on the host with the C library's logf, like the oracle.
static void derive_one(double Kn, double en, double et, double mu, double dt, int32_t law, mwd_material* m)
{
    const float pii = (float)3.141592653589793;
    const float Len = logf((float)en), Let = logf((float)et);
    const float Xen = pii * pii + Len * Len;
    const float Xet = pii * pii + Let * Let;
    const float tc = (float)sqrt(mu * (double)Xen / Kn);
    m->Kn_f = (float)Kn;
    m->mu_f = (float)mu;
    m->Gn = (float)((-1) * 2 * mu / (double)tc * (double)Len);
    m->ln_et = Let;
    m->dt_f = (float)dt;
    m->ln_en = Len;
    m->Xn = Xen;
    m->Xt = Xet;
    m->mu = mu;
    m->inv_mu = 1 / mu;
    m->KtA = Kn * (double)Xet / (double)Xen;
    m->physical = law == MWD_LAW_PHYSICAL ? 1 : 0;
    m->inv_mu_hi = (float)m->inv_mu;
    m->inv_mu_lo = (float)(m->inv_mu - (double)m->inv_mu_hi);
    m->KtA_hi = (float)m->KtA;
    m->KtA_lo = (float)(m->KtA - (double)m->KtA_hi);
    m->pad = 0;
}

}  // namespace mwd

thread_local int mwd::g_launch_priority = 0;

namespace {

// The second stream and the two events of the overlapped multi-step mwd_step, one set per device and
// calling thread (so that calls from several threads never re-record each other's events).  They are
// created outside any stream capture: by the thread's first mwd_step call that could overlap (a
// one-step call included, such as the warm-up step before a graph capture); a call that finds none
// while its stream is being captured steps without the overlap.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    int prio_high = 0;
};
// Destroys a thread's streams and events when the thread exits (a pool of short-lived host threads
// would otherwise leave one stream and two events per thread and device behind).  At process exit
// the runtime may already be unloaded; the calls then fail harmlessly and their errors are cleared.
struct SideStreams {
    SideStream dev[64];
    ~SideStreams()
    {
        int cur = -1;
        if (cudaGetDevice(&cur) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        for (int d = 0; d < 64; ++d) {
            SideStream& ss = dev[d];
            if (!ss.s) continue;
            if (cudaSetDevice(d) == cudaSuccess) {
                cudaEventDestroy(ss.fork);
                cudaEventDestroy(ss.join);
                cudaStreamDestroy(ss.s);
            }
            ss = SideStream();
        }
        cudaSetDevice(cur);
        cudaGetLastError();
    }
};
thread_local SideStreams g_side;

const SideStream* side_stream(cudaStream_t main)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    SideStream& ss = g_side.dev[dev];
    if (ss.s) return &ss;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(main, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return nullptr;
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, least) != cudaSuccess) return nullptr;
    if (cudaEventCreateWithFlags(&a, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b, cudaEventDisableTiming) != cudaSuccess) {
        if (a) cudaEventDestroy(a);
        cudaStreamDestroy(st);
        return nullptr;
    }
    ss.fork = a;
    ss.join = b;
    ss.prio_high = greatest;
    ss.s = st;
    return &ss;
}

// MWD_OVERLAP=0 in the environment: multi-step calls run the plain loop
bool overlap_enabled()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("MWD_OVERLAP");
        v = (e && e[0] == '0') ? 0 : 1;
    }
    return v == 1;
}

}  // namespace

bool mwd::pdl_enabled()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("MWD_PDL");
        v = (e && e[0] == '0') ? 0 : 1;
    }
    return v == 1;
}

using namespace mwd;

extern "C" {

const char* mwd_last_error(void) { return g_err; }
int mwd_version(void) { return 1; }
int32_t mwd_num_sms(void) { return num_sms(); }
int64_t mwd_scan_tmp_ints(int64_t n) { return scan_tmp_ints(n); }

int32_t mwd_integrate_kernels(int64_t n) { return integrate_in_one_kernel(n) ? 1 : 2; }

int32_t mwd_cell_table(int64_t n, int64_t total_cells, int32_t mode)
{
    const int64_t m = (total_cells > n ? total_cells : n) + 1;
    return broad_sparse(n, total_cells, scan_tmp_ints(m) - scan_tile_sums_offset(m), mode) ? 2 : 1;
}

int32_t mwd_cell_table_ints(int64_t n, int64_t total_cells, int32_t mode, int64_t* count_ints, int64_t* start_ints)
{
    const int32_t kind = mwd_cell_table(n, total_cells, mode);
    int64_t c = 0, st = 0;
    broad_table_ints(n, total_cells, kind == 2 ? 1 : 0, &c, &st);
    if (count_ints) *count_ints = c;
    if (start_ints) *start_ints = st;
    return kind;
}
int64_t mwd_det_scratch_bytes(int32_t n, int64_t epa_cap)
{
    return n < 0 || epa_cap < 0 ? -1 : (int64_t)det_scratch_bytes(n, epa_cap);
}

int mwd_derive_material(const mwd_contact_params* prm, mwd_material m[2])
{
    if (!prm || !m) {
        set_error("mwd_derive_material: null argument");
        return MWD_ERR_INVALID;
    }
    if (prm->law != MWD_LAW_REFERENCE && prm->law != MWD_LAW_PHYSICAL) {
        set_error("mwd_derive_material: unknown contact law %d", prm->law);
        return MWD_ERR_INVALID;
    }
    derive_one(prm->Kn, prm->en, prm->et, prm->mu, prm->dt, prm->law, &m[0]);
    derive_one(prm->Kn_wall, prm->en_wall, prm->et_wall, prm->mu_wall, prm->dt, prm->law, &m[1]);
    return MWD_OK;
}

int mwd_contact_pairs(int64_t n_pairs, int32_t V, int32_t n_particles, const float* A_com, const float* B_com,
                      const float* A_verts, const float* B_verts, const float* A_vel, const float* B_vel,
                      const float* A_angvel, const float* B_angvel, const int32_t* A_nv, const int32_t* B_nv,
                      const int32_t* A_id, const int32_t* B_id, float* hist, float* force, float* torque,
                      const float* qA, const float* qB, const float* IsA, const float* IsB, int32_t* collision,
                      const mwd_contact_params* prm, float* diag, uint32_t* status, mwd_stream_t stream)
{
    if (!prm || n_pairs < 0 || n_particles < 0) {
        set_error("mwd_contact_pairs: bad arguments");
        return MWD_ERR_INVALID;
    }
    if (n_pairs == 0) return MWD_OK;
    if (!A_com || !B_com || !A_verts || !B_verts || !A_vel || !B_vel || !A_angvel || !B_angvel || !A_nv || !B_nv ||
        !A_id || !B_id || !hist || !force || !torque || !qA || !qB || !IsA || !IsB || !collision) {
        set_error("mwd_contact_pairs: null array");
        return MWD_ERR_INVALID;
    }
    if (V < 1 || V > MWD_HULL_CAP) {
        set_error("num_vertices_max %d outside 1..%d", V, MWD_HULL_CAP);
        return MWD_ERR_UNSUPPORTED;
    }
    if (prm->deterministic) {
        set_error("deterministic accumulation is not available for the per-pair layout");
        return MWD_ERR_UNSUPPORTED;
    }
    if (prm->law != MWD_LAW_REFERENCE) {
        set_error("the per-pair layout carries no masses: only the reference contact law is available");
        return MWD_ERR_UNSUPPORTED;
    }
    int lanes;
    int rc = check_lanes(prm->lanes, &lanes);
    if (rc) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    NarrowArgs a = {};
    a.A_com = A_com; a.B_com = B_com; a.A_verts = A_verts; a.B_verts = B_verts;
    a.A_vel = A_vel; a.B_vel = B_vel; a.A_w = A_angvel; a.B_w = B_angvel;
    a.qA = qA; a.qB = qB; a.IsA = IsA; a.IsB = IsB;
    a.A_nv = A_nv; a.B_nv = B_nv; a.A_id = A_id; a.B_id = B_id;
    a.hist_in = hist;
    a.hist_out = hist;
    a.force = force;
    a.torque = torque;
    a.V = V;
    a.n_wall = prm->n_wall;
    a.hist_mode = prm->hist_mode ? 1 : 0;
    a.n_pairs = n_pairs;
    mwd_derive_material(prm, a.mat);
    a.collision = collision;
    a.diag = diag;
    a.status = status;
    a.hull_cap = V;
    if (!a.hist_mode) {
        Carver c;
        size_t o_stage = c.take<float4>(n_pairs);
        size_t o_wrote = c.take<uint8_t>(n_pairs);
        void* base;
        rc = scratch(c.off, &base);
        if (rc) return rc;
        a.hist_stage = reinterpret_cast<float*>((char*)base + o_stage);
        a.hist_wrote = reinterpret_cast<uint8_t*>((char*)base + o_wrote);
        MWD_CUDA(cudaMemsetAsync(a.hist_wrote, 0, n_pairs, s));
    }
    rc = launch_narrow(a, 0, lanes, n_pairs, s);
    if (rc) return rc;
    if (!a.hist_mode) return launch_hist_resolve(hist, a.hist_stage, a.hist_wrote, n_pairs, s);
    return MWD_OK;
}

int mwd_verlet_ref(int32_t N, double* v, double* v12, double* w12bf, double* q12, double* q, double* qall,
                   double* wbf, double* w, const double* F, const double* T, double* verts, double* com,
                   const double* mass, const double* Iinv, const double* I, double* dxall,
                   const mwd_verlet_params* prm, int32_t* n_reset, mwd_stream_t stream)
{
    if (!prm || N < 0 || prm->V < 0) {
        set_error("mwd_verlet_ref: bad arguments");
        return MWD_ERR_INVALID;
    }
    if (N == 0) return MWD_OK;
    if (!v || !v12 || !w12bf || !q12 || !q || !qall || !wbf || !w || !F || !T || (!verts && prm->V) || !com ||
        !mass || !Iinv || !I || !dxall) {
        set_error("mwd_verlet_ref: null array");
        return MWD_ERR_INVALID;
    }
    VerletRefArgs a;
    a.N = N;
    a.v = v; a.v12 = v12; a.w12bf = w12bf; a.q12 = q12; a.q = q; a.qall = qall; a.wbf = wbf; a.w = w;
    a.F = F; a.T = T; a.verts = verts; a.com = com; a.mass = mass; a.Iinv = Iinv; a.I = I; a.dxall = dxall;
    a.n_reset = n_reset;
    a.p = *prm;
    return launch_verlet_ref(a, reinterpret_cast<cudaStream_t>(stream));
}

int mwd_cell_keys(int32_t N, const double* com, double csx, double csy, double csz, int64_t nx, int64_t ny,
                  int64_t* keys, mwd_stream_t stream)
{
    if (N < 0 || (N && (!com || !keys))) {
        set_error("mwd_cell_keys: bad arguments");
        return MWD_ERR_INVALID;
    }
    return launch_keys(N, com, csx, csy, csz, nx, ny, keys, reinterpret_cast<cudaStream_t>(stream));
}

int mwd_wall_pairs(int32_t n_wall, int32_t n_lo, int32_t n_hi, const double* com, const double* wall_normal,
                   const double* wall_center, double range, int32_t* pairs, int64_t cap, int64_t* n_out,
                   uint32_t* status, mwd_stream_t stream)
{
    if (n_wall < 0 || n_hi < n_lo || !n_out || (cap > 0 && !pairs)) {
        set_error("mwd_wall_pairs: bad arguments");
        return MWD_ERR_INVALID;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t total = (int64_t)n_wall * (n_hi - n_lo);
    if (total > INT32_MAX / 2) {
        set_error("mwd_wall_pairs: %lld tests exceed the 32-bit scan", (long long)total);
        return MWD_ERR_UNSUPPORTED;
    }
    Carver c;
    size_t o_flags = c.take<int32_t>(total + 1);
    size_t o_offs = c.take<int32_t>(total + 1);
    size_t o_tmp = c.take<int32_t>(scan_tmp_ints(total));
    void* base;
    int rc = scratch(c.off, &base);
    if (rc) return rc;
    return launch_wall_pairs(n_wall, n_lo, n_hi, com, wall_normal, wall_center, range,
                             reinterpret_cast<int32_t*>((char*)base + o_flags),
                             reinterpret_cast<int32_t*>((char*)base + o_offs),
                             reinterpret_cast<int32_t*>((char*)base + o_tmp), pairs, cap, n_out, status, s);
}

int mwd_linked_cell_hash(int32_t n_lo, int32_t n_hi, const int64_t* keys, int64_t nx, int64_t ny, int32_t* pairs,
                         int64_t cap, int64_t* n_out, uint32_t* status, mwd_stream_t stream)
{
    if (n_lo < 0 || n_hi < n_lo || !n_out || (n_hi > n_lo && !keys) || (cap > 0 && !pairs)) {
        set_error("mwd_linked_cell_hash: bad arguments");
        return MWD_ERR_INVALID;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n_hi == n_lo) {
        MWD_CUDA(cudaMemsetAsync(n_out, 0, sizeof(int64_t), s));
        return MWD_OK;
    }
    // key range (one host synchronisation)
    void* base;
    int rc = scratch(4096, &base);
    if (rc) return rc;
    unsigned long long init[2] = {~0ull, 0ull}, mm[2];
    MWD_CUDA(cudaMemcpyAsync(base, init, sizeof(init), cudaMemcpyHostToDevice, s));
    rc = launch_minmax(keys, n_lo, n_hi, reinterpret_cast<unsigned long long*>(base), s);
    if (rc) return rc;
    MWD_CUDA(cudaMemcpyAsync(mm, base, sizeof(mm), cudaMemcpyDeviceToHost, s));
    MWD_CUDA(cudaStreamSynchronize(s));
    const int64_t kmin = (int64_t)(mm[0] ^ 0x8000000000000000ull);
    const int64_t kmax = (int64_t)(mm[1] ^ 0x8000000000000000ull);
    const int64_t R = kmax - kmin + 1;
    const int64_t rows = n_hi - n_lo;
    const int64_t m = (R > rows ? R : rows) + 1;
    // a dense cell table up to 2^28 cells; beyond, the compressed one (a bit per cell, a count and a
    // start per row), which a sparse key range of up to 2^31 cells fits
    int sparse = 0;
    if (R > (int64_t)1 << 28)
        sparse = R <= INT32_MAX - 64 ? broad_sparse(rows, R, scan_tmp_ints(m) - scan_tile_sums_offset(m), 2) : 0;
    if (R <= 0 || (R > (int64_t)1 << 28 && !sparse)) {
        set_error("cell key range %lld is too wide for the cell tables", (long long)R);
        return MWD_ERR_UNSUPPORTED;
    }
    int64_t count_ints = 0, start_ints = 0;
    broad_table_ints(rows, R, sparse, &count_ints, &start_ints);
    Carver c;
    size_t o_scene = c.take<mwd_scene>(1);
    size_t o_count = c.take<int32_t>(count_ints);
    size_t o_start = c.take<int32_t>(start_ints);
    size_t o_cellof = c.take<int32_t>(n_hi);
    size_t o_scat = c.take<int32_t>(n_hi);
    size_t o_sorted = c.take<int32_t>(n_hi);
    size_t o_pc = c.take<int32_t>(rows + 1);
    size_t o_tmp = c.take<int32_t>(scan_tmp_ints(m));
    rc = scratch(c.off, &base);
    if (rc) return rc;
    char* b = (char*)base;
    mwd_scene sc = {};
    sc.nx = nx;
    sc.ny = ny;
    sc.key_min = kmin;
    sc.n_keys = R;
    sc.cell_base = 0;
    MWD_CUDA(cudaMemcpyAsync(b + o_scene, &sc, sizeof(sc), cudaMemcpyHostToDevice, s));
    MWD_CUDA(cudaMemsetAsync(b + o_count, 0, count_ints * sizeof(int32_t), s));
    int32_t* tile_sums = nullptr;
    if (sparse) {  // the compressed table's per-tile counts, zero on entry
        tile_sums = reinterpret_cast<int32_t*>(b + o_tmp) + scan_tile_sums_offset(m);
        MWD_CUDA(cudaMemsetAsync(tile_sums, 0, (scan_tmp_ints(m) - scan_tile_sums_offset(m)) * sizeof(int32_t), s));
    }
    BroadArgs a = {};
    a.row_lo = n_lo;
    a.row_hi = n_hi;
    a.keys = keys;
    a.scenes = reinterpret_cast<const mwd_scene*>(b + o_scene);
    a.walls = 0;
    a.cell_count = reinterpret_cast<int32_t*>(b + o_count);
    a.cell_start = reinterpret_cast<int32_t*>(b + o_start);
    a.cell_of = reinterpret_cast<int32_t*>(b + o_cellof);
    a.scatter_out = reinterpret_cast<int32_t*>(b + o_scat);
    a.sorted = reinterpret_cast<int32_t*>(b + o_sorted);
    a.pair_count = reinterpret_cast<int32_t*>(b + o_pc);
    a.scan_tmp = reinterpret_cast<int32_t*>(b + o_tmp);
    a.pairs = pairs;
    a.n_pairs = n_out;
    a.status = status;
    a.total_cells = R;
    a.pair_cap = cap;
    a.tile_sums = tile_sums;
    a.sparse = sparse;
    rc = launch_broad(a, s);
    if (rc) return rc;
    // the host copy of the scene must outlive the async copy
    MWD_CUDA(cudaStreamSynchronize(s));
    return MWD_OK;
}

int mwd_broadphase(const mwd_state* st, const mwd_scene* scenes_dev, const mwd_scene* scenes_host, int32_t n_scenes,
                   mwd_work* work, mwd_stream_t stream)
{
    if (!st || !scenes_dev || !work || n_scenes < 1) {
        set_error("mwd_broadphase: bad arguments");
        return MWD_ERR_INVALID;
    }
    (void)scenes_host;
    BroadArgs a = {};
    a.row_lo = 0;
    a.row_hi = st->n;
    a.keys = nullptr;
    a.pos = st->pos;
    a.wall_normal = st->wall_normal;
    a.info = st->info;
    a.scenes = scenes_dev;
    a.walls = 1;
    a.cell_count = work->cell_count;
    a.cell_start = work->cell_start;
    a.cell_of = work->cell_of;
    a.scatter_out = work->pair_count;  // free until the count pass
    a.sorted = work->sorted;
    a.pair_count = work->pair_count;
    a.scan_tmp = work->scan_tmp;
    a.pairs = work->pairs;
    a.n_pairs = work->n_pairs;
    a.status = work->status;
    a.total_cells = work->total_cells;
    a.pair_cap = work->pair_cap;
    a.cull = work->cull_pairs ? 1 : 0;
    a.append = work->deterministic ? 0 : 1;  // deterministic: the list in cell order
    a.epa_count = work->epa_rec ? work->epa_count : nullptr;
    a.sorted_pos = reinterpret_cast<float4*>(work->sorted_pos);
    a.sorted_cell = work->sorted_cell;
    // scan_tmp holds mwd_scan_tmp_ints(max(total_cells, n) + 1) ints: its second half keeps the
    // per-tile cell counts the assign pass adds up (zero on entry and on exit)
    {
        const int64_t rows = (int64_t)st->n;
        const int64_t m = (work->total_cells > rows ? work->total_cells : rows) + 1;
        a.tile_sums = work->scan_tmp + scan_tile_sums_offset(m);
        a.sparse = broad_sparse(rows, work->total_cells, scan_tmp_ints(m) - scan_tile_sums_offset(m),
                                work->cell_table);
    }
    return launch_broad(a, reinterpret_cast<cudaStream_t>(stream));
}

static int narrow_force(const mwd_state* st, const mwd_scene* scenes_dev, mwd_work* work, int32_t lanes,
                        mwd_stream_t stream, bool epa_zeroed);

int mwd_narrow_force(const mwd_state* st, const mwd_scene* scenes_dev, mwd_work* work, int32_t lanes,
                     mwd_stream_t stream)
{
    return narrow_force(st, scenes_dev, work, lanes, stream, false);
}

static int narrow_force(const mwd_state* st, const mwd_scene* scenes_dev, mwd_work* work, int32_t lanes,
                        mwd_stream_t stream, bool epa_zeroed)
{
    if (!st || !scenes_dev || !work) {
        set_error("mwd_narrow_force: bad arguments");
        return MWD_ERR_INVALID;
    }
    if (st->max_verts < 1 || st->max_verts > MWD_HULL_CAP) {
        set_error("max_verts %d outside 1..%d", st->max_verts, MWD_HULL_CAP);
        return MWD_ERR_UNSUPPORTED;
    }
    int lp;
    // the GJK pass of the two-pass narrow phase also runs one lane per pair
    const bool gjk_one = (lanes & 0xff) == 1 && work->epa_rec;
    int rc = gjk_one ? MWD_OK : check_lanes(lanes & 0xff, &lp);
    if (rc) return rc;
    if (gjk_one) lp = 1;
    const int elp = (lanes >> 8) & 0xff;
    NarrowArgs a = {};
    a.epa_global = (lanes >> 16) & 1;
    a.st = *st;
    a.scenes = scenes_dev;
    a.pairs = work->pairs;
    a.n_pairs_dev = work->n_pairs;
    a.pair_cap = work->pair_cap;
    a.collision = work->collision;
    a.status = work->status;
    a.work_counters = reinterpret_cast<unsigned long long*>(work->work_counters);
    a.hull_cap = st->max_verts;
    a.face_ids = work->face_ids;
    if (work->epa_rec && work->epa_count && work->epa_cap > 0) {
        a.epa_count = work->epa_count;
        a.epa_rec = work->epa_rec;
        a.epa_cap = work->epa_cap;
        a.pre_culled = work->cull_pairs ? 1 : 0;
        a.epa_zeroed = epa_zeroed ? 1 : 0;
        if (work->hist_keys) {
            if (!work->hist_vals || !work->hist_parity || work->hist_cap < 2 ||
                (work->hist_cap & (work->hist_cap - 1))) {
                set_error("persistent history needs hist_vals, hist_parity and a power-of-two hist_cap");
                return MWD_ERR_INVALID;
            }
            a.hist_keys = work->hist_keys;
            a.hist_vals = reinterpret_cast<float4*>(work->hist_vals);
            a.hist_cap = work->hist_cap;
            a.hist_parity = work->hist_parity;
        }
        if (work->deterministic) {
            if (!work->det_scratch) {
                set_error("deterministic accumulation needs work->det_scratch");
                return MWD_ERR_INVALID;
            }
            DetArgs d = det_carve(work->det_scratch, st->n, work->epa_cap);
            d.pairs = work->pairs;
            d.recs = reinterpret_cast<const SimplexRec*>(work->epa_rec);
            d.epa_count = work->epa_count;
            d.info = st->info;
            d.force = st->force;
            d.torque = st->torque;
            a.det_out = d.out;
            rc = launch_narrow_two_pass(a, lp | (elp << 8), reinterpret_cast<cudaStream_t>(stream));
            if (rc) return rc;
            return launch_det_reduce(d, reinterpret_cast<cudaStream_t>(stream));
        }
        return launch_narrow_two_pass(a, lp | (elp << 8), reinterpret_cast<cudaStream_t>(stream));
    }
    if (work->deterministic || work->hist_keys) {
        set_error("deterministic accumulation and persistent history need the two-pass narrow phase (work->epa_rec)");
        return MWD_ERR_UNSUPPORTED;
    }
    return launch_narrow(a, 1, lp, -1, reinterpret_cast<cudaStream_t>(stream));
}

int mwd_integrate(mwd_state* st, const mwd_scene* scenes_dev, uint32_t* status, mwd_stream_t stream)
{
    if (!st || !scenes_dev) {
        set_error("mwd_integrate: bad arguments");
        return MWD_ERR_INVALID;
    }
    return launch_integrate(*st, scenes_dev, status, reinterpret_cast<cudaStream_t>(stream));
}

int mwd_integrate_rows(mwd_state* st, const mwd_scene* scenes_dev, uint32_t* status, mwd_stream_t stream)
{
    if (!st || !scenes_dev || !st->vert_owner || !st->xform) {
        set_error("mwd_integrate_rows: needs scenes and a state with vert_owner and xform");
        return MWD_ERR_INVALID;
    }
    return launch_integrate(*st, scenes_dev, status, reinterpret_cast<cudaStream_t>(stream), false);
}

int mwd_integrate_rows_mirror(mwd_state* st, const mwd_scene* scenes_dev, uint32_t* status, void* mirror,
                              const void* block, int64_t block_bytes, mwd_stream_t stream)
{
    if (!st || !scenes_dev || !st->vert_owner || !st->xform || !mirror || !block || block_bytes <= 0) {
        set_error("mwd_integrate_rows_mirror: needs scenes, a state with vert_owner and xform, a mirror and its block");
        return MWD_ERR_INVALID;
    }
    // every array the row pass writes (the force/torque accumulators aside) must lie in the block
    const char* b0 = static_cast<const char*>(block);
    const char* b1 = b0 + block_bytes;
    const int64_t n = st->n;
    const struct {
        const void* p;
        int64_t bytes;
    } arrays[] = {{st->pos, 32 * n},      {st->dx_all, 32 * n}, {st->vel, 16 * n},    {st->vel_half, 16 * n},
                  {st->w_half_bf, 16 * n}, {st->w_bf, 16 * n},   {st->w, 16 * n},      {st->q, 16 * n},
                  {st->q_half, 16 * n},    {st->q_all, 16 * n},  {st->q_acc, 16 * n}};
    for (const auto& a : arrays) {
        const char* p = static_cast<const char*>(a.p);
        if (!p || p < b0 || p + a.bytes > b1) {
            set_error("mwd_integrate_rows_mirror: a state array lies outside the mirrored block");
            return MWD_ERR_INVALID;
        }
    }
    if ((reinterpret_cast<uintptr_t>(mirror) - reinterpret_cast<uintptr_t>(block)) & 31) {
        set_error("mwd_integrate_rows_mirror: the mirror must have the block's alignment modulo 32 bytes");
        return MWD_ERR_INVALID;
    }
    const int64_t delta = static_cast<const char*>(mirror) - b0;
    return launch_integrate_rows_mirror(*st, scenes_dev, status, delta, reinterpret_cast<cudaStream_t>(stream));
}

int mwd_host_mapped(const void* host, void** device_address)
{
    if (!host || !device_address) {
        set_error("mwd_host_mapped: null argument");
        return MWD_ERR_INVALID;
    }
    void* d = nullptr;
    cudaError_t e = cudaHostGetDevicePointer(&d, const_cast<void*>(host), 0);
    if (e != cudaSuccess || !d) {
        cudaGetLastError();
        set_error("mwd_host_mapped: not page-locked host memory mapped for the device (%s)", cudaGetErrorString(e));
        return MWD_ERR_INVALID;
    }
    *device_address = d;
    return MWD_OK;
}

int mwd_world_vertices(mwd_state* st, mwd_stream_t stream)
{
    if (!st || !st->vert_owner || !st->xform) {
        set_error("mwd_world_vertices: needs a state with vert_owner and xform");
        return MWD_ERR_INVALID;
    }
    return launch_world_verts(*st, reinterpret_cast<cudaStream_t>(stream));
}

int mwd_refresh_vertices(mwd_state* st, mwd_stream_t stream)
{
    if (!st || !st->vert_owner || !st->xform) {
        set_error("mwd_refresh_vertices: needs a state with vert_owner and xform");
        return MWD_ERR_INVALID;
    }
    return launch_refresh_vertices(*st, reinterpret_cast<cudaStream_t>(stream));
}

int mwd_step(mwd_state* st, const mwd_scene* scenes_dev, const mwd_scene* scenes_host, int32_t n_scenes, mwd_work* work,
             int32_t lanes, int32_t n_steps, mwd_stream_t stream)
{
    // Several steps in one call: the world-vertex pass of step i-1 runs on a second stream beside the
    // broad phase of step i (which reads centres and radii, not vertices), whose kernels get the
    // higher launch priority, and is joined before the narrow phase; the last step's pass runs in
    // line, so the state is complete when the call's work ends.  Every kernel computes what it
    // computes in the plain loop, so the results are the same.
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const SideStream* side = nullptr;
    if (!work->inlet && st->vert_owner && st->xform && st->n > 0 && st->n_verts > 0 && overlap_enabled())
        side = side_stream(s);
    // (the vertex pass overlaps the next broad phase only where the integrator runs it as a pass of its
    // own; for row counts that take the one-kernel integrator the plain loop is faster)
    const bool ovl = side && n_steps > 1 && !integrate_in_one_kernel(st->n);
    for (int i = 0; i < n_steps; ++i) {
        if (work->inlet) {
            int rc0 = mwd_inlet_step(st, work->inlet, stream);
            if (rc0) return rc0;
        }
        const bool fork = ovl && i > 0;
        if (fork) {
            MWD_CUDA(cudaEventRecord(side->fork, s));
            MWD_CUDA(cudaStreamWaitEvent(side->s, side->fork, 0));
            int rcv = launch_world_verts(*st, side->s);
            if (rcv) return rcv;
            MWD_CUDA(cudaEventRecord(side->join, side->s));
        }
        int rc;
        {
            LaunchPriority lp(fork ? side->prio_high : 0);
            rc = mwd_broadphase(st, scenes_dev, scenes_host, n_scenes, work, stream);
        }
        if (rc) return rc;
        if (fork) MWD_CUDA(cudaStreamWaitEvent(s, side->join, 0));
        // the broad phase zeroed the EPA counter (assign_kernel): no memset node between the kernels
        rc = narrow_force(st, scenes_dev, work, lanes, stream, true);
        if (rc) return rc;
        rc = (ovl && i < n_steps - 1) ? launch_integrate(*st, scenes_dev, work->status, s, false)
                                      : mwd_integrate(st, scenes_dev, work->status, stream);
        if (rc) return rc;
    }
    return MWD_OK;
}

}  // extern "C"
