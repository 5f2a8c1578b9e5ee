// mwd_contact_pairs_noalloc: the narrow phase + contact force over per-pair arrays (same inputs,
// outputs and results as mwd_contact_pairs) for callers that cannot let this library allocate
// device memory -- a host application whose own allocator owns (nearly) all of the GPU's memory, a
// process given a fixed slice of device memory up front, or a loop that cannot take the device-wide
// stall of the cudaFree that mwd_contact_pairs makes when its scratch grows.  The only scratch this
// path needs (the staging of the reference's overlapping stride-1 history writes: 17 bytes per pair)
// lives in a fixed-size array compiled into the library, so no call allocates or frees anything.
//
// Limits and sharing:
//  * at most MWD_NOALLOC_MAX_PAIRS pairs per call; larger calls fail with MWD_ERR_INVALID;
//  * the array, 4,456,448 bytes (4.25 MiB), belongs to every GPU that loads the library until the
//    process exits;
//  * every call uses the same array and leaves its contents behind; calls that overlap on the GPU
//    (different streams, or different host threads on one device) race on it and must be ordered
//    by the caller;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//    that device current; make that first call before any stream capture.
#include <mutex>

#include "common.cuh"
#include "narrow.cuh"

namespace mwd {
namespace {

constexpr int64_t kMaxPairs = MWD_NOALLOC_MAX_PAIRS;
// 16 bytes of staged history + 1 written flag per pair
constexpr size_t kStageBytes = (size_t)kMaxPairs * 16;
constexpr size_t kScratchBytes = kStageBytes + (size_t)kMaxPairs;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_addr_mu;
void* g_addr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device (looked up once per device).
int scratch_address(void** out)
{
    int dev = 0;
    MWD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return MWD_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_check(e == cudaSuccess ? cudaErrorInvalidSymbol : e,
                                                     "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return MWD_OK;
}

}  // namespace
}  // namespace mwd

using namespace mwd;

extern "C" int mwd_contact_pairs_noalloc(int64_t n_pairs, int32_t V, int32_t n_particles, const float* A_com,
                                         const float* B_com, const float* A_verts, const float* B_verts,
                                         const float* A_vel, const float* B_vel, const float* A_angvel,
                                         const float* B_angvel, const int32_t* A_nv, const int32_t* B_nv,
                                         const int32_t* A_id, const int32_t* B_id, float* hist, float* force,
                                         float* torque, const float* qA, const float* qB, const float* IsA,
                                         const float* IsB, int32_t* collision, const mwd_contact_params* prm,
                                         float* diag, uint32_t* status, mwd_stream_t stream)
{
    if (!prm || n_pairs < 0 || n_particles < 0) {
        set_error("mwd_contact_pairs_noalloc: bad arguments");
        return MWD_ERR_INVALID;
    }
    if (n_pairs > kMaxPairs) {
        set_error("mwd_contact_pairs_noalloc: %lld pairs exceed the fixed scratch of %lld pairs "
                  "(use mwd_contact_pairs for larger calls)", (long long)n_pairs, (long long)kMaxPairs);
        return MWD_ERR_INVALID;
    }
    if (n_pairs == 0) return MWD_OK;
    if (!A_com || !B_com || !A_verts || !B_verts || !A_vel || !B_vel || !A_angvel || !B_angvel || !A_nv || !B_nv ||
        !A_id || !B_id || !hist || !force || !torque || !qA || !qB || !IsA || !IsB || !collision) {
        set_error("mwd_contact_pairs_noalloc: null array");
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
    int lanes = prm->lanes ? prm->lanes : 8;
    if (lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32) {
        set_error("lanes per pair must be 4, 8, 16 or 32 (got %d)", lanes);
        return MWD_ERR_INVALID;
    }
    void* base = nullptr;
    int rc = scratch_address(&base);
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
        a.hist_stage = reinterpret_cast<float*>(base);
        a.hist_wrote = reinterpret_cast<uint8_t*>(base) + kStageBytes;
        // the flags must start at zero; the array still holds the previous call's
        MWD_CUDA(cudaMemsetAsync(a.hist_wrote, 0, (size_t)n_pairs, s));
    }
    rc = launch_narrow(a, 0, lanes, n_pairs, s);
    if (rc) return rc;
    if (!a.hist_mode) return launch_hist_resolve(hist, a.hist_stage, a.hist_wrote, n_pairs, s);
    return MWD_OK;
}
