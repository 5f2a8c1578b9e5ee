// Shared device helpers for libmwdem (sm_103a).
//
// Every translation unit of the library is compiled with --fmad=false and IEEE division/sqrt
// (no -use_fast_math): the narrow phase must round exactly like the reference kernel's
// operation sequence, which the oracle evaluates on the CPU without FMA contraction.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/mwdem.h"

namespace mwd {

struct f3 {
    float x, y, z;
};

__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z)
{
    f3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__host__ __device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ f3 operator/(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
// left-to-right sum of products, the reference's dot (gpu_fine_contact_detection.cu:21-24)
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ f3 cross(f3 a, f3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float norm2(f3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ f3 xyz(float4 v) { return mk3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 f4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }

// Hamilton product (w, x, y, z), operand order of gpu_fine_contact_detection.cu:613-624:
// vector part = b*a0 + a*b0 + a x b, scalar part = a0 b0 - a.b
__host__ __device__ __forceinline__ float4 qmul(float4 a, float4 b)
{
    f3 u = mk3(a.y, a.z, a.w), v = mk3(b.y, b.z, b.w);
    f3 s = (v * a.x + u * b.x) + cross(u, v);
    float f = a.x * b.x - dot(u, v);
    return make_float4(f, s.x, s.y, s.z);
}
__host__ __device__ __forceinline__ float4 qconj(float4 q) { return make_float4(q.x, q.y * (-1.f), q.z * (-1.f), q.w * (-1.f)); }
// q1 (0,v) q2, vector part (gpu_fine_contact_detection.cu:626-643)
__host__ __device__ __forceinline__ f3 qtrip(float4 q1, f3 v, float4 q2)
{
    float4 m1 = qmul(make_float4(0.f, v.x, v.y, v.z), q2);
    float4 m2 = qmul(q1, m1);
    return mk3(m2.y, m2.z, m2.w);
}

// Bounding-sphere test of two rows (pos.xyz = centre, pos.w = largest vertex distance from it).
// True when the centres are farther apart than rA + rB plus a rounding margin.  For such a pair the
// reference's first GJK test, d.(a* - b*) < 0 with d = cB - cA (gpu_fine_contact_detection.cu:1010-1023),
// is negative: d.a* <= d.cA + |d| rA and -d.b* <= -d.cB + |d| rB give d.(a* - b*) <= -|d| (|d| - rA - rB).
// The margin (1e-3 relative, 1e-5 of the coordinate magnitude) covers the FP32 rounding of the
// centres, the world vertices and the dot product, so the reference classifies the pair "no contact".
__device__ __forceinline__ bool spheres_apart(double4 pa, double4 pb)
{
    const float dx = (float)(pb.x - pa.x), dy = (float)(pb.y - pa.y), dz = (float)(pb.z - pa.z);
    const float mag = fmaxf(fmaxf(fabsf((float)pa.x), fabsf((float)pa.y)), fabsf((float)pa.z)) +
                      fmaxf(fmaxf(fabsf((float)pb.x), fabsf((float)pb.y)), fabsf((float)pb.z));
    const float r = (float)(pa.w + pb.w) * 1.001f + 1e-5f * mag + 1e-6f;
    return dx * dx + dy * dy + dz * dz > r * r;
}

// The same test on float copies of the centres (x, y, z, radius): the margin is far above the
// float rounding of the coordinates (6e-8 relative against 1e-5 of the magnitude).
__device__ __forceinline__ bool spheres_apart_f(float4 pa, float4 pb)
{
    const float dx = pb.x - pa.x, dy = pb.y - pa.y, dz = pb.z - pa.z;
    const float mag = fmaxf(fmaxf(fabsf(pa.x), fabsf(pa.y)), fabsf(pa.z)) + fmaxf(fmaxf(fabsf(pb.x), fabsf(pb.y)), fabsf(pb.z));
    const float r = (pa.w + pb.w) * 1.001f + 1e-5f * mag + 1e-6f;
    return dx * dx + dy * dy + dz * dz > r * r;
}

__device__ __forceinline__ void set_status(uint32_t* st, uint32_t bits)
{
    if (st && bits) atomicOr(st, bits);
}

}  // namespace mwd

// error plumbing shared by the host side of every translation unit
namespace mwd {
void set_error(const char* fmt, ...);
int cuda_check(cudaError_t e, const char* what);
int num_sms();

// Programmatic dependent launch.  The kernels of the device step are launched with launch_pdl: the
// next kernel's blocks may be scheduled while the previous kernel drains, and each of those kernels
// calls pdl_wait() before it reads anything (the wait returns once every earlier grid of the stream
// has completed and its writes are visible), then pdl_launch_dependents() so its own successor can
// be scheduled as soon as all of its blocks run.  MWD_PDL=0 in the environment turns it off.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
bool pdl_enabled();

// Priority given to the kernels launch_pdl launches from this thread (0: the stream's own).  A
// multi-step mwd_step raises it for the broad phase while the previous step's world-vertex pass runs
// beside it on a second stream, so that the broad phase's blocks take the SMs first.
extern thread_local int g_launch_priority;
struct LaunchPriority {
    int saved;
    explicit LaunchPriority(int p) : saved(g_launch_priority) { g_launch_priority = p; }
    ~LaunchPriority() { g_launch_priority = saved; }
};

// offsets of 256-byte aligned sub-arrays in one scratch allocation
struct Carver {
    size_t off = 0;
    template <class T>
    size_t take(size_t count)
    {
        size_t o = (off + 255) & ~size_t(255);
        off = o + count * sizeof(T);
        return o;
    }
};

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    unsigned na = 0;
    if (pdl_enabled()) {
        at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    if (g_launch_priority) {
        at[na].id = cudaLaunchAttributePriority;
        at[na].val.priority = g_launch_priority;
        ++na;
    }
    cfg.attrs = at;
    cfg.numAttrs = na;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
}  // namespace mwd

#define MWD_CUDA(call)                                                  \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return ::mwd::cuda_check(e_, #call);     \
    } while (0)

namespace mwd {

// Launch set-up of one kernel, per device: the raised dynamic shared-memory limit (a property of the
// function on the device that was current when it was set) and the resident blocks per SM for the
// last shared-memory size asked for.  Each is queried once per device and size, so that launches made
// during stream capture issue no other runtime calls; a mutex guards calls from several host threads.
struct LaunchSetup {
    std::mutex mu;
    bool attr[64] = {};
    size_t shm[64] = {};
    int per_sm[64] = {};
};

template <typename... KArgs>
int launch_setup(LaunchSetup& c, void (*kernel)(KArgs...), int threads, size_t shm, size_t shm_limit, int* per_sm)
{
    int dev = 0;
    MWD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return MWD_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(c.mu);
    if (shm_limit && !c.attr[dev]) {
        MWD_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm_limit));
        c.attr[dev] = true;
    }
    if (c.shm[dev] != shm || !c.per_sm[dev]) {
        int v = 0;
        MWD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, threads, shm));
        c.per_sm[dev] = v < 1 ? 1 : v;
        c.shm[dev] = shm;
    }
    *per_sm = c.per_sm[dev];
    return MWD_OK;
}

}  // namespace mwd
