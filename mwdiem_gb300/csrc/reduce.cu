// Deterministic force/torque accumulation for the device step.
//
// The reference adds each pair's force and torques into the particle arrays with float atomics
// (gpu_fine_contact_detection.cu:1304-1319), so its sums depend on thread timing; its host build,
// run serially, adds them in pair order.  In deterministic mode the EPA pass writes each contact's
// F, TA, TB to its record slot, and these kernels add them per particle in pair-list order:
//
//   count    contacts per particle (walls excluded: the reference zeroes their rows, MWDiem.py:977-978)
//   scan     exclusive scan = each particle's segment
//   fill     keys (pair index << 32 | record << 1 | side) into the segments (counting sort)
//   reduce   per particle: sort its keys (a handful), then F += +-F_p, T += TA_p / TB_p in that order
//
// The FP32 sums are then the ones a serial loop over the pair list computes: reproducible from run
// to run and bit-identical to the oracle fed the same list.
#include "broad.cuh"
#include "common.cuh"
#include "narrow.cuh"
#include "reduce.cuh"

namespace mwd {

namespace {

__device__ __forceinline__ int64_t rec_pair(const DetArgs& d, int64_t i) { return d.recs[i].P; }

__device__ __forceinline__ int64_t n_records(const DetArgs& d)
{
    const int64_t c = *d.epa_count;
    return c < d.epa_cap ? c : d.epa_cap;
}

__global__ void det_count_kernel(DetArgs d)
{
    pdl_wait();
    pdl_launch_dependents();
    const int64_t m = n_records(d);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int2 pr = reinterpret_cast<const int2*>(d.pairs)[rec_pair(d, i)];
        if (!(d.info[pr.x] & 1)) atomicAdd(d.cnt + pr.x, 1);
        if (!(d.info[pr.y] & 1)) atomicAdd(d.cnt + pr.y, 1);
    }
}

__global__ void det_fill_kernel(DetArgs d)
{
    pdl_wait();
    pdl_launch_dependents();
    const int64_t m = n_records(d);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = rec_pair(d, i);
        const int2 pr = reinterpret_cast<const int2*>(d.pairs)[P];
        const int64_t key = (P << 32) | (i << 1);
        if (!(d.info[pr.x] & 1)) {
            const int slot = atomicSub(d.cnt + pr.x, 1) - 1;  // leaves the counts at zero
            d.keys[d.start[pr.x] + slot] = key;
        }
        if (!(d.info[pr.y] & 1)) {
            const int slot = atomicSub(d.cnt + pr.y, 1) - 1;
            d.keys[d.start[pr.y] + slot] = key | 1;
        }
    }
}

__global__ void det_reduce_kernel(DetArgs d)
{
    pdl_wait();
    pdl_launch_dependents();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= d.n) return;
    if (d.info[r] & 1) return;
    int64_t* k = d.keys + d.start[r];
    const int c = d.start[r + 1] - d.start[r];
    for (int j = 1; j < c; ++j) {  // insertion sort: a particle has a handful of contacts
        const int64_t v = k[j];
        int i = j;
        while (i > 0 && k[i - 1] > v) {
            k[i] = k[i - 1];
            --i;
        }
        k[i] = v;
    }
    f3 F = mk3(0.f, 0.f, 0.f), T = mk3(0.f, 0.f, 0.f);
    for (int j = 0; j < c; ++j) {
        const int64_t rec = (k[j] & 0xffffffffll) >> 1;
        const bool side_b = k[j] & 1;
        const float4* o = d.out + 3 * rec;
        if (side_b) {
            const float4 f = o[0], t = o[2];
            F = F + mk3(-1 * f.x, -1 * f.y, -1 * f.z);
            T = T + xyz(t);
        } else {
            const float4 f = o[0], t = o[1];
            F = F + xyz(f);
            T = T + xyz(t);
        }
    }
    reinterpret_cast<float4*>(d.force)[r] = f4(F, 0.f);
    reinterpret_cast<float4*>(d.torque)[r] = f4(T, 0.f);
}

}  // namespace

size_t det_scratch_bytes(int64_t n, int64_t epa_cap)
{
    Carver c;
    c.take<float4>(3 * epa_cap);
    c.take<int32_t>(n + 1);
    c.take<int32_t>(n + 1);
    c.take<int32_t>(scan_tmp_ints(n + 1));
    c.take<int64_t>(2 * epa_cap);
    return c.off;
}

DetArgs det_carve(void* scratch, int64_t n, int64_t epa_cap)
{
    Carver c;
    const size_t o_out = c.take<float4>(3 * epa_cap);
    const size_t o_cnt = c.take<int32_t>(n + 1);
    const size_t o_start = c.take<int32_t>(n + 1);
    const size_t o_tmp = c.take<int32_t>(scan_tmp_ints(n + 1));
    const size_t o_keys = c.take<int64_t>(2 * epa_cap);
    char* b = reinterpret_cast<char*>(scratch);
    DetArgs d = {};
    d.out = reinterpret_cast<float4*>(b + o_out);
    d.cnt = reinterpret_cast<int32_t*>(b + o_cnt);
    d.start = reinterpret_cast<int32_t*>(b + o_start);
    d.scan_tmp = reinterpret_cast<int32_t*>(b + o_tmp);
    d.keys = reinterpret_cast<int64_t*>(b + o_keys);
    d.n = (int32_t)n;
    d.epa_cap = epa_cap;
    return d;
}

int launch_det_reduce(const DetArgs& d, cudaStream_t s)
{
    const int T = 128;
    const unsigned gr = (unsigned)(num_sms() * 4);
    MWD_CUDA(launch_pdl(det_count_kernel, gr, T, 0, s, d));
    int rc = launch_scan(d.cnt, d.n, d.start, d.scan_tmp, nullptr, INT64_MAX, nullptr, 0, s);
    if (rc) return rc;
    MWD_CUDA(launch_pdl(det_fill_kernel, gr, T, 0, s, d));
    MWD_CUDA(launch_pdl(det_reduce_kernel, (unsigned)((d.n + T - 1) / T), T, 0, s, d));
    return MWD_OK;
}

}  // namespace mwd
