// Particle inlet: rows enter the domain during the run (MWDiem.py:685-714, where every 5 steps a new
// hull is made with Spherical_convex_polygon_maker_3D and translated to a random point of the inlet
// region).  Here every row exists from the start with its shape in the vertex tables; a waiting row
// carries MWD_INFO_INACTIVE, which the broad phase and the integrator skip.  One block per step
// counts the steps and, every `period` of them, activates the next rows: centre from the spawn table,
// at rest, identity orientation (the shape's orientation is in its body-frame vertices), world
// vertices written so the narrow phase of the same step sees them.
#include "common.cuh"

namespace mwd {
namespace {

struct alignas(32) dpos4 {
    double x, y, z, w;
};

__global__ void inlet_kernel(mwd_state st, mwd_inlet in)
{
    pdl_wait();
    pdl_launch_dependents();
    __shared__ int s_first, s_count;
    if (threadIdx.x == 0) {
        const int step = *in.step;
        *in.step = step + 1;
        const int first = *in.next_row;
        int count = 0;
        if (step % in.period == 0) {
            count = in.row_end - first;
            if (count > in.per_spawn) count = in.per_spawn;
            if (count < 0) count = 0;
            *in.next_row = first + count;
        }
        s_first = first;
        s_count = count;
    }
    __syncthreads();
    for (int k = 0; k < s_count; ++k) {
        const int r = s_first + k;
        const dpos4 sp = reinterpret_cast<const dpos4*>(in.spawn_pos)[r];
        dpos4 pos = reinterpret_cast<dpos4*>(st.pos)[r];
        pos.x = sp.x;
        pos.y = sp.y;
        pos.z = sp.z;
        if (threadIdx.x == 0) {
            reinterpret_cast<dpos4*>(st.pos)[r] = pos;
            reinterpret_cast<dpos4*>(st.dx_all)[r] = dpos4{0.0, 0.0, 0.0, 0.0};
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f), id = make_float4(1.f, 0.f, 0.f, 0.f);
            float4* f4s[] = {reinterpret_cast<float4*>(st.vel), reinterpret_cast<float4*>(st.vel_half),
                             reinterpret_cast<float4*>(st.w_half_bf), reinterpret_cast<float4*>(st.w_bf),
                             reinterpret_cast<float4*>(st.w), reinterpret_cast<float4*>(st.force),
                             reinterpret_cast<float4*>(st.torque)};
            for (float4* a : f4s) a[r] = z;
            reinterpret_cast<float4*>(st.q)[r] = id;
            reinterpret_cast<float4*>(st.q_half)[r] = id;
            reinterpret_cast<float4*>(st.q_all)[r] = id;
            reinterpret_cast<float4*>(st.q_acc)[r] = id;
            const_cast<int32_t*>(st.info)[r] &= ~MWD_INFO_INACTIVE;
        }
        // world = centre + r0 (identity rotation), formed as the integrator forms it: hi + (r0 + lo)
        const float hx = (float)pos.x, hy = (float)pos.y, hz = (float)pos.z;
        const float lx = (float)(pos.x - (double)hx), ly = (float)(pos.y - (double)hy), lz = (float)(pos.z - (double)hz);
        const float4* bv = reinterpret_cast<const float4*>(st.body_verts);
        float4* wv = reinterpret_cast<float4*>(st.world_verts);
        for (int j = st.vert_off[r] + threadIdx.x; j < st.vert_off[r + 1]; j += blockDim.x) {
            const float4 b = bv[j];
            const float rx = 1.f * b.x + 0.f * b.y + 0.f * b.z;
            const float ry = 0.f * b.x + 1.f * b.y + 0.f * b.z;
            const float rz = 0.f * b.x + 0.f * b.y + 1.f * b.z;
            wv[j] = make_float4(hx + (rx + lx), hy + (ry + ly), hz + (rz + lz), 0.f);
        }
        if (st.xform && threadIdx.x == 0) {
            float4* o = reinterpret_cast<float4*>(st.xform) + 4 * (size_t)r;
            o[0] = make_float4(1.f, 0.f, 0.f, 0.f);
            o[1] = make_float4(1.f, 0.f, 0.f, 0.f);
            o[2] = make_float4(1.f, hx, lx, hy);
            o[3] = make_float4(ly, hz, lz, 0.f);
        }
    }
}

}  // namespace
}  // namespace mwd

using namespace mwd;

extern "C" int mwd_inlet_step(mwd_state* st, const mwd_inlet* in, mwd_stream_t stream)
{
    if (!st || !in || in->period < 1 || in->per_spawn < 0 || !in->next_row || !in->step || !in->spawn_pos ||
        in->row_end > st->n) {
        set_error("mwd_inlet_step: bad arguments");
        return MWD_ERR_INVALID;
    }
    MWD_CUDA(launch_pdl(inlet_kernel, 1, 128, 0, reinterpret_cast<cudaStream_t>(stream), *st, *in));
    return MWD_OK;
}
