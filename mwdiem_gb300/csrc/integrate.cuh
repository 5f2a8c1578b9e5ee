// Launch arguments of the integrator kernels (internal to libmwdem).
#pragma once

#include "common.cuh"

namespace mwd {

struct VerletRefArgs {
    int32_t N;
    double *v, *v12, *w12bf, *q12, *q, *qall, *wbf, *w;
    const double *F, *T;
    double *verts, *com;
    const double *mass, *Iinv, *I;
    double* dxall;
    int32_t* n_reset;
    mwd_verlet_params p;
};

int launch_verlet_ref(const VerletRefArgs& a, cudaStream_t s);
// with_verts false (only with st.vert_owner and st.xform): the row pass alone; the world vertices are
// then rewritten from st.xform by a later launch_world_verts
int launch_integrate(const mwd_state& st, const mwd_scene* scenes, uint32_t* status, cudaStream_t s,
                     bool with_verts = true);
// true when launch_integrate with vertices runs one kernel for n rows (rows, then their vertices)
bool integrate_in_one_kernel(int64_t n);
// world vertices from st.xform (row transforms) through st.vert_owner, one thread per vertex
int launch_world_verts(const mwd_state& st, cudaStream_t s);
// the row pass, every state array it writes also written `mirror` bytes further on
int launch_integrate_rows_mirror(const mwd_state& st, const mwd_scene* scenes, uint32_t* status, int64_t mirror,
                                 cudaStream_t s);
// row transforms + world vertices from the current state (no integration)
int launch_refresh_vertices(const mwd_state& st, cudaStream_t s);

}  // namespace mwd
