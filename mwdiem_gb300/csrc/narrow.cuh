// Launch arguments of the narrow-phase kernel (internal to libmwdem).
#pragma once

#include "common.cuh"

namespace mwd {

constexpr int NARROW_THREADS = 128;

// a pair the GJK pass found in contact, with the simplex it stopped on (the EPA pass's input)
struct SimplexRec {
    float4 S[4];     // simplex points (w unused)
    int64_t P;       // pair index
    uint32_t ia;     // support indices on A, 8 bits each
    uint32_t ib;     // support indices on B
};

struct NarrowArgs {
    // mode 0: per-pair arrays in the reference's layout
    const float *A_com, *B_com, *A_verts, *B_verts, *A_vel, *B_vel, *A_w, *B_w, *qA, *qB, *IsA, *IsB;
    const int32_t *A_nv, *B_nv, *A_id, *B_id;
    const float* hist_in;   // history as read by the pairs
    float* hist_out;        // stride-4 mode: written in place
    float* hist_stage;      // stride-1 mode: (P,4) staging of each pair's four writes
    uint8_t* hist_wrote;    // stride-1 mode: (P,) 1 when the pair wrote
    float* force;           // (N,3)
    float* torque;          // (N,3)
    int32_t V;
    int32_t n_wall;
    int32_t hist_mode;
    int32_t pad0;
    int64_t n_pairs;
    mwd_material mat[2];
    // mode 1: particle tables
    mwd_state st;
    const mwd_scene* scenes;
    const int32_t* pairs;
    const int64_t* n_pairs_dev;
    int64_t pair_cap;
    // common
    int32_t* collision;     // optional
    float* diag;            // optional (P,10)
    int32_t* face_ids;      // optional (P,6): support indices of the final EPA face, A then B
    uint32_t* status;       // optional
    unsigned long long* work_counters;  // optional (3,): vertex dot products, EPA faces, support queries
    int32_t hull_cap;       // hull vertices staged per side
    int32_t pad1;
    // two-pass mode (table mode): list of pairs in contact and the simplex GJK stopped on
    int32_t* epa_count;
    void* epa_rec;          // (epa_cap,) 80-byte records
    int64_t epa_cap;
    int32_t pre_culled;     // the pair list holds only pairs whose bounding spheres overlap
    int32_t epa_zeroed;     // 1: epa_count was zeroed by an earlier kernel of the stream (the broad phase)
    float4* det_out;        // deterministic mode: (epa_cap, 3) F, TA, TB per EPA record instead of atomics
    int32_t epa_global;     // 1: the EPA pass reads the hulls from global memory (L1) instead of staging them
    int32_t pad3;
    // persistent tangential history (two-pass mode): tables read at *hist_parity, written at the other
    unsigned long long* hist_keys;
    float4* hist_vals;
    int64_t hist_cap;
    int32_t* hist_parity;
};

int launch_narrow(const NarrowArgs& a, int mode, int lanes, int64_t n_hint, cudaStream_t s);
int launch_narrow_two_pass(const NarrowArgs& a, int lanes, cudaStream_t s);
int launch_hist_resolve(float* hist, const float* stage, const uint8_t* wrote, int64_t n, cudaStream_t s);
size_t narrow_smem_bytes(int lpp, int hull_cap);

}  // namespace mwd
