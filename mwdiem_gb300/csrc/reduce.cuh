// Deterministic per-particle accumulation of the device step's contact forces (internal to libmwdem).
#pragma once

#include "common.cuh"
#include "narrow.cuh"

namespace mwd {

struct DetArgs {
    const int32_t* pairs;      // (P,2) pair list
    const SimplexRec* recs;    // EPA records (pair index of each contact)
    const int32_t* epa_count;  // (1,) records written by the GJK pass
    int64_t epa_cap;
    const int32_t* info;       // (n,) scene << 1 | is_wall
    float4* out;               // (epa_cap, 3) F, TA, TB per record (written by the EPA pass)
    int32_t* cnt;              // (n+1,) zero on entry and on exit
    int32_t* start;            // (n+1,)
    int32_t* scan_tmp;
    int64_t* keys;             // (2 epa_cap,)
    float* force;              // (n,4) written (not added to)
    float* torque;
    int32_t n;
    int32_t pad;
};

size_t det_scratch_bytes(int64_t n, int64_t epa_cap);
DetArgs det_carve(void* scratch, int64_t n, int64_t epa_cap);
int launch_det_reduce(const DetArgs& d, cudaStream_t s);

}  // namespace mwd
