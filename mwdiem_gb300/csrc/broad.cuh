// Launch arguments of the broad-phase kernels (internal to libmwdem).
#pragma once

#include "common.cuh"

namespace mwd {

struct BroadArgs {
    int32_t row_lo, row_hi;      // rows considered
    const int64_t* keys;         // given keys per row (reference-layout entry) or NULL: computed from pos
    const double* pos;           // (n,4) centres (FP64), used when keys == NULL and for walls
    const double* wall_normal;   // (n,4) wall normals
    const int32_t* info;         // (n,) scene << 1 | is_wall, or NULL: one scene, no walls
    const mwd_scene* scenes;     // device scene table
    int32_t walls;               // 1: emit wall candidates
    int32_t cull;                // 1: drop pairs whose bounding spheres are apart (pos.w = radius)
    int32_t append;              // 1: one kernel appends pairs (one atomic per warp, list order varies);
                                 // 0: count, scan, emit (list in cell order)
    int32_t pad_;
    int32_t* cell_count;         // (total_cells,) zero on entry and on exit
    int32_t* cell_start;         // (total_cells+1,)
    int32_t* cell_of;            // (n,)
    int32_t* scatter_out;        // (n,) rows scattered into their cells (any order within a cell)
    int32_t* sorted;             // (n,) rows in cell order, members in set order
    float4* sorted_pos;          // (n,) optional: their centres and radii, in the same order
    int32_t* sorted_cell;        // (n,) with sorted_pos: their cells
    int32_t* pair_count;         // (rows+1,)
    int32_t* scan_tmp;
    int32_t* pairs;              // (pair_cap,2)
    int64_t* n_pairs;
    int32_t* epa_count;          // optional: zeroed by assign_kernel for the narrow phase that follows
    uint32_t* status;
    int64_t total_cells;
    int64_t pair_cap;
    int32_t* tile_sums;          // optional: per-scan-tile cell counts, added to by assign_kernel, read by
                                 // the cell scan (no reduce pass) and zeroed by place_kernel
    int32_t walk_parts;          // append mode: threads per row (1, or 8: walls + own cell, 7 neighbours)
    // occupancy-compressed cell table (sparse = 1; needs tile_sums): a bit per cell of the dense
    // table, the cells' ranks among the occupied ones, and counts and starts per occupied cell, all
    // carved out of cell_count and cell_start (launch_broad sets these)
    int32_t sparse;
    int32_t n_words;             // bitmap words, ceil(total_cells / 32)
    int32_t words_pad;           // n_words + 1 rounded up to a multiple of 4: start of the next array
    int32_t compact_len;         // entries of the per-occupied-cell counts (rows + 1, rounded up to 4)
};

int64_t scan_tmp_ints(int64_t n);
int64_t scan_tile_sums_offset(int64_t n);  // where the persistent cell-tile counts start in scan_tmp
int launch_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* tmp, int64_t* total_out, int64_t cap,
                uint32_t* status, uint32_t overflow_bit, cudaStream_t s);
int launch_broad(const BroadArgs& a, cudaStream_t s);
// 1 when launch_broad would use the occupancy-compressed table for these sizes (mode: 0 automatic,
// 1 dense, 2 compressed where it fits)
int broad_sparse(int64_t rows, int64_t total_cells, int64_t tile_sum_ints, int mode);
// ints the cell_count and cell_start arrays need for that table (the compressed one carves its arrays
// out of their first entries)
void broad_table_ints(int64_t rows, int64_t total_cells, int sparse, int64_t* count_ints, int64_t* start_ints);
int launch_keys(int N, const double* com, double csx, double csy, double csz, int64_t nx, int64_t ny, int64_t* keys,
                cudaStream_t s);
int launch_minmax(const int64_t* keys, int lo, int hi, unsigned long long* mm, cudaStream_t s);
int launch_wall_pairs(int n_wall, int n_lo, int n_hi, const double* com, const double* wn, const double* wc,
                      double range, int32_t* flags, int32_t* offs, int32_t* tmp, int32_t* pairs, int64_t cap,
                      int64_t* n_out, uint32_t* status, cudaStream_t s);

}  // namespace mwd
