// Cell-hash broad phase for sm_103a.
//
// Reference: MWDiem.py:808-817 (wall candidates, cell keys) and
// LIBRARIES/LIBRARY_Coarse_contact_detection.py:84-155 (Linked_cell_hash).  The reference groups ids
// in a dict of Python sets keyed by the integer cell key and walks an 8-cell forward stencil with
// linear key offsets (+1, +nx, +nx*ny, +nx*ny+1, +nx*ny+1+nx, +nx*ny+nx, +nx+1), no row-wrap
// guard, same-cell pairs in set iteration order.  Here:
//
//   assign   key -> dense cell index (per scene key range), atomic count per cell
//   scan     exclusive scan of the counts = cell-start table (a one-digit radix/counting sort)
//   place    rows into their cell's slot range, each shared cell's members sorted by id and then
//            put in CPython 3.12 set iteration order by its last-arriving member (counts back to zero)
//   count    per row: wall candidates + later members of its cell + members of the 7 neighbours
//   scan     exclusive scan of the counts = output offsets
//   emit     the same walk, writing [A, B] pairs
//
// The list of (count, scan, emit) depends only on the inputs and is in cell order.  The device
// step's broad phase (append mode) replaces those three stages by one kernel: each thread walks its
// row twice (count, then write) and a warp reserves its slots with one atomic, so the same oriented
// pairs come out in an order that varies from run to run (the orientation, A before B, still comes
// from the set order).
#include "broad.cuh"
#include "common.cuh"

namespace mwd {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh, int* total)
{
    // sh: SCAN_THREADS / 32 ints
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = lane < SCAN_THREADS / 32 ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_THREADS / 32) sh[lane] = w;
    }
    __syncthreads();
    int base = wid ? sh[wid - 1] : 0;
    *total = sh[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void scan_reduce_kernel(const int32_t* in, int64_t n, int32_t* block_sums)
{
    pdl_wait();
    pdl_launch_dependents();
    __shared__ int sh[SCAN_THREADS / 32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int s = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        int64_t i = base + (int64_t)k * SCAN_THREADS + threadIdx.x;
        if (i < n) s += in[i];
    }
    int tot;
    block_exclusive_scan(s, sh, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// out[i] = sum(in[0..i)), out[n] = total; in and out may alias.  Each block adds up the tile totals
// of the blocks before it (at most a few thousand values), so no separate pass scans the totals.
// exclusive scan of up to SCAN_SMALL_MAX elements by one block (one launch instead of two)
constexpr int SCAN_SMALL_THREADS = 1024;
constexpr int64_t SCAN_SMALL_MAX = 64 * SCAN_SMALL_THREADS;
__global__ void __launch_bounds__(SCAN_SMALL_THREADS) scan_small_kernel(const int32_t* in, int64_t n, int32_t* out,
                                                                        int64_t* total_out, int64_t cap,
                                                                        uint32_t* status, uint32_t overflow_bit)
{
    pdl_wait();
    pdl_launch_dependents();
    __shared__ int sh[SCAN_SMALL_THREADS / 32];
    const int per = (int)((n + SCAN_SMALL_THREADS - 1) / SCAN_SMALL_THREADS);
    const int64_t base = (int64_t)threadIdx.x * per;
    int sum = 0;
    for (int k = 0; k < per; ++k)
        if (base + k < n) sum += in[base + k];
    // block scan of the per-thread sums (SCAN_SMALL_THREADS / 32 warps)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = sh[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    int ex = (wid ? sh[wid - 1] : 0) + x - sum;
    for (int k = 0; k < per; ++k) {
        if (base + k >= n) break;
        const int v = in[base + k];
        out[base + k] = ex;
        ex += v;
    }
    if (threadIdx.x == 0) {
        const int64_t t = sh[SCAN_SMALL_THREADS / 32 - 1];
        out[n] = (int32_t)t;
        if (total_out) *total_out = t < cap ? t : cap;
        if (t > cap) set_status(status, overflow_bit);
    }
}

// The final pass of the scan: block b writes the exclusive prefix of its tile, offset by the totals of
// tiles 0..b-1.  The tile's values are loaded first (two int4 per thread when vec: both arrays 16-byte
// aligned), so that their latency overlaps the loads of the earlier tiles' totals, and one block pass
// (a single barrier) both scans the thread sums and adds up those totals.
// WORDS: the input is a bitmap whose set bits are counted (v = popc(word)); each word is also copied to
// words_copy and zeroed in place (the bitmap is rebuilt by the next broad phase).
template <bool WORDS>
__global__ void scan_final_kernel(const int32_t* in, int64_t n, const int32_t* block_sums, int32_t* out, int nb,
                                  int64_t* total_out, int64_t cap, uint32_t* status, uint32_t overflow_bit, int vec,
                                  int32_t* words_copy)
{
    static_assert(SCAN_ITEMS == 8, "two int4 per thread");
    pdl_wait();
    pdl_launch_dependents();
    constexpr int W = SCAN_THREADS / 32;
    __shared__ int sh_x[W], sh_p[W];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    const bool full = vec && base + SCAN_ITEMS <= n;
    int v[SCAN_ITEMS];
    if (full) {
        const int4 q0 = reinterpret_cast<const int4*>(in + base)[0];
        const int4 q1 = reinterpret_cast<const int4*>(in + base)[1];
        v[0] = q0.x; v[1] = q0.y; v[2] = q0.z; v[3] = q0.w;
        v[4] = q1.x; v[5] = q1.y; v[6] = q1.z; v[7] = q1.w;
        if (WORDS) {
            reinterpret_cast<int4*>(words_copy + base)[0] = q0;
            reinterpret_cast<int4*>(words_copy + base)[1] = q1;
            int32_t* z = const_cast<int32_t*>(in) + base;
            reinterpret_cast<int4*>(z)[0] = make_int4(0, 0, 0, 0);
            reinterpret_cast<int4*>(z)[1] = make_int4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            v[k] = base + k < n ? in[base + k] : 0;
            if (WORDS && base + k < n) {
                words_copy[base + k] = v[k];
                const_cast<int32_t*>(in)[base + k] = 0;
            }
        }
    }
    if (WORDS) {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) v[k] = __popc((unsigned)v[k]);
    }
    // the totals of the tiles before this one, eight independent loads in flight per thread (a
    // 15M-cell table has 7,300 tiles); integer sums, so the order does not matter
    constexpr int U = 8;
    const int lim = (int)blockIdx.x;
    int acc[U] = {};
    int i = threadIdx.x;
    for (; i + (U - 1) * SCAN_THREADS < lim; i += U * SCAN_THREADS) {
#pragma unroll
        for (int u = 0; u < U; ++u) acc[u] += block_sums[i + u * SCAN_THREADS];
    }
    for (; i < lim; i += SCAN_THREADS) acc[0] += block_sums[i];
    int part = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) part += acc[u];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) sum += v[k];
    // warp: inclusive scan of the thread sums, total of the tile totals; block: one barrier
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const int ps = __reduce_add_sync(0xffffffffu, part);
    if (lane == 31) sh_x[wid] = x;
    if (lane == 0) sh_p[wid] = ps;
    __syncthreads();
    int before = 0, tot = 0, offset = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int xs = sh_x[w];
        before += w < wid ? xs : 0;
        tot += xs;
        offset += sh_p[w];
    }
    int ex = offset + before + x - sum;
    if (full) {
        int e[SCAN_ITEMS];
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            e[k] = ex;
            ex += v[k];
        }
        reinterpret_cast<int4*>(out + base)[0] = make_int4(e[0], e[1], e[2], e[3]);
        reinterpret_cast<int4*>(out + base)[1] = make_int4(e[4], e[5], e[6], e[7]);
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            if (base + k < n) out[base + k] = ex;
            ex += v[k];
        }
    }
    if ((int)blockIdx.x == nb - 1 && threadIdx.x == 0) {
        const int64_t t = (int64_t)offset + tot;
        out[n] = (int32_t)t;
        if (total_out) *total_out = t < cap ? t : cap;
        if (t > cap) set_status(status, overflow_bit);
    }
}

inline int aligned16(const void* p, const void* q)
{
    return ((reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(q)) & 15u) == 0 ? 1 : 0;
}

// ---------------------------------------------------------------- CPython set iteration order

// Members m[0..k) (ascending ids, the insertion order of the reference's dict walk) reordered as
// list(set) would list them in CPython 3.12: open addressing on hash(i) = i, up to 9 linear probes
// when they fit below the mask, then perturbation (perturb >>= 5; i = 5 i + 1 + perturb), table of
// 8 slots grown to the next power of two above 4*used when fill*5 >= mask*3.
// ids are hashed as (row - base): the particle number inside its own scene, which is what the
// reference hashes (each scene's particles are numbered from 0)
template <unsigned TABCAP>
__device__ bool pyset_order(const int* m, int k, int* out, int* tab, unsigned char* used, int* tmp,
                            unsigned char* used2, int base)
{
    unsigned mask = 7;
    for (int s = 0; s < 8; ++s) used[s] = 0;
    int fill = 0;
    for (int e = 0; e < k; ++e) {
        const uint64_t h = (uint64_t)(uint32_t)(m[e] - base);
        unsigned i = (unsigned)(h & mask);
        uint64_t perturb = h;
        for (;;) {
            unsigned j = i;
            int probes = (i + 9 <= mask) ? 9 : 0;
            bool found = false;
            for (;;) {
                if (!used[j]) { found = true; break; }
                if (probes-- == 0) break;
                j++;
            }
            if (found) { i = j; break; }
            perturb >>= 5;
            i = (unsigned)((i * 5ull + 1ull + perturb) & mask);
        }
        used[i] = 1;
        tab[i] = m[e];
        fill++;
        if ((unsigned)fill * 5u >= mask * 3u) {
            unsigned newsize = 8, minused = (unsigned)fill * 4u;
            while (newsize <= minused) newsize <<= 1;
            if (newsize > TABCAP) return false;
            unsigned newmask = newsize - 1;
            for (unsigned s = 0; s < newsize; ++s) used2[s] = 0;
            for (unsigned s = 0; s <= mask; ++s) {
                if (!used[s]) continue;
                const uint64_t hh = (uint64_t)(uint32_t)(tab[s] - base);
                unsigned ii = (unsigned)(hh & newmask);
                uint64_t pp = hh;
                for (;;) {
                    if (!used2[ii]) break;
                    bool placed = false;
                    if (ii + 9 <= newmask)
                        for (unsigned q = 1; q <= 9; ++q)
                            if (!used2[ii + q]) { ii += q; placed = true; break; }
                    if (placed) break;
                    pp >>= 5;
                    ii = (unsigned)((ii * 5ull + 1ull + pp) & newmask);
                }
                used2[ii] = 1;
                tmp[ii] = tab[s];
            }
            mask = newmask;
            for (unsigned s = 0; s <= mask; ++s) {
                used[s] = used2[s];
                tab[s] = tmp[s];
            }
        }
    }
    int c = 0;
    for (unsigned s = 0; s <= mask; ++s)
        if (used[s]) out[c++] = tab[s];
    return true;
}

// list({lo, hi}) in CPython 3.12 (lo < hi inserted in that order, ids hashed as id - base): true when lo
// comes first.  Two entries leave the 8-slot table unresized, and no slot index i has i + 9 <= 7, so a
// collision goes straight to perturbation (pyset_order with k = 2); once the perturbation has shifted
// out, i -> 5 i + 1 (mod 8) visits every slot, so the loop ends within 15 steps.
__device__ __forceinline__ bool pyset_pair_lo_first(int lo, int hi, int base)
{
    const unsigned ia = (unsigned)(lo - base) & 7u;
    const uint64_t h = (uint64_t)(uint32_t)(hi - base);
    unsigned i = (unsigned)(h & 7u);
    uint64_t perturb = h;
    while (i == ia) {
        perturb >>= 5;
        i = (unsigned)((i * 5ull + 1ull + perturb) & 7u);
    }
    return ia < i;
}

// cells up to SMALL_CELL members are ordered by one thread with the table in local memory; larger
// cells go to a list handled by one warp each with the table in shared memory
constexpr int SMALL_CELL = 32;
constexpr int SMALL_TAB = 128;   // table size CPython reaches for <= 32 members
constexpr int BIG_TAB = 512;     // ... for <= 306 members
constexpr int BIG_CELL = 306;

// ---------------------------------------------------------------- broad-phase kernels

__device__ __forceinline__ int scene_of(const BroadArgs& a, int r)
{
    return a.info ? ((a.info[r] & ~MWD_INFO_INACTIVE) >> 1) : 0;
}
__device__ __forceinline__ bool inactive(const BroadArgs& a, int r) { return a.info && (a.info[r] & MWD_INFO_INACTIVE); }
__device__ __forceinline__ bool is_wall(const BroadArgs& a, int r) { return a.info ? (a.info[r] & 1) : false; }

struct alignas(32) dpos {
    double x, y, z, w;
};

// The occupancy-compressed cell table (a.sparse; on request), for many rows spread over a much larger
// dense key range (batched scenes: 2M rows, 15M cells).  Instead of a count and a start for every cell:
//   cell_count[0 .. n_words)            a bit per cell, set by the rows in it (zero on entry and exit)
//   cell_start[0 .. n_words]            occupied cells before each word (the scan of the words' popc)
//   cell_start[words_pad ..)            a copy of the bits, read by the later passes
//   cell_count[words_pad ..)            rows per occupied cell, indexed by the cell's rank among the
//                                       occupied ones (zero on entry and exit)
//   cell_start[2 words_pad ..)          the scan of those counts: each occupied cell's range in the list
// A cell's rank is two loads from small arrays (3.8 MB for 15M cells, resident in L2) and a popc.  The
// sorted list, the pairs and their order are those of the dense table.
__device__ __forceinline__ uint32_t* occ_bits(const BroadArgs& a) { return reinterpret_cast<uint32_t*>(a.cell_count); }
__device__ __forceinline__ int32_t* occ_count(const BroadArgs& a) { return a.cell_count + a.words_pad; }
__device__ __forceinline__ const uint32_t* occ_copy(const BroadArgs& a)
{
    return reinterpret_cast<const uint32_t*>(a.cell_start + a.words_pad);
}
__device__ __forceinline__ int32_t* occ_start(const BroadArgs& a) { return a.cell_start + 2 * a.words_pad; }
__device__ __forceinline__ int words_tiles(const BroadArgs& a) { return (a.n_words + SCAN_TILE - 1) / SCAN_TILE; }
// per-tile counts of the occupied-cell scan, after those of the word scan
__device__ __forceinline__ int32_t* occ_tile_sums(const BroadArgs& a) { return a.tile_sums + words_tiles(a) + 1; }

// rank of cell g among the occupied cells (sparse table), -1 when it is empty
__device__ __forceinline__ int occ_index(const BroadArgs& a, int g)
{
    const uint32_t w = occ_copy(a)[g >> 5];
    const uint32_t bit = 1u << (g & 31);
    return (w & bit) ? a.cell_start[g >> 5] + __popc(w & (bit - 1u)) : -1;
}

// [start, end) of cell g in the sorted list
__device__ __forceinline__ int2 cell_range(const BroadArgs& a, int g)
{
    if (!a.sparse) return make_int2(a.cell_start[g], a.cell_start[g + 1]);
    const int c = occ_index(a, g);
    if (c < 0) return make_int2(0, 0);
    const int32_t* st = occ_start(a);
    return make_int2(st[c], st[c + 1]);
}

// rows in the sorted list (those with a cell)
__device__ __forceinline__ int n_sorted_rows(const BroadArgs& a)
{
    return a.sparse ? occ_start(a)[a.compact_len] : a.cell_start[a.total_cells];
}

// trunc(fl64(p / cs)), numpy's astype(int) of the FP64 quotient (MWDiem.py:813-816).  The float
// quotient q = (float)p * (float)(1/cs) is within 1.8e-7 |q| of the double one (three roundings of
// 2^-24), so when its fractional part is more than 2^-21 |q| away from 0 and from 1 it truncates to
// the same integer; otherwise (and for inv = 0, |q| >= 2^23, NaN) the FP64 division decides.  FP64
// runs at 1/64 of the FP32 rate on this GPU and the division is a long sequence of it.
__device__ __forceinline__ int64_t cell_coord(double p, double cs, float inv)
{
    if (inv != 0.f) {
        const float q = (float)p * inv;
        const float aq = fabsf(q);
        if (aq < 8388608.f) {
            const float t = truncf(q);
            const float fr = aq - fabsf(t);  // exact: |t| <= aq < |t| + 1
            const float band = aq * 4.76837158203125e-7f;
            if (fr > band && fr < 1.f - band) return (int64_t)t;
        }
    }
    return (int64_t)(p / cs);
}

__device__ __forceinline__ int64_t row_key(const BroadArgs& a, const mwd_scene& sc, int r)
{
    if (a.keys) return a.keys[r];
    const dpos p = reinterpret_cast<const dpos*>(a.pos)[r];
    const int64_t xc = cell_coord(p.x, sc.cs[0], sc.inv_cs[0]);
    const int64_t yc = cell_coord(p.y, sc.cs[1], sc.inv_cs[1]);
    const int64_t zc = cell_coord(p.z, sc.cs[2], sc.inv_cs[2]);
    return xc + yc * sc.nx + zc * sc.nx * sc.ny;
}

__global__ void assign_kernel(BroadArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.append) *a.n_pairs = 0;  // appended to by pairs_append_kernel
        if (a.epa_count)  // the EPA record count, the EPA pass's work queue and retry count
            for (int k = 0; k < 8; ++k) a.epa_count[k] = 0;
    }
    const int r = a.row_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.row_hi) return;
    if (is_wall(a, r) || inactive(a, r)) {  // walls and rows waiting at an inlet have no cell
        a.cell_of[r] = -1;
        return;
    }
    const mwd_scene& sc = a.scenes[scene_of(a, r)];
    const int64_t local = row_key(a, sc, r) - sc.key_min;
    if (local < 0 || local >= sc.n_keys) {
        a.cell_of[r] = -1;
        set_status(a.status, MWD_ST_CELL_RANGE);
        return;
    }
    const int g = (int)(sc.cell_base + local);
    a.cell_of[r] = g;
    if (a.sparse) {
        // the cell's bit; the first row to set it adds one occupied cell to its word's scan tile
        const uint32_t bit = 1u << (g & 31);
        if (!(atomicOr(occ_bits(a) + (g >> 5), bit) & bit)) {
            const int tile = (g >> 5) / SCAN_TILE;
            const unsigned peers = __match_any_sync(__activemask(), tile);
            if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(a.tile_sums + tile, __popc(peers));
        }
        return;
    }
    atomicAdd(a.cell_count + g, 1);
    if (a.tile_sums) {
        // one atomic per tile per warp (consecutive rows mostly share a tile)
        const int tile = g / SCAN_TILE;
        const unsigned peers = __match_any_sync(__activemask(), tile);
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(a.tile_sums + tile, __popc(peers));
    }
}

// sparse table: rows per occupied cell (by rank), with per-tile totals for the scan that follows
__global__ void occ_count_kernel(BroadArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    {  // the word scan has read the word tiles' totals: zero them for the next broad phase
        const int nb = words_tiles(a);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= nb; i += gridDim.x * blockDim.x) a.tile_sums[i] = 0;
    }
    const int r = a.row_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.row_hi) return;
    const int g = a.cell_of[r];
    if (g < 0) return;
    const int c = occ_index(a, g);
    atomicAdd(occ_count(a) + c, 1);
    const int tile = c / SCAN_TILE;
    const unsigned peers = __match_any_sync(__activemask(), tile);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(occ_tile_sums(a) + tile, __popc(peers));
}

// write row v at sorted position i of cell g, with its centre/radius and cell alongside
__device__ __forceinline__ void place(const BroadArgs& a, int i, int v, int g)
{
    a.sorted[i] = v;
    if (a.sorted_pos) {
        const double4 p = reinterpret_cast<const double4*>(a.pos)[v];
        a.sorted_pos[i] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
        a.sorted_cell[i] = g;
    }
}

// members of cell g (k of them, from scatter_out[s..s+k), written by other threads of this grid and
// read past L1) ranked by id, then written in set order
__device__ __forceinline__ void order_small_cell(const BroadArgs& a, int g, int s, int k)
{
    int m[SMALL_CELL];
    for (int j = 0; j < k; ++j) {
        int v = __ldcg(a.scatter_out + s + j);
        int i = j;
        while (i > 0 && m[i - 1] > v) {
            m[i] = m[i - 1];
            --i;
        }
        m[i] = v;
    }
    int o[SMALL_CELL];
    int tab[SMALL_TAB], tmp[SMALL_TAB];
    unsigned char used[SMALL_TAB], used2[SMALL_TAB];
    const int base = a.info ? a.scenes[scene_of(a, m[0])].row_begin : 0;
    pyset_order<SMALL_TAB>(m, k, o, tab, used, tmp, used2, base);
    for (int j = 0; j < k; ++j) place(a, s + j, o[j], g);
}

// The place pass: every row into its cell's range of the sorted list (the counting sort's scatter)
// and each cell's members into CPython set order, in one kernel.  A row alone in its cell (most rows)
// is written at its cell's start and the cell's count set back to zero.  The members of a shared
// cell claim slots with atomicSub on the cell's count (low 16 bits, counting down to zero), write
// themselves into scatter_out, and then add 1 << 16 to the same word with an acquire-release atomic:
// each member's add releases its write, and the member whose add finds k - 1 earlier ones (acquiring
// all of them) orders the cell, in its own thread up to SMALL_CELL members, else by the first warp of its block with the
// tables in shared memory; it sets the count back to zero.  (With PAIRS, of a two-member cell the
// first member to arrive leaves its id in the count word by an atomic exchange and the second,
// finding it there, places both.)  Cells beyond BIG_CELL members are written in ascending ids, beyond
// 65,535 (the packed count) in claim order; both are flagged MWD_ST_CELL_CROWDED.
constexpr int PLACE_THREADS = 128;
constexpr int PACKED_MAX = 0xffff;
// PAIRS: two-member cells take the exchange path below instead of the claim-and-count one -- on the
// large row counts that launch this instance (a shorter chain: one atomic); the smaller counts keep the
// smaller kernel, whose code is fetched cold after the L2 flush of a short step
template <bool PAIRS>
__global__ void __launch_bounds__(PLACE_THREADS) place_kernel(BroadArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    __shared__ int s_crowd[PLACE_THREADS];
    __shared__ int s_nc;
    if (threadIdx.x == 0) s_nc = 0;
    if (a.tile_sums) {  // read by the cell scan, which has finished: zero for the next broad phase
        int32_t* ts = a.sparse ? occ_tile_sums(a) : a.tile_sums;
        const int64_t nb = a.sparse ? (a.compact_len + SCAN_TILE - 1) / SCAN_TILE
                                    : (a.total_cells + SCAN_TILE - 1) / SCAN_TILE;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nb; i += (int64_t)gridDim.x * blockDim.x)
            ts[i] = 0;
    }
    __syncthreads();
    const int r = a.row_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (r < a.row_hi) {
        // the row's own centre, loaded beside its cell lookups (most rows are alone in their cell)
        double4 pr = make_double4(0.0, 0.0, 0.0, 0.0);
        if (a.sorted_pos) pr = reinterpret_cast<const double4*>(a.pos)[r];
        const int g = a.cell_of[r];
        if (g >= 0) {
            // the cell's count word and range: by cell (dense table) or by its rank (sparse table)
            const int c = a.sparse ? occ_index(a, g) : g;
            int32_t* cnt = (a.sparse ? occ_count(a) : a.cell_count) + c;
            const int32_t* st = (a.sparse ? occ_start(a) : a.cell_start) + c;
            const int s = st[0], k = st[1] - s;
            if (k == 1) {
                *cnt = 0;
                a.sorted[s] = r;
                if (a.sorted_pos) {
                    a.sorted_pos[s] = make_float4((float)pr.x, (float)pr.y, (float)pr.z, (float)pr.w);
                    a.sorted_cell[s] = g;
                }
            } else if (PAIRS && k == 2) {
                // the first member leaves its id in the count word (flagged), the second finds it there,
                // orders both and sets the word back to zero: the id travels in the atomic, no fence
                const unsigned prev = atomicExch(reinterpret_cast<unsigned*>(cnt), 0x80000000u | (unsigned)r);
                if (prev & 0x80000000u) {
                    *cnt = 0;
                    const int o = (int)(prev & 0x7fffffffu);
                    const int lo = min(r, o), hi = max(r, o);
                    const int base = a.info ? a.scenes[scene_of(a, lo)].row_begin : 0;
                    const bool lo_first = pyset_pair_lo_first(lo, hi, base);
                    place(a, s + (lo_first ? 0 : 1), lo, g);
                    place(a, s + (lo_first ? 1 : 0), hi, g);
                }
            } else if (k > PACKED_MAX) {
                const int slot = atomicSub(cnt, 1) - 1;
                place(a, s + slot, r, g);
                if (slot == 0) set_status(a.status, MWD_ST_CELL_CROWDED);
            } else {
                unsigned* w = reinterpret_cast<unsigned*>(cnt);
                const int slot = (int)(atomicSub(w, 1u) & 0xffffu) - 1;
                a.scatter_out[s + slot] = r;
                unsigned prev;  // (two full fences around a relaxed add measured 1-2 us slower per pour step)
                asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;"
                             : "=r"(prev) : "l"(w), "r"(0x10000u) : "memory");
                const unsigned before = prev >> 16;
                if ((int)before == k - 1) {
                    *w = 0u;
                    if (k <= SMALL_CELL) order_small_cell(a, g, s, k);
                    else s_crowd[atomicAdd(&s_nc, 1)] = g;
                }
            }
        }
    }
    __syncthreads();
    const int nc = s_nc;
    if (nc == 0 || threadIdx.x >= 32) return;
    // the block's crowded cells, one at a time by its first warp: members ranked by id in parallel,
    // lane 0 replaying the set inserts with the table in shared memory
    __shared__ int m[BIG_CELL];
    __shared__ int o[BIG_CELL];
    __shared__ int tab[BIG_TAB], tmp[BIG_TAB];
    __shared__ unsigned char used[BIG_TAB], used2[BIG_TAB];
    for (int c = 0; c < nc; ++c) {
        const int g = s_crowd[c];
        const int2 se = cell_range(a, g);
        const int s = se.x, k = se.y - se.x;
        if (k > BIG_CELL) {
            // beyond the emulated table size: ascending ids, flagged
            for (int j = threadIdx.x; j < k; j += 32) {
                int v = __ldcg(a.scatter_out + s + j), rank = 0;
                for (int i = 0; i < k; ++i) rank += __ldcg(a.scatter_out + s + i) < v;
                place(a, s + rank, v, g);
            }
            if (threadIdx.x == 0) set_status(a.status, MWD_ST_CELL_CROWDED);
            __syncwarp();
            continue;
        }
        for (int j = threadIdx.x; j < k; j += 32) {
            int v = __ldcg(a.scatter_out + s + j), rank = 0;
            for (int i = 0; i < k; ++i) rank += __ldcg(a.scatter_out + s + i) < v;
            m[rank] = v;
        }
        __syncwarp();
        const int base = a.info ? a.scenes[scene_of(a, m[0])].row_begin : 0;
        if (threadIdx.x == 0) pyset_order<BIG_TAB>(m, k, o, tab, used, tmp, used2, base);
        __syncwarp();
        for (int j = threadIdx.x; j < k; j += 32) place(a, s + j, o[j], g);
        __syncwarp();
    }
}

// walls of one scene staged as floats (centre + radius, normal) by the append kernel
constexpr int WALL_STAGE = 16;
struct WallStage {
    const float4* c;  // (nw,) centre, bounding radius
    const float4* n;  // (nw,) normal, and n . c in float
    const float2* m;  // (nw,) |n|_1, and |c|_1 |n|_1 + range: the parts of the margin fixed per wall
    int scene;        // the scene they belong to (-1: nothing staged)
    int nw;
};

// the reference's forward stencil in linear keys, o = 0..6: +1, +nx, +nx*ny, +nx*ny+1, +nx*ny+1+nx,
// +nx*ny+nx, +nx+1 (LIBRARY_Coarse_contact_detection.py:96-129), from bit masks (no local array)
__device__ __forceinline__ int64_t forward_offset(int o, int64_t nx, int64_t nxy)
{
    return (((0x3c >> o) & 1) ? nxy : 0) + (((0x72 >> o) & 1) ? nx : 0) + ((0x59 >> o) & 1);
}

// every candidate of the row at sorted position t (row r, cell g), passed to sink(A, B).
// ws: optional float copies of the row's scene walls for the wall-distance test.
// part: -1 the whole walk; 0 the walls and the later members of the row's own cell; 1..7 the
// members of forward neighbour cell part - 1 (the eight parts together are the whole walk).
// what: WALK_WALLS, WALK_CELLS or both (walls first).
constexpr int WALK_WALLS = 1, WALK_CELLS = 2;
template <class Sink>
__device__ __forceinline__ void walk_pairs(const BroadArgs& a, int t, int r, int g, const mwd_scene& sc, int scene,
                                           const WallStage* ws, Sink&& sink, int part = -1,
                                           int what = WALK_WALLS | WALK_CELLS)
{
    const bool cull = a.cull && a.sorted_pos;
    const float4 me = a.sorted_pos ? a.sorted_pos[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    // wall candidates (MWDiem.py:808-811): pair [particle, wall] when |n . (p - c)| < wall_range (FP64)
    if (a.walls && part <= 0 && (what & WALK_WALLS)) {
        if (ws && ws->scene == scene && a.sorted_pos) {
            // FP32 test with a margin above its rounding error: s = n . p - n . c with the inputs rounded
            // to float, three products, three sums and n . c rounded once at staging is within
            // 6 u |n|_1 (|p|_1 + |c|_1) of the exact value (u = 2^-24); the margin, 1e-6 (~16.8 u) times
            // that sum plus the range, covers it with room.  Inside the margin band the FP64 test decides.
            const float range = (float)sc.wall_range;
            const float me1 = fabsf(me.x) + fabsf(me.y) + fabsf(me.z);
            for (int k = 0; k < ws->nw; ++k) {
                const float4 c = ws->c[k], nr = ws->n[k];
                const float2 wm = ws->m[k];
                const float sf = (nr.x * me.x + nr.y * me.y + nr.z * me.z) - nr.w;
                const float mg = 1e-6f * (me1 * wm.x + wm.y);
                bool in;
                if (fabsf(sf) < range - mg) in = true;
                else if (fabsf(sf) > range + mg) in = false;
                else {
                    const int w = sc.row_begin + k;
                    const dpos p = reinterpret_cast<const dpos*>(a.pos)[r];
                    const dpos wc = reinterpret_cast<const dpos*>(a.pos)[w];
                    const dpos wn = reinterpret_cast<const dpos*>(a.wall_normal)[w];
                    const double s = wn.x * (p.x - wc.x) + wn.y * (p.y - wc.y) + wn.z * (p.z - wc.z);
                    in = fabs(s) < sc.wall_range;
                }
                // optional exact-outcome filter: pairs the reference's GJK rejects at its first test
                if (in && !(cull && spheres_apart_f(me, c))) sink(r, sc.row_begin + k);
            }
        } else {
            const dpos p = reinterpret_cast<const dpos*>(a.pos)[r];
            for (int k = sc.row_begin; k < sc.wall_end; ++k) {
                const dpos wc = reinterpret_cast<const dpos*>(a.pos)[k];
                const dpos wn = reinterpret_cast<const dpos*>(a.wall_normal)[k];
                double s = wn.x * (p.x - wc.x) + wn.y * (p.y - wc.y) + wn.z * (p.z - wc.z);
                if (!(fabs(s) < sc.wall_range)) continue;
                if (cull) {
                    const float4 pb = make_float4((float)wc.x, (float)wc.y, (float)wc.z, (float)wc.w);
                    if (spheres_apart_f(me, pb)) continue;
                }
                sink(r, k);
            }
        }
    }
    if (!(what & WALK_CELLS)) return;
    auto put = [&](int B, int j) {
        if (cull && spheres_apart_f(me, a.sorted_pos[j])) return;
        sink(r, B);
    };
    // later members of the same cell, in set order
    if (part <= 0) {
        const int ce = cell_range(a, g).y;
        for (int j = t + 1; j < ce; ++j) put(a.sorted[j], j);
    }
    if (part == 0) return;
    // forward neighbours
    const int64_t local = (int64_t)g - sc.cell_base;
    const int64_t nx = sc.nx, nxy = sc.nx * sc.ny;
    if (part > 0) {
        const int64_t l2 = local + forward_offset(part - 1, nx, nxy);
        if (l2 < 0 || l2 >= sc.n_keys) return;
        const int2 se = cell_range(a, (int)(sc.cell_base + l2));
        for (int j = se.x; j < se.y; ++j) put(a.sorted[j], j);
        return;
    }
    // the 7 neighbour ranges are loaded first (independent loads), then walked
    int rs[7], re[7];
#pragma unroll
    for (int o = 0; o < 7; ++o) {
        const int64_t l2 = local + forward_offset(o, nx, nxy);
        rs[o] = re[o] = 0;
        if (l2 < 0 || l2 >= sc.n_keys) continue;
        const int2 se = cell_range(a, (int)(sc.cell_base + l2));
        rs[o] = se.x;
        re[o] = se.y;
    }
#pragma unroll
    for (int o = 0; o < 7; ++o)
        for (int j = rs[o]; j < re[o]; ++j) put(a.sorted[j], j);
}

template <bool EMIT>
__global__ void pairs_kernel(BroadArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_sorted = n_sorted_rows(a);
    if (t >= n_sorted) {
        if (!EMIT && t < a.row_hi - a.row_lo) a.pair_count[t] = 0;
        return;
    }
    const int r = a.sorted[t];
    const int g = a.sorted_cell ? a.sorted_cell[t] : a.cell_of[r];
    const int scene = scene_of(a, r);
    const mwd_scene& sc = a.scenes[scene];
    if (EMIT) {
        int64_t out = a.pair_count[t];
        const int64_t cap = a.pair_cap;
        int2* pairs = reinterpret_cast<int2*>(a.pairs);
        walk_pairs(a, t, r, g, sc, scene, nullptr, [&](int A, int B) {
            if (out < cap) pairs[out] = make_int2(A, B);
            ++out;
        });
    } else {
        int c = 0;
        walk_pairs(a, t, r, g, sc, scene, nullptr, [&](int, int) { ++c; });
        a.pair_count[t] = c;
    }
}

constexpr int APPEND_THREADS = 128;
constexpr int APPEND_KEEP = 8;   // pairs a thread keeps from its walk; threads with more walk again
constexpr int APPEND_PARTS = 8;  // threads per row: walls + own cell, and each forward neighbour cell

// one walk (the first APPEND_KEEP pairs kept in shared memory), reserve (one atomic per warp on
// n_pairs, zeroed by assign_kernel), write.  With walk_parts = APPEND_PARTS each row's walk is split
// over that many threads (its own cell and walls, and one per forward neighbour), so the chain of
// dependent loads per thread is short (a 20k-row step: 72.9 -> 68.7 us); with many rows one thread
// per row does less redundant work (2M rows: 1.33 -> 0.99 ms).  The list order is arbitrary anyway
// in this mode.
__global__ void __launch_bounds__(APPEND_THREADS) pairs_append_kernel(BroadArgs a)
{
    pdl_wait();
    pdl_launch_dependents();
    __shared__ int2 keep[APPEND_KEEP][APPEND_THREADS];
    __shared__ float4 s_wc[WALL_STAGE], s_wn[WALL_STAGE];
    __shared__ float2 s_wm[WALL_STAGE];
    __shared__ int s_scene, s_nw;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = a.walk_parts > 1 ? tid / APPEND_PARTS : tid;
    const int part = a.walk_parts > 1 ? tid % APPEND_PARTS : -1;
    const int n_sorted = n_sorted_rows(a);
    const bool live = t < n_sorted;
    // the walls of the scene of the block's first row, as floats, staged by the first warp alone
    // (its lane 0 finds the scene, its lanes copy one wall each); the other warps walk the cells
    // meanwhile, and every thread tests the walls after one block barrier
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int sc0 = -1, nw = 0;
        const int t0 = blockIdx.x * blockDim.x / (a.walk_parts > 1 ? APPEND_PARTS : 1);
        if (lane == 0 && a.walls && a.sorted_pos && t0 < n_sorted) {
            sc0 = scene_of(a, a.sorted[t0]);
            const mwd_scene& sc = a.scenes[sc0];
            nw = sc.wall_end - sc.row_begin;
            if (nw > WALL_STAGE) sc0 = -1;
        }
        sc0 = __shfl_sync(0xffffffffu, sc0, 0);
        nw = sc0 >= 0 ? __shfl_sync(0xffffffffu, nw, 0) : 0;
        if (lane < nw) {
            const mwd_scene& sc = a.scenes[sc0];
            const int w = sc.row_begin + lane;
            const dpos c = reinterpret_cast<const dpos*>(a.pos)[w];
            const dpos n = reinterpret_cast<const dpos*>(a.wall_normal)[w];
            const float4 cf = make_float4((float)c.x, (float)c.y, (float)c.z, (float)c.w);
            const float4 nf = make_float4((float)n.x, (float)n.y, (float)n.z, 0.f);
            const float n1 = fabsf(nf.x) + fabsf(nf.y) + fabsf(nf.z);
            s_wc[lane] = cf;
            s_wn[lane] = make_float4(nf.x, nf.y, nf.z, nf.x * cf.x + nf.y * cf.y + nf.z * cf.z);
            s_wm[lane] = make_float2(n1, (fabsf(cf.x) + fabsf(cf.y) + fabsf(cf.z)) * n1 + (float)sc.wall_range);
        }
        if (lane == 0) {
            s_scene = sc0;
            s_nw = nw;
        }
    }
    const WallStage ws = {s_wc, s_wn, s_wm, -1, 0};  // scene and count read after the barrier
    int r = 0, g = 0, c = 0, scene = 0;
    const mwd_scene* sc = nullptr;
    auto keep_pair = [&](int A, int B) {
        if (c < APPEND_KEEP) keep[c][threadIdx.x] = make_int2(A, B);
        ++c;
    };
    if (live) {
        r = a.sorted[t];
        g = a.sorted_cell ? a.sorted_cell[t] : a.cell_of[r];
        scene = scene_of(a, r);
        sc = &a.scenes[scene];
        walk_pairs(a, t, r, g, *sc, scene, &ws, keep_pair, part, WALK_CELLS);
    }
    __syncthreads();
    WallStage wst = ws;
    wst.scene = s_scene;
    wst.nw = s_nw;
    if (live) walk_pairs(a, t, r, g, *sc, scene, &wst, keep_pair, part, WALK_WALLS);
    const int lane = threadIdx.x & 31;
    int inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    unsigned long long base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(reinterpret_cast<unsigned long long*>(a.n_pairs), (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (!live || c == 0) return;
    const int64_t out = (int64_t)base + inc - c;
    const int64_t cap = a.pair_cap;
    if (out + c > cap) set_status(a.status, MWD_ST_PAIR_OVERFLOW);
    int2* pairs = reinterpret_cast<int2*>(a.pairs);
    const int kept = c < APPEND_KEEP ? c : APPEND_KEEP;
    for (int i = 0; i < kept; ++i)
        if (out + i < cap) pairs[out + i] = keep[i][threadIdx.x];
    if (c > APPEND_KEEP) {  // the same two walks again, writing the pairs past the kept ones
        int i = 0;
        auto write_rest = [&](int A, int B) {
            if (i >= APPEND_KEEP && out + i < cap) pairs[out + i] = make_int2(A, B);
            ++i;
        };
        walk_pairs(a, t, r, g, *sc, scene, &wst, write_rest, part, WALK_CELLS);
        walk_pairs(a, t, r, g, *sc, scene, &wst, write_rest, part, WALK_WALLS);
    }
}

// wall-major candidates for the reference-layout entry point (MWDiem.py:808-811)
__global__ void wall_flags_kernel(int n_wall, int n_lo, int n_hi, const double* com, const double* wn, const double* wc,
                                  double range, int32_t* flags)
{
    const int64_t np = n_hi - n_lo;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= np * n_wall) return;
    const int k = (int)(t / np);
    const int j = n_lo + (int)(t - (int64_t)k * np);
    double dx = com[3 * j] - wc[3 * k], dy = com[3 * j + 1] - wc[3 * k + 1], dz = com[3 * j + 2] - wc[3 * k + 2];
    double s = wn[3 * k] * dx + wn[3 * k + 1] * dy + wn[3 * k + 2] * dz;
    flags[t] = fabs(s) < range ? 1 : 0;
}

__global__ void wall_emit_kernel(int n_wall, int n_lo, int n_hi, const int32_t* flags, const int32_t* offs,
                                 int32_t* pairs, int64_t cap)
{
    const int64_t np = n_hi - n_lo;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= np * n_wall) return;
    if (offs[t + 1] == offs[t]) return;
    const int k = (int)(t / np);
    const int j = n_lo + (int)(t - (int64_t)k * np);
    const int64_t o = offs[t];
    if (o < cap) reinterpret_cast<int2*>(pairs)[o] = make_int2(j, k);
}

__global__ void keys_kernel(int N, const double* com, double csx, double csy, double csz, int64_t nx, int64_t ny,
                            int64_t* keys)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int64_t xc = (int64_t)(com[3 * i] / csx);
    const int64_t yc = (int64_t)(com[3 * i + 1] / csy);
    const int64_t zc = (int64_t)(com[3 * i + 2] / csz);
    keys[i] = xc + yc * nx + zc * nx * ny;
}

__global__ void minmax_kernel(const int64_t* keys, int lo, int hi, unsigned long long* mm)
{
    // mm[0] = min, mm[1] = max of keys in [lo, hi), as order-preserving unsigned values
    const int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long v_min = ~0ull, v_max = 0ull;
    if (i < hi) {
        unsigned long long u = (unsigned long long)keys[i] ^ 0x8000000000000000ull;
        v_min = v_max = u;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long a = __shfl_xor_sync(0xffffffffu, v_min, o);
        unsigned long long b = __shfl_xor_sync(0xffffffffu, v_max, o);
        v_min = a < v_min ? a : v_min;
        v_max = b > v_max ? b : v_max;
    }
    if ((threadIdx.x & 31) == 0 && i - (int)(threadIdx.x & 31) < hi) {
        atomicMin(mm, v_min);
        atomicMax(mm + 1, v_max);
    }
}

inline unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// block totals of a scan of n elements, then (device-resident broad phase) as many persistent
// per-tile cell counts
int64_t scan_tmp_ints(int64_t n) { return 2 * ((n + SCAN_TILE - 1) / SCAN_TILE + 2); }
int64_t scan_tile_sums_offset(int64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 2; }

int launch_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* tmp, int64_t* total_out, int64_t cap,
                uint32_t* status, uint32_t overflow_bit, cudaStream_t s)
{
    if (n <= SCAN_SMALL_MAX) {
        MWD_CUDA(launch_pdl(scan_small_kernel, 1, SCAN_SMALL_THREADS, 0, s, in, n, out, total_out, cap, status,
                            overflow_bit));
        return MWD_OK;
    }
    const int nb = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
    const int nbl = nb > 0 ? nb : 1;
    MWD_CUDA(launch_pdl(scan_reduce_kernel, nbl, SCAN_THREADS, 0, s, in, n, tmp));
    MWD_CUDA(launch_pdl(scan_final_kernel<false>, nbl, SCAN_THREADS, 0, s, in, n, tmp, out, nbl, total_out, cap,
                        status, overflow_bit, aligned16(in, out), (int32_t*)nullptr));
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

namespace {
struct SparseLayout {
    int64_t n_words, words_pad, compact_len;
};
SparseLayout sparse_layout(int64_t rows, int64_t total_cells)
{
    SparseLayout L;
    L.n_words = (total_cells + 31) / 32;
    L.words_pad = (L.n_words + 1 + 3) / 4 * 4;
    L.compact_len = (rows + 1 + 3) / 4 * 4;
    return L;
}
}  // namespace

int broad_sparse(int64_t rows, int64_t total_cells, int64_t tile_sum_ints, int mode)
{
    // automatic: the dense table up to 2^27 cells (1 GB of count and start arrays), the compressed one
    // beyond where it fits.  On 256 batched scenes (2.0M rows, 15.2M cells) the compressed table
    // measured slower (broad phase 0.263 vs 0.229 ms): its lower atomic and scan traffic does not pay for
    // the extra level of dependent loads (bit word and rank before each range) in the place and append
    // passes and its two more launches; on a sparse domain it takes a fraction of the memory.
    if (mode == 1 || tile_sum_ints <= 0 || rows <= 0) return 0;
    if (mode == 0 && total_cells <= ((int64_t)1 << 27)) return 0;
    if (total_cells < 4 * rows + 4096 || total_cells > INT32_MAX - 64) return 0;
    const SparseLayout L = sparse_layout(rows, total_cells);
    // the carved arrays fit in cell_count (total_cells ints) and cell_start (total_cells + 1)
    if (L.words_pad + L.compact_len > total_cells || 2 * L.words_pad + L.compact_len + 1 > total_cells + 1) return 0;
    // and the tile totals of both scans in the tile-sum area
    const int64_t tiles = (L.n_words + SCAN_TILE - 1) / SCAN_TILE + 1 + (L.compact_len + SCAN_TILE - 1) / SCAN_TILE + 1;
    return tiles <= tile_sum_ints ? 1 : 0;
}

void broad_table_ints(int64_t rows, int64_t total_cells, int sparse, int64_t* count_ints, int64_t* start_ints)
{
    if (sparse) {
        const SparseLayout L = sparse_layout(rows, total_cells);
        *count_ints = L.words_pad + L.compact_len;
        *start_ints = 2 * L.words_pad + L.compact_len + 1;
    } else {
        *count_ints = total_cells > 0 ? total_cells : 1;
        *start_ints = total_cells + 1;
    }
}

int launch_broad(const BroadArgs& a_in, cudaStream_t s)
{
    const int T = 128;  // row kernels: 20k rows already span every SM
    BroadArgs a = a_in;
    const int64_t rows = a.row_hi - a.row_lo;
    if (rows <= 0 || a.total_cells <= 0) {
        MWD_CUDA(cudaMemsetAsync(a.n_pairs, 0, sizeof(int64_t), s));
        return MWD_OK;
    }
    if (a.sparse) {
        if (!a.tile_sums) return MWD_ERR_INVALID;
        const SparseLayout L = sparse_layout(rows, a.total_cells);
        a.n_words = (int32_t)L.n_words;
        a.words_pad = (int32_t)L.words_pad;
        a.compact_len = (int32_t)L.compact_len;
    }
    MWD_CUDA(launch_pdl(assign_kernel, blocks(rows, T), T, 0, s, a));
    int rc = MWD_OK;
    if (a.sparse) {
        // the bitmap's scan (ranks of the occupied cells, a copy of the bits, the bits zeroed), the rows
        // per occupied cell, their scan
        const int nbw = (a.n_words + SCAN_TILE - 1) / SCAN_TILE;
        int32_t* copy = a.cell_start + a.words_pad;
        MWD_CUDA(launch_pdl(scan_final_kernel<true>, nbw, SCAN_THREADS, 0, s, (const int32_t*)a.cell_count,
                            (int64_t)a.n_words, (const int32_t*)a.tile_sums, a.cell_start, nbw, (int64_t*)nullptr,
                            (int64_t)INT64_MAX, (uint32_t*)nullptr, 0u,
                            aligned16(a.cell_count, a.cell_start) & aligned16(copy, copy), copy));
        MWD_CUDA(launch_pdl(occ_count_kernel, blocks(rows, T), T, 0, s, a));
        const int nbc = (a.compact_len + SCAN_TILE - 1) / SCAN_TILE;
        int32_t* cnt = a.cell_count + a.words_pad;
        int32_t* start = a.cell_start + 2 * a.words_pad;
        MWD_CUDA(launch_pdl(scan_final_kernel<false>, nbc, SCAN_THREADS, 0, s, (const int32_t*)cnt,
                            (int64_t)a.compact_len, (const int32_t*)(a.tile_sums + nbw + 1), start, nbc,
                            (int64_t*)nullptr, (int64_t)INT64_MAX, (uint32_t*)nullptr, 0u, aligned16(cnt, start),
                            (int32_t*)nullptr));
    } else if (a.tile_sums && a.total_cells > SCAN_SMALL_MAX) {
        // the tile totals were added up by assign_kernel: only the final pass of the scan remains (each
        // block adds up the totals of the tiles before it; turning them into prefixes in a separate
        // one-block pass first measured no faster with 7,300 tiles)
        const int nb = (int)((a.total_cells + SCAN_TILE - 1) / SCAN_TILE);
        MWD_CUDA(launch_pdl(scan_final_kernel<false>, nb, SCAN_THREADS, 0, s, (const int32_t*)a.cell_count,
                            a.total_cells, (const int32_t*)a.tile_sums, a.cell_start, nb, (int64_t*)nullptr,
                            (int64_t)INT64_MAX, (uint32_t*)nullptr, 0u, aligned16(a.cell_count, a.cell_start),
                            (int32_t*)nullptr));
    } else {
        rc = launch_scan(a.cell_count, a.total_cells, a.cell_start, a.scan_tmp, nullptr, INT64_MAX, nullptr, 0, s);
        if (rc) return rc;
    }
    // the two-member exchange path from two full waves of place blocks up (a 256-scene batch of 2M
    // rows: broad phase 0.221 -> 0.211 ms; a 20k-row pour is 1-2 us slower with it)
    if (rows >= 2 * (int64_t)num_sms() * (2048 / PLACE_THREADS) * PLACE_THREADS)
        MWD_CUDA(launch_pdl(place_kernel<true>, blocks(rows, PLACE_THREADS), PLACE_THREADS, 0, s, a));
    else
        MWD_CUDA(launch_pdl(place_kernel<false>, blocks(rows, PLACE_THREADS), PLACE_THREADS, 0, s, a));
    // rows that have a cell are at most `rows`; threads past cell_start[total] exit
    if (a.append) {
        // split each row's walk over APPEND_PARTS threads while the rows alone leave the GPU short of
        // threads (a latency-bound step); with many rows one thread per row does less redundant work
        BroadArgs b = a;
        const int64_t resident = (int64_t)num_sms() * 2048;
        b.walk_parts = rows * APPEND_PARTS <= 4 * resident ? APPEND_PARTS : 1;
        MWD_CUDA(launch_pdl(pairs_append_kernel, blocks(rows * b.walk_parts, APPEND_THREADS), APPEND_THREADS, 0, s,
                            b));
        MWD_CUDA(cudaGetLastError());
        return MWD_OK;
    }
    pairs_kernel<false><<<blocks(rows, T), T, 0, s>>>(a);
    rc = launch_scan(a.pair_count, rows, a.pair_count, a.scan_tmp, a.n_pairs, a.pair_cap, a.status,
                     MWD_ST_PAIR_OVERFLOW, s);
    if (rc) return rc;
    pairs_kernel<true><<<blocks(rows, T), T, 0, s>>>(a);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

int launch_keys(int N, const double* com, double csx, double csy, double csz, int64_t nx, int64_t ny, int64_t* keys,
                cudaStream_t s)
{
    if (N <= 0) return MWD_OK;
    keys_kernel<<<blocks(N, 256), 256, 0, s>>>(N, com, csx, csy, csz, nx, ny, keys);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

int launch_minmax(const int64_t* keys, int lo, int hi, unsigned long long* mm, cudaStream_t s)
{
    if (hi <= lo) return MWD_OK;
    minmax_kernel<<<blocks(hi - lo, 256), 256, 0, s>>>(keys, lo, hi, mm);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

int launch_wall_pairs(int n_wall, int n_lo, int n_hi, const double* com, const double* wn, const double* wc,
                      double range, int32_t* flags, int32_t* offs, int32_t* tmp, int32_t* pairs, int64_t cap,
                      int64_t* n_out, uint32_t* status, cudaStream_t s)
{
    const int64_t total = (int64_t)n_wall * (n_hi - n_lo);
    if (total <= 0) {
        MWD_CUDA(cudaMemsetAsync(n_out, 0, sizeof(int64_t), s));
        return MWD_OK;
    }
    wall_flags_kernel<<<blocks(total, 256), 256, 0, s>>>(n_wall, n_lo, n_hi, com, wn, wc, range, flags);
    int rc = launch_scan(flags, total, offs, tmp, n_out, cap, status, MWD_ST_PAIR_OVERFLOW, s);
    if (rc) return rc;
    wall_emit_kernel<<<blocks(total, 256), 256, 0, s>>>(n_wall, n_lo, n_hi, flags, offs, pairs, cap);
    MWD_CUDA(cudaGetLastError());
    return MWD_OK;
}

}  // namespace mwd
