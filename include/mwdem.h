/* mwdem.h -- C ABI of libmwdem.so, the GB300 (sm_103a) implementation of MWDiEM's per-step DEM
 * hot path: cell-hash broad phase, GJK/EPA narrow phase, spring-dashpot + Coulomb contact force,
 * quaternion leapfrog integrator.
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless its comment says "host".
 *  - Every entry point returns 0 (MWD_OK) or a positive MWD_ERR_* code and never aborts or traps.
 *    mwd_last_error() returns a one-line description of the last failure on the calling thread.
 *  - Kernels report data-dependent conditions (EPA did not converge, capacity exceeded, ...) by
 *    OR-ing MWD_ST_* bits into an optional device status word; the host reads it when it wants.
 *  - Work is enqueued on the given stream; nothing synchronises unless the comment says so.
 *  - Array layouts of the "reference layout" entry points are exactly the numpy arrays the
 *    reference passes to pycuda (row-major, float32 / int32 / float64 as noted).
 */
#ifndef MWDEM_H
#define MWDEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* mwd_stream_t; /* == cudaStream_t */

enum {
    MWD_OK = 0,
    MWD_ERR_INVALID = 1,     /* bad argument (null pointer, size out of range, ...) */
    MWD_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    MWD_ERR_UNSUPPORTED = 3, /* valid but unsupported (e.g. more hull vertices than the kernel stages) */
    MWD_ERR_NOMEM = 4        /* device allocation of library scratch failed */
};

/* device status bits */
enum {
    MWD_ST_EPA_NOCONV = 1u,     /* EPA hit the reference's iteration cap (gpu_fine_contact_detection.cu:443-446) */
    MWD_ST_EPA_OVERFLOW = 2u,   /* EPA needed more polytope faces/vertices than MWD_EPA_FACE_CAP */
    MWD_ST_GJK_NOCONV = 4u,     /* GJK ran 50 tetrahedron iterations without a decision (.cu:1104) */
    MWD_ST_PAIR_OVERFLOW = 8u,  /* broad phase produced more candidate pairs than the pair buffer holds */
    MWD_ST_CELL_RANGE = 16u,    /* a centre's cell key fell outside the scene's dense cell table */
    MWD_ST_CELL_CROWDED = 32u,  /* a cell held more members than the set-order emulation supports */
    MWD_ST_BAD_SHAPE = 64u,     /* a hull with more vertices than the staging capacity */
    MWD_ST_DEGENERATE_FACE = 128u, /* differentiable step: a logged contact face of zero area (skipped) */
    MWD_ST_LOG_OVERFLOW = 256u,    /* differentiable step: more contacts than the topology log holds */
    MWD_ST_FLY_RESET = 512u,       /* differentiable step: a particle left the box and was stopped */
    MWD_ST_HIST_OVERFLOW = 1024u   /* persistent history: more contacts than the history table holds */
};

#define MWD_EPA_FACE_CAP 128   /* EPA faces per pair, deleted ones included as in the reference (a pair
                                  that needs more runs again with the deleted faces removed) */
#define MWD_EPA_COUNT_INTS 256 /* ints of mwd_work.epa_count */
#define MWD_EPA_VERT_CAP 32    /* EPA polytope vertices per pair (4 + 25 iterations + 1) */
#define MWD_HULL_CAP 64        /* hull vertices per side staged in shared memory */
#define MWD_CELL_CAP 306       /* members per cell handled by the CPython set-order emulation */

/* ------------------------------------------------------------------------------------------
 * Contact law.  The reference bakes these into its kernel source as literals
 * (gpu_fine_contact_detection.py:92-103); here they are a POD argument.  mu is both the effective
 * mass in tc/Gn/Kt/Gt and the Coulomb coefficient, as in the reference (.cu:690-693, .cu:774-788).
 * ------------------------------------------------------------------------------------------ */
typedef struct {
    double Kn, en, et, mu;                     /* particle-particle */
    double Kn_wall, en_wall, et_wall, mu_wall; /* particle-wall */
    double dt;                                 /* timestep used in the history update */
    int32_t n_wall;    /* ids < n_wall are walls (num_particles_wall) */
    int32_t hist_mode; /* 0: the reference's stride-1 history indexing (.cu:974-976); 1: stride 4 */
    int32_t lanes;     /* lanes per pair in the narrow phase: 4, 8, 16, 32; 0 = default (8) */
    int32_t deterministic; /* 1: per-particle sums in pair order instead of float atomics */
    int32_t law;       /* MWD_LAW_REFERENCE (the reference's law as written) or MWD_LAW_PHYSICAL */
    int32_t pad;
} mwd_contact_params;

/* Contact laws.  MWD_LAW_REFERENCE reproduces .cu:647-871 as written: mu stands in for the effective
 * mass in tc, Gn, Kt and Gt, and the contact point is (cpA - cpB) / 2, which puts the torque arm near
 * -c_A.  MWD_LAW_PHYSICAL (device-resident step only) is the same linear spring-dashpot law with
 *   m_n = 1 / (1/m_A + 1/m_B)                         normal effective mass (a wall's 1/m is 0)
 *   m_t = 1 / (1/m_A + 1/m_B + dA^2/I_A + dB^2/I_B)   tangential effective mass (a wall adds no term)
 *   tc = sqrt(m_n (pi^2 + ln^2 en) / Kn),  Gn = -2 m_n ln en / tc
 *   Kt = m_t (pi^2 + ln^2 et) / tc^2,      Gt = -2 m_t ln et / tc
 * and the contact point (cpA + cpB) / 2, so a normal impact of two bodies rebounds with restitution
 * en whatever their masses; mu is only the Coulomb coefficient.  I is the inertia size (trace / 3),
 * as in the reference's tangential term. */
#define MWD_LAW_REFERENCE 0
#define MWD_LAW_PHYSICAL 1

/* Per-material constants of the contact law that do not depend on the pair, derived once on the
 * host from mwd_contact_params with the same float/double operand types the reference uses
 * (.cu:685-701): tc = sqrt(mu (pi^2 + ln^2 en) / Kn), Gn = -2 mu / tc ln en,
 * KtA = Kn (pi^2 + ln^2 et) / (pi^2 + ln^2 en).  Per pair the kernel finishes
 * Kt = KtA / (1/mu + dA^2/IsA + dB^2/IsB) and Gt = -2 / (...) ln et. */
typedef struct {
    float Kn_f;   /* (float)Kn */
    float mu_f;   /* (float)mu */
    float Gn;     /* normal damping */
    float ln_et;  /* logf((float)et) */
    float dt_f;   /* (float)dt */
    float ln_en;  /* logf((float)en) */
    float Xn;     /* pi^2 + ln^2 en (float) */
    float Xt;     /* pi^2 + ln^2 et (float) */
    double mu;    /* mu as a double (Coulomb test is done in double, .cu:774) */
    double inv_mu;
    double KtA;
    int32_t physical; /* MWD_LAW_PHYSICAL: tc, Gn, Kt, Gt per pair from the masses (see above) */
    float inv_mu_hi, inv_mu_lo; /* inv_mu as a float pair: hi = (float)inv_mu, lo = (float)(inv_mu - hi) */
    float KtA_hi, KtA_lo;       /* KtA likewise (the kernel's float-float evaluation of Kt and Gt) */
    int32_t pad;
} mwd_material;

/* Fills m[0] (particle-particle) and m[1] (particle-wall) from prm (host pointers). */
int mwd_derive_material(const mwd_contact_params* prm, mwd_material m[2]);

/* Narrow phase + contact force over per-pair arrays in the reference's layout.
 *
 * Replaces gpu_fine_contact_detection.gpu_contact_detection / contact_detection
 * (LIBRARIES/gpu_fine_contact_detection.py:18-73, LIBRARIES/gpu_fine_contact_detection.cu:874-1322).
 * Inputs (P = n_pairs, V = num_vertices_max, N = particles):
 *   A_com, B_com (P,3) f32; A_verts, B_verts (P,V,3) f32 world-frame, zero padded;
 *   A_vel, B_vel, A_angvel, B_angvel (P,3) f32; A_nv, B_nv, A_id, B_id (P,) i32;
 *   qA, qB (P,4) f32; IsA, IsB (P,) f32 (moment_of_inertia_size).
 * In/out: hist (P,4) f32 tangential history; force, torque (N,3) f32, accumulated into.
 * Out: collision (P,) i32 in {-1, 0, 1}.
 * Optional (may be NULL): diag (P,10) f32 = depth, normal(3), cpA(3), cpB(3) of colliding pairs;
 *   status (1,) u32 device status word (OR-ed).
 * Uses library-owned scratch (allocated on first use per device and kept). */
int mwd_contact_pairs(int64_t n_pairs, int32_t V, int32_t n_particles,
                      const float* A_com, const float* B_com, const float* A_verts, const float* B_verts,
                      const float* A_vel, const float* B_vel, const float* A_angvel, const float* B_angvel,
                      const int32_t* A_nv, const int32_t* B_nv, const int32_t* A_id, const int32_t* B_id,
                      float* hist, float* force, float* torque, const float* qA, const float* qB,
                      const float* IsA, const float* IsB, int32_t* collision,
                      const mwd_contact_params* prm /* host */, float* diag, uint32_t* status,
                      mwd_stream_t stream);

/* The same narrow phase + contact force as mwd_contact_pairs, same arguments and results, for
 * callers that cannot let this library allocate device memory: a host application whose own
 * allocator owns (nearly) all of the GPU's memory, so that a cudaMalloc from inside the library
 * would fail or bypass its accounting; a process given a fixed slice of device memory up front; and
 * a loop that cannot take the device-wide stall of the cudaFree that mwd_contact_pairs makes when
 * its scratch grows.  No counterpart in the reference (which allocates and copies on every call).
 * Its scratch (17 bytes per pair, for the stride-1 history staging) is a fixed array compiled into
 * the library, 4,456,448 bytes (4.25 MiB): at most MWD_NOALLOC_MAX_PAIRS pairs per call (larger calls
 * return MWD_ERR_INVALID); every GPU that loads the library holds the array until the process exits;
 * all calls share it and it keeps the last call's contents, so calls that overlap on the GPU race
 * and must be ordered by the caller.  The first call on a device looks up the array's address with
 * that device current; make that first call before any stream capture.  Calls no cudaMalloc,
 * cudaFree or other allocating routine. */
#define MWD_NOALLOC_MAX_PAIRS (1 << 18)
int mwd_contact_pairs_noalloc(int64_t n_pairs, int32_t V, int32_t n_particles,
                              const float* A_com, const float* B_com, const float* A_verts, const float* B_verts,
                              const float* A_vel, const float* B_vel, const float* A_angvel, const float* B_angvel,
                              const int32_t* A_nv, const int32_t* B_nv, const int32_t* A_id, const int32_t* B_id,
                              float* hist, float* force, float* torque, const float* qA, const float* qB,
                              const float* IsA, const float* IsB, int32_t* collision,
                              const mwd_contact_params* prm /* host */, float* diag, uint32_t* status,
                              mwd_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Integrator over the reference's FP64 arrays.
 * Replaces gpu_Verlet.gpu_Verlett / Verlet (LIBRARIES/gpu_Verlet.py:18-50, gpu_Verlet.cu:85-431).
 * ------------------------------------------------------------------------------------------ */
typedef struct {
    double dt;
    double box[6];   /* syssize x_max, x_min, y_max, y_min, z_max, z_min (fly-away box) */
    int32_t n_min;   /* num_part_min: first integrated row */
    int32_t n_max;   /* num_part_max: one past the last integrated row */
    int32_t V;       /* num_vertices_max */
    int32_t pad;
} mwd_verlet_params;

/* Arrays (N rows): v, v12, w12bf, wbf, w, F, T, com, dxall (N,3); q12, q, qall (N,4);
 * verts (N,V,3); mass (N,); Iinv, I (N,3,3); all float64, updated in place like pycuda's InOut.
 * n_reset (optional, device int32) receives the number of fly-away resets (added to). */
int mwd_verlet_ref(int32_t N, double* v, double* v12, double* w12bf, double* q12, double* q,
                   double* qall, double* wbf, double* w, const double* F, const double* T,
                   double* verts, double* com, const double* mass, const double* Iinv,
                   const double* I, double* dxall, const mwd_verlet_params* prm /* host */,
                   int32_t* n_reset, mwd_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Broad phase pieces in the reference's representation.
 * ------------------------------------------------------------------------------------------ */

/* key[i] = trunc(com_x/csx) + trunc(com_y/csy)*nx + trunc(com_z/csz)*nx*ny for i < N (FP64 divide,
 * truncation toward zero as numpy's astype(int)).  Replaces MWDiem.py:813-816. */
int mwd_cell_keys(int32_t N, const double* com, double csx, double csy, double csz, int64_t nx,
                  int64_t ny, int64_t* keys, mwd_stream_t stream);

/* Wall candidates: for walls k < n_wall and particles j in [n_lo, n_hi), emit [j, k] when
 * |n_k . (c_j - c_k)| < range, ordered wall-major like MWDiem.py:808-811.
 * pairs (cap,2) i32; n_out (device int64) receives the total (may exceed cap -> MWD_ST_PAIR_OVERFLOW). */
int mwd_wall_pairs(int32_t n_wall, int32_t n_lo, int32_t n_hi, const double* com,
                   const double* wall_normal, const double* wall_center, double range,
                   int32_t* pairs, int64_t cap, int64_t* n_out, uint32_t* status, mwd_stream_t stream);

/* Cell candidates.  Replaces LIBRARY_Coarse_contact_detection.Linked_cell_hash
 * (LIBRARIES/LIBRARY_Coarse_contact_detection.py:84-155): ids [n_lo, n_hi) grouped by keys[id];
 * same-cell pairs oriented in CPython set iteration order, cross-cell pairs for the offsets
 * +1, +nx, +nx*ny, +nx*ny+1, +nx*ny+1+nx, +nx*ny+nx, +nx+1 with A from the lower-offset cell.
 * The emitted SET of oriented pairs equals the reference list; the list order is by cell.
 * keys: (n_hi,) i64 (rows below n_lo ignored).  pairs (cap,2) i32; n_out device int64 (total).
 * A key range (max - min + 1) up to 2^28 cells takes a dense cell table; wider ranges, up to 2^31
 * cells with at most about a quarter as many ids, the occupancy-compressed one (MWD_ERR_UNSUPPORTED
 * beyond). */
int mwd_linked_cell_hash(int32_t n_lo, int32_t n_hi, const int64_t* keys, int64_t nx, int64_t ny,
                         int32_t* pairs, int64_t cap, int64_t* n_out, uint32_t* status,
                         mwd_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Device-resident simulation (the GB300-native step).  State lives in HBM as structure-of-arrays
 * of float4 (FP32) with FP64 centres; shapes are body-frame vertex tables addressed through a CSR
 * offset per particle; several independent scenes can share one set of arrays ("batched").
 * A step = broad phase -> narrow phase + force -> integrator, all on one stream, no host sync,
 * capturable in a CUDA graph.  Replaces the per-step body of MWDiem.py:671-1001.
 * ------------------------------------------------------------------------------------------ */
typedef struct {
    /* per particle row (n rows) */
    double* pos;         /* (n,4) centre of mass, FP64; .w = bounding radius (largest |r0|) of the row */
    double* dx_all;      /* (n,4) displacement accumulated since the last host sync */
    float* vel;          /* (n,4) v */
    float* vel_half;     /* (n,4) v_1/2 */
    float* w_half_bf;    /* (n,4) omega_1/2, body frame */
    float* w_bf;         /* (n,4) omega, body frame */
    float* w;            /* (n,4) omega, world frame */
    float* q;            /* (n,4) orientation (w,x,y,z) at the full step */
    float* q_half;       /* (n,4) orientation at the half step */
    float* q_all;        /* (n,4) rotation accumulated since the last host sync */
    float* q_acc;        /* (n,4) rotation applied to the body-frame vertices (world = pos + R(q_acc) r0) */
    float* force;        /* (n,4) contact force accumulator (zeroed by the integrator) */
    float* torque;       /* (n,4) contact torque accumulator (zeroed by the integrator) */
    const float* ext_force;  /* (n,4) external force, e.g. mass * g (MWDiem.py:980) */
    const float* ext_torque; /* (n,4) external torque */
    const float* inertia;    /* (n,4) body-frame principal moments Ixx, Iyy, Izz, inertia size */
    const float* inv_inertia;/* (n,4) 1/Ixx, 1/Iyy, 1/Izz, 1/mass */
    const int32_t* info;     /* (n,) scene id << 1 | is_wall */
    const double* wall_normal; /* (n,4) plane normal of wall rows (unused for particles) */
    const int32_t* vert_off; /* (n+1,) CSR offsets into the vertex tables */
    const float* body_verts; /* (nv,4) body-frame vertices r0 */
    float* world_verts;      /* (nv,4) world-frame vertices, rewritten by the integrator */
    int32_t n;
    int32_t n_verts;
    int32_t max_verts;       /* largest vertex count of any row (<= MWD_HULL_CAP) */
    int32_t pad;
    const int32_t* vert_owner; /* optional (nv,) row of each vertex; with xform the integrator rewrites
                                  the world vertices one thread per vertex up to the row count
                                  mwd_integrate_kernels gives 1 for (NULL, or above it: one block per
                                  128 rows and their vertices) */
    float* xform;            /* optional (n,16) scratch: R(q_acc) row-major, then the centre as float
                                hi + lo per axis */
} mwd_state;

typedef struct {
    double cs[3];        /* cell size x, y, z */
    double box[6];       /* fly-away box x_max, x_min, y_max, y_min, z_max, z_min */
    double dt;
    double wall_range;   /* 6 * max_particlesize (MWDiem.py:810) */
    int64_t nx, ny;      /* cells per row / per layer (key = xc + yc nx + zc nx ny) */
    int64_t key_min;     /* smallest key of the dense cell table */
    int64_t n_keys;      /* dense table length (key_max - key_min + 1) */
    int64_t cell_base;   /* offset of this scene's table in the global cell arrays */
    int32_t row_begin, wall_end, row_end, pad; /* rows [row_begin, wall_end) are walls */
    mwd_contact_params law; /* contact law of the scene */
    mwd_material mat[2];    /* derived from law by mwd_derive_material (particle, wall) */
    float inv_cs[3];        /* optional (float)(1 / cs): cell coordinates from a float quotient away
                               from cell boundaries (0: always the FP64 division) */
    int32_t pad2;
} mwd_scene;

/* Particle inlet (MWDiem.py:685-714: every few steps new hulls enter the domain).  Every row is
 * allocated with its shape up front; rows waiting to enter carry MWD_INFO_INACTIVE in mwd_state.info
 * and are skipped by the broad phase and the integrator.  mwd_inlet_step, run at the start of a step
 * (mwd_step does when mwd_work.inlet is set), counts steps on the device and every `period` steps
 * activates the next `per_spawn` rows: centre from spawn_pos, at rest, identity orientation, world
 * vertices written.  The captured graph of a step stays valid as rows enter. */
#define MWD_INFO_INACTIVE (1 << 30)
typedef struct {
    int32_t period;          /* steps between spawns (> 0) */
    int32_t per_spawn;       /* rows activated per spawn */
    int32_t row_end;         /* rows [*next_row, row_end) are waiting */
    int32_t pad;
    int32_t* next_row;       /* (1,) device: next row to activate */
    int32_t* step;           /* (1,) device: steps seen (spawns when step % period == 0) */
    const double* spawn_pos; /* (n,4) centre of each row when it enters (.w unused) */
} mwd_inlet;

int mwd_inlet_step(mwd_state* st, const mwd_inlet* inlet, mwd_stream_t stream);

typedef struct {
    int32_t* cell_count;   /* (total_cells,) zero on entry, left zero on exit; with cell_table = 2 the
                              count mwd_cell_table_ints gives suffices */
    int32_t* cell_start;   /* (total_cells + 1,), or with cell_table = 2 mwd_cell_table_ints's count */
    int32_t* cell_of;      /* (n,) global cell of each row, -1 for walls */
    int32_t* sorted;       /* (n,) rows ordered by cell, members in CPython set order */
    int32_t* pair_count;   /* (n + 1,) per-row candidate counts, then their exclusive scan */
    int32_t* pairs;        /* (pair_cap, 2) candidate pairs A, B */
    int32_t* scan_tmp;     /* scan scratch, mwd_scan_tmp_ints(max(total_cells, n) + 1) ints */
    int64_t* n_pairs;      /* (1,) candidate count of the last broad phase */
    uint32_t* status;      /* (1,) status word */
    int32_t* collision;    /* (pair_cap,) optional contact flags (NULL to skip) */
    uint64_t* work_counters; /* optional (3,), added to by the narrow phase: vertex dot products of the
                              support queries, EPA faces created, support queries (NULL: not counted) */
    int32_t* epa_count;    /* (MWD_EPA_COUNT_INTS,) 8-byte aligned, two-pass narrow phase: [0] pairs found in
                              contact by the GJK pass, [2..3] the EPA pass's work queue (uint64), [4] and
                              [8..] the records whose EPA face list overflowed (run again after the
                              pass); [0..7] are zeroed by the broad phase of mwd_step, or by
                              mwd_narrow_force when it runs alone */
    void* epa_rec;         /* (epa_cap, 80 B): their simplex; NULL selects the single-pass kernel */
    int64_t epa_cap;
    float* sorted_pos;     /* (n,4) centre and radius of each row in cell order (used with cull_pairs) */
    int32_t* sorted_cell;  /* (n,) cell of each row in cell order (used with cull_pairs) */
    int32_t cull_pairs;    /* 1: the broad phase lists only pairs whose bounding spheres (pos.w) overlap
                              within a rounding margin -- the others are exactly the candidates the
                              reference's first GJK test rejects; 0: the reference's full candidate list */
    int32_t cell_table;    /* layout of cell_count / cell_start: 0 automatic (dense up to 2^27 cells,
                              compressed beyond where it fits), 1 dense (a count and a start per cell),
                              2 occupancy-compressed where it fits (a bit per cell, counts and starts
                              per occupied cell, carved out of the same two arrays; needs total_cells >=
                              4 n + 4096).  The same pairs either way. */
    int64_t total_cells;
    int64_t pair_cap;
    int32_t* face_ids;     /* optional (pair_cap, 6): support-vertex indices (into each row's vertex table)
                              of the final EPA face, A's three then B's, written where collision is 1 */
    int32_t deterministic; /* 1: the pair list is built in cell order and each particle's force and torque
                              are summed in pair-list order (as a serial loop over the pairs adds them)
                              instead of with float atomics; needs epa_rec and det_scratch */
    int32_t pad2;
    void* det_scratch;     /* (mwd_det_scratch_bytes(n, epa_cap),) zeroed before the first step */
    /* Persistent tangential history (optional; needs epa_rec).  The reference drops every stored
     * history each step (MWDiem.py:953-966), so its contacts always start from zero.  With these set,
     * the history of each pair in contact is kept from step to step in a device hash table keyed by
     * the unordered pair: two tables of hist_cap (a power of two) entries, read *hist_parity and
     * written the other, the roles swapping every narrow phase.  Values are the tangential
     * displacement in the (lower id, higher id) orientation. */
    int64_t hist_cap;
    unsigned long long* hist_keys; /* (2, hist_cap) min id << 32 | max id, 0 = empty; zeroed before use */
    float* hist_vals;              /* (2, hist_cap, 4) */
    int32_t* hist_parity;          /* (1,) */
    const mwd_inlet* inlet;        /* optional (host pointer): mwd_step runs mwd_inlet_step first */
} mwd_work;


/* Scratch bytes of the deterministic accumulation for n rows and epa_cap contacts. */
int64_t mwd_det_scratch_bytes(int32_t n, int64_t epa_cap);

/* Scratch ints the device-wide scans need for arrays of n elements: the block totals of a scan, and
 * as many again for the per-tile cell counts the device-resident broad phase keeps between its
 * assign pass and its cell scan (zero on entry and on exit; allocate zeroed). */
int64_t mwd_scan_tmp_ints(int64_t n);

/* Kernels mwd_integrate launches for n rows of a state with vert_owner and xform: 2 (the row pass,
 * then one thread per vertex) or 1 (each block's rows, then their vertices: from two full waves of
 * blocks up, where the transforms' and vertex owners' trips through memory cost more than the
 * vertex pass's spread).  In the one-kernel case st->xform is not written and mwd_step runs its steps
 * without the vertex pass overlap.  Host utility; no reference counterpart. */
int32_t mwd_integrate_kernels(int64_t n);

/* The cell table mwd_broadphase uses for n rows, total_cells cells and mwd_work.cell_table = mode:
 * 1 dense, 2 occupancy-compressed.  Host utility; no reference counterpart. */
int32_t mwd_cell_table(int64_t n, int64_t total_cells, int32_t mode);

/* mwd_cell_table, and the ints mwd_work.cell_count and cell_start need for that table: total_cells
 * and total_cells + 1 for the dense one; for the compressed one a bit per cell (three copies) and a
 * count and a start per row, a small fraction of the dense table's size on a sparse domain. */
int32_t mwd_cell_table_ints(int64_t n, int64_t total_cells, int32_t mode, int64_t* count_ints, int64_t* start_ints);

/* One broad phase over all scenes (rows of every scene; walls excluded from the cell hash). */
int mwd_broadphase(const mwd_state* st, const mwd_scene* scenes_dev, const mwd_scene* scenes_host,
                   int32_t n_scenes, mwd_work* work, mwd_stream_t stream);

/* Narrow phase + force over work->pairs[0 .. *work->n_pairs) into st->force/torque.
 * lanes: lanes per pair of the GJK pass (1 with the two-pass kernel, 4, 8, 16, 32), plus, in bits
 * 8-15, those of the EPA pass of the two-pass kernel (0: the same); bit 16 set: the EPA pass reads
 * the hulls in place from the vertex table instead of staging them in shared memory (less shared
 * memory, more resident pairs); bits 20-21 and 22-23: threads per block of the GJK and EPA passes
 * of the two-pass kernel (0: 128, 1: 64, 2: 256). */
#define MWD_LANES_EPA_IN_PLACE (1 << 16)
#define MWD_LANES_GJK_BLOCK_SHIFT 20
#define MWD_LANES_EPA_BLOCK_SHIFT 22
int mwd_narrow_force(const mwd_state* st, const mwd_scene* scenes_dev, mwd_work* work,
                     int32_t lanes, mwd_stream_t stream);

/* Integrator over every non-wall row: consumes force/torque (+ external), updates the state,
 * rewrites world_verts, zeroes force/torque. */
int mwd_integrate(mwd_state* st, const mwd_scene* scenes_dev, uint32_t* status, mwd_stream_t stream);

/* The integrator's row pass (mwd_integrate_rows) that also writes every state array it updates --
 * pos, dx_all, vel, vel_half, w_half_bf, w_bf, w, q, q_half, q_all, q_acc -- into `mirror`, a copy of
 * the memory block `block` (block_bytes long, holding all of those arrays) in page-locked host memory
 * the GPU can address (mwd_host_mapped), at the same offsets.  No reference counterpart: for a
 * caller that keeps its state in host memory, as the reference's loop does (MWDiem.py:986-1001), the
 * state returns to the host during the pass instead of by a copy after it.  Rows the pass leaves
 * unchanged (walls, rows waiting at an inlet) are not written: the mirror must already hold them. */
int mwd_integrate_rows_mirror(mwd_state* st, const mwd_scene* scenes_dev, uint32_t* status, void* mirror,
                              const void* block, int64_t block_bytes, mwd_stream_t stream);

/* Device address of page-locked host memory (cudaHostGetDevicePointer), for mwd_integrate_rows_mirror.
 * Host utility; no reference counterpart. */
int mwd_host_mapped(const void* host, void** device_address);

/* mwd_integrate in two parts (a state with vert_owner and xform): the row pass (state, forces zeroed,
 * each row's transform into st->xform), then the vertex pass (world_verts from st->xform).  Between
 * the two the state is final, so a copy of it may run beside the vertex pass. */
int mwd_integrate_rows(mwd_state* st, const mwd_scene* scenes_dev, uint32_t* status, mwd_stream_t stream);
int mwd_world_vertices(mwd_state* st, mwd_stream_t stream);

/* World vertices (and the row transforms in st->xform) from the current centres and orientations:
 * world = pos + R(q_acc) r0 for every row.  Needs vert_owner and xform. */
int mwd_refresh_vertices(mwd_state* st, mwd_stream_t stream);

/* broad phase + narrow phase + integrator, n_steps times.  With n_steps > 1 (and a state with
 * vert_owner and xform, no inlet, and a row count for which mwd_integrate_kernels gives 2) the
 * world-vertex pass of each step but the last runs during the
 * next step's broad phase, on a second stream of the library's (one per device and calling thread)
 * that is joined before the narrow phase: the same results, and the state is complete when the
 * call's work on `stream` ends.
 * MWD_OVERLAP=0 in the environment turns this off. */
int mwd_step(mwd_state* st, const mwd_scene* scenes_dev, const mwd_scene* scenes_host, int32_t n_scenes,
             mwd_work* work, int32_t lanes, int32_t n_steps, mwd_stream_t stream);

/* FP32 issue-rate probe (multiply and add chains, no FMA): runs iters x 16 FLOP per thread on
 * 8 x SM-count blocks of 256 threads, times it with CUDA events (synchronises the stream) and
 * writes the rate in TFLOP/s.  scratch: >= 8 x SM-count floats.  The narrow phase's roofline. */
int mwd_probe_fp32(int32_t iters, float* scratch, double* tflops_out /* host */, mwd_stream_t stream);

/* ------------------------------------------------------------------ differentiable step
 *
 * No reference counterpart: the reference has no gradients.  A single-scene FP64 restatement of
 * the device step whose contact topology -- the pairs in contact and, per pair, the support
 * vertices of the final EPA face -- is detected by the FP32 broad + narrow phase above and logged
 * per step.  Given that topology, depth, normal and contact points are smooth functions of the two
 * bodies' centres and vertex orientations (q_acc), so the step (contact force with zero tangential
 * history, as the reference wipes it every step, MWDiem.py:966, then the leapfrog of
 * gpu_Verlet.cu:164-323) is differentiable, and mwd_diff_adjoint applies its transpose.
 *
 * FP64 state row (32 doubles): centre 0-2, v 3-5, v_half 6-8, w_half_bf 9-11, w_bf 12-14, w 15-17,
 * q 18-21, q_half 22-25, q_acc 26-29, unused 30-31; quaternions (w, x, y, z). */
#define MWD_DIFF_ROW 32

typedef struct {
    int32_t A, B;        /* rows */
    int32_t fa[3], fb[3]; /* final EPA face: support-vertex indices into A's and B's vertex tables */
} mwd_contact_rec;

typedef struct {
    int32_t n;              /* rows, walls included (info bit 0) */
    int32_t n_particles;    /* non-wall rows: the centre-of-mass average */
    int32_t n_steps;        /* capacity of step_off / step_count / com (steps of one forward) */
    int32_t ckpt_every;     /* checkpoint interval K: ckpt[k] holds the state after step k K */
    int32_t contact_point;  /* 0: the reference's (cpA - cpB) / 2 (gpu_fine_contact_detection.cu:677), whose
                               torque arm is about minus the centre's position vector; 1: the midpoint
                               (cpA + cpB) / 2 */
    int32_t pad;
    double dt;
    double box[6];          /* fly-away box x_max, x_min, y_max, y_min, z_max, z_min */
    const double* inertia;  /* (n,4) Ix, Iy, Iz, inertia size (the contact law's I) */
    const double* inv_inertia; /* (n,4) 1/Ix, 1/Iy, 1/Iz, 1/m */
    const double* ext;      /* (n,4) external force (gravity) */
    const float* body_verts; /* CSR body-frame vertices (float4), as in mwd_state */
    const int32_t* vert_off;
    const int32_t* info;
    const double* law;      /* (8,) Kn, en, et, mu of particle pairs, then of wall pairs */
    double* F;              /* (n,4) contact force accumulator, zero between steps */
    double* T;              /* (n,4) contact torque accumulator, zero between steps */
    mwd_contact_rec* rec;   /* topology log */
    int64_t rec_cap;
    int64_t* step_off;      /* (n_steps + 1,) first record of each step; step_off[0] = 0 */
    int32_t* step_count;    /* (n_steps,) records of each step; zero before a forward */
    int32_t* t_dev;         /* (1,) device step counter (steps of a captured forward read it) */
    uint32_t* sync;         /* (1,) zero: block counter of the integrator's step advance */
    double* com;            /* optional (n_steps, 4): centre of mass of the particle rows after each step */
    double* ckpt;           /* optional (n_steps / ckpt_every + 1, n, 32) */
    uint32_t* status;       /* (1,) status word (MWD_ST_*) */
    const int32_t* t_base;  /* optional (1,): an explicit step argument t >= 0 means step *t_base + t, so one
                               captured segment of the backward replays at any checkpoint */
} mwd_diff;

/* Log the contacts of the narrow phase just run (work->collision == 1, work->face_ids) as step
 * *d->t_dev of the topology log.  work->collision and work->face_ids must be set. */
int mwd_diff_collect(const mwd_diff* d, const mwd_work* work, mwd_stream_t stream);

/* Contact force and torque of step t (t < 0: *d->t_dev) from the logged topology and the FP64
 * state x, added to d->F, d->T. */
int mwd_diff_force(const mwd_diff* d, const double* x, int32_t t, mwd_stream_t stream);

/* Integrator of step t (t < 0: *d->t_dev, and the counter advances) from x with d->F + ext and
 * d->T into x_out (may alias x); zeroes d->F, d->T.  Optional: FT_store (n,8) receives the total
 * force and torque used; mirror (not NULL) receives the FP32 copies the detection reads (pos,
 * vel, w, q, q_acc, world_verts; force/torque zeroed); with t < 0 also com[t] and the checkpoint. */
int mwd_diff_integrate(const mwd_diff* d, const double* x, double* x_out, double* FT_store, mwd_state* mirror,
                       int32_t t, mwd_stream_t stream);

/* FP32 copies of the FP64 state x into mirror (pos, vel, w, q, q_acc, world_verts). */
int mwd_diff_mirror(const mwd_diff* d, const double* x, mwd_state* mirror, mwd_stream_t stream);

/* Transpose of step t: lam is the gradient with respect to the state after the step; com_grad
 * (optional, (n_steps,4)) the gradient with respect to com[t].  Writes the gradient with respect
 * to the state before the step into lam_prev (overwritten; must not alias lam) and adds the law's
 * gradient to glaw (8,).  x: state before the step; FT: the force/torque of the step (FT_store of
 * mwd_diff_integrate); gFT: (n,8) scratch. */
int mwd_diff_adjoint(const mwd_diff* d, const double* x, const double* FT, int32_t t, const double* lam,
                     double* lam_prev, const double* com_grad, double* gFT, double* glaw, mwd_stream_t stream);

/* Library information. */
const char* mwd_last_error(void);
int mwd_version(void);
int32_t mwd_num_sms(void);

#ifdef __cplusplus
}
#endif
#endif
