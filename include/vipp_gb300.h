/*
 * vipp_gb300.h — C-ABI of the GB300 (sm_103a) gravity FMM solver.
 *
 * This is the drop-in boundary for the reference's gravity solver path
 * (satoshigeyuki/vipp-nbody-bench). The reference's boundary is the
 * compile-time Solver concept selected by `gravity::Solver<M,T,X,V,A,G>`
 * (gravity/include/solver.hpp:6-9) with three methods
 * (gravity/include/solver_ref.hpp:11-27):
 *
 *   preprocess(problem, x, v)   -> gb_create + gb_upload
 *   solve(problem, t, x, v)     -> gb_rk4_step(dt = problem.delta_t() / t)
 *   postprocess(problem, x, v)  -> gb_download
 *
 * The header-only C++ adapter `gravity::SolverGB300<M,T,X,V,A,G>`
 * (include/gravity/solver_gb300.hpp in the package directory) wraps these calls
 * and rethrows errors as std::runtime_error, as the reference does.
 *
 * Conventions: plain pointers and sizes; positions/velocities/accelerations
 * are array-of-structs doubles (x0,y0,z0,x1,...) exactly like the reference's
 * std::vector<Vector<double>>. Every call returns GB_OK (0) or an error code
 * and never throws; gb_last_error() describes the last failure of a context.
 * A context owns all of its device memory and its CUDA stream, and is used by
 * one host thread at a time.
 */
#ifndef VIPP_GB300_H
#define VIPP_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define GB_API
#else
#define GB_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum gb_status {
    GB_OK = 0,
    GB_ERR_INVALID = 1,       /* bad argument (N, s, p, null pointer, ...) */
    GB_ERR_NONFINITE = 2,     /* a position is NaN or infinite */
    GB_ERR_DEPTH = 3,         /* the tree would need more than 21 levels */
    GB_ERR_CUDA = 4,          /* a CUDA runtime call failed */
    GB_ERR_NO_DEVICE = 5,     /* no CUDA device / extension cannot run */
    GB_ERR_STATE = 6,         /* call out of order (e.g. step before upload) */
    GB_ERR_CAPACITY = 7       /* internal capacity exceeded and could not grow */
};

/* Arithmetic of the force evaluation. */
enum gb_precision {
    GB_PREC_FP64 = 0,   /* every stage in FP64 on CUDA cores (the plain form) */
    GB_PREC_MIXED = 1   /* P2P FP32 (relative coordinates, compensated sums),
                           expansions FP32 scaled per cell, M2L on the tensor
                           cores (3xTF32); RK4 combination in FP64 */
};

/* Method of the force evaluation. */
enum gb_mode {
    GB_MODE_REF = 0,      /* the reference's method (solver_ref.hpp:164-232): trees,
                             lists and results as the reference's; its far field
                             expands the unsoftened 1/r and carries no G */
    GB_MODE_ACCURATE = 1  /* no counterpart in the reference: the same tree,
                             lists and expansions, the far field multiplied by G,
                             plus the far field of the softening difference
                             (eps^2 + r^2)^-3/2 - r^-3 expanded to second order
                             about each far source cell's centre of mass; with
                             p = 10 it follows the softened direct sum to ~1e-5
                             RMS, where the reference's method stops at ~eps^2/r^2 */
};

typedef struct gb_config {
    int p;          /* expansion order, 1..10 (Problem::p, problem.hpp:229) */
    int s;          /* leaf parameter; a cell splits above floor(sqrt(8) s)
                       particles (octree.hpp:83) */
    double eps;     /* Plummer softening (Problem::epsilon) */
    double G;       /* gravitational constant; like the reference, only the
                       near field (P2P) is multiplied by it (fmm.hpp:531-540) */
    double m;       /* mass of every particle (Problem::m = M/N) */
    int precision;  /* enum gb_precision */
    int device;     /* CUDA device ordinal */
    int flags;      /* bit set of gb_flags, 0 by default */
    int mode;       /* enum gb_mode, GB_MODE_REF by default */
} gb_config;

enum gb_flags {
    GB_FLAG_P2P_NEWTON = 1,  /* mixed P2P: refine the FP32 rsqrt with one Newton
                                step (off by default: it changes the RMS error by
                                about 1e-10 and costs about 20% of P2P time) */
    GB_FLAG_M2L_CUDA_CORES = 2, /* mixed M2L on CUDA cores in FP32 instead of the
                                   default tensor-core M2L (tcgen05) */
    GB_FLAG_SERIAL = 4,         /* run the near field (P2P) after the far field on
                                   one stream instead of concurrently on a second
                                   stream of the context (same results) */
    GB_FLAG_NO_GRAPH = 8,       /* launch every kernel of an RK4 step instead of
                                   replaying the step's captured CUDA graph (same
                                   results; graphs are also off while kernel
                                   timing is enabled) */
    GB_FLAG_M2L_BF16 = 16,      /* tensor-core M2L with a BF16 hi/lo split
                                   (~2^-17 relative per product; half the gathered
                                   bytes and MMA time, ~17% less M2L time) instead
                                   of the default three-term TF32 split (~2^-21) */
    GB_FLAG_BATCH_CONTEXTS = 32 /* gb_batch_create: one context per system (the
                                   contexts form) instead of the forest form */
};

typedef struct gb_ctx gb_ctx;

/* Statistics of the last force evaluation. */
typedef struct gb_stats {
    int64_t n;            /* particles */
    int64_t ncells;       /* cells, root included, empty leaves included */
    int64_t nleaves;
    int64_t depth;        /* deepest level (root = 0) */
    int64_t m2l_pairs;    /* M2L (target, source) pairs, targets at level >= 2 */
    int64_t p2p_pairs;    /* near-field (target, source) particle pairs */
    int64_t p2p_ranges;   /* source ranges over all leaves after merging */
    int64_t retries;      /* evaluations of this context repeated after growing its buffers */
    int64_t graph_steps;  /* RK4 steps run by replaying the captured step graph */
    int64_t direct_steps; /* RK4 steps run by launching every kernel */
    int64_t graph_captures; /* step graphs captured (a new n, dt or buffer set) */
    int64_t steps;        /* RK4 steps taken since the state was set (upload or
                             initial conditions; a checkpoint load restores the
                             saved count) */
} gb_stats;

/* Create a context on cfg->device. Validates cfg (p in 1..10, s >= 1). */
GB_API int gb_create(const gb_config *cfg, gb_ctx **out);
GB_API void gb_destroy(gb_ctx *ctx);
/* Message for the last error of ctx (or of the last failed gb_create when ctx is NULL). */
GB_API const char *gb_last_error(const gb_ctx *ctx);

/* Replace p, s, eps, G, m and precision of an existing context (Problem fields
 * read by SolverRef::solve, solver_ref.hpp:21-25). */
GB_API int gb_set_config(gb_ctx *ctx, const gb_config *cfg);

/* Batches of independent systems (the batching form of the benchmark: many
 * Plummer systems of uneven N concatenated with segment offsets). No
 * counterpart in the reference, which runs one Problem per Solver. System k
 * holds particles [seg_offsets[k], seg_offsets[k+1]) of the concatenated AoS
 * arrays (seg_offsets[0] = 0), particle mass m_per_system[k] (cfg->m when
 * NULL) and the rest of cfg. A batch step advances every system by one RK4
 * step. Two forms, with the same results per system:
 *   forest (default): one context over all systems; every kernel of a force
 *     evaluation is one launch over all of them (tiles of the far field hold
 *     one system's cells each), one step graph per batch step. Each system
 *     keeps its own root box, tree (the reference's for that system alone),
 *     operators, mass and G m. A forest holds at most 2^31 - 1 particles, and
 *     a system's tree at most floor((64 - ceil(log2 nsys)) / 3) levels (18
 *     for 512 systems); a deeper system fails the step with GB_ERR_DEPTH.
 *   contexts (cfg->flags & GB_FLAG_BATCH_CONTEXTS, and always for
 *     GB_MODE_ACCURATE): one context, tree and step graph per system; all
 *     systems' steps are queued before any is waited for.
 * gb_batch_system gives system k's context in the contexts form (the batch
 * owns it) and NULL in the forest form; gb_batch_accel, gb_batch_conserved
 * and gb_batch_stats work in both. */
typedef struct gb_batch gb_batch;
GB_API int gb_batch_create(const gb_config *cfg, size_t nsys, const uint64_t *seg_offsets, const double *m_per_system,
                           gb_batch **out);
GB_API void gb_batch_destroy(gb_batch *b);
GB_API const char *gb_batch_last_error(const gb_batch *b);
GB_API int gb_batch_upload(gb_batch *b, const double *x_aos, const double *v_aos);
/* Every system of the batch generated on the device instead of uploaded: a
 * Plummer sphere of total mass 1 (G = 1) with radii capped at r_max scale
 * radii, scaled to a scale radius R_k uniform in [r_lo, r_hi] (positions
 * times R_k, velocities times R_k^-1/2); radii (may be NULL) receives the
 * nsys R_k. Each system's particle mass stays as given at gb_batch_create. */
GB_API int gb_batch_init_plummer(gb_batch *b, uint64_t seed, double r_lo, double r_hi, double r_max, double *radii);
/* The same with this batch's system k drawn as system first + k of the seeded
 * family: a batch split over ranks into contiguous runs of systems draws
 * exactly the systems of the whole batch. */
GB_API int gb_batch_init_plummer_at(gb_batch *b, uint64_t seed, uint64_t first, double r_lo, double r_hi, double r_max,
                                    double *radii);
GB_API int gb_batch_download(gb_batch *b, double *x_aos, double *v_aos);
GB_API int gb_batch_rk4_step(gb_batch *b, double dt);
GB_API int gb_batch_size(const gb_batch *b, size_t *nsys, uint64_t *n_total);
GB_API gb_ctx *gb_batch_system(gb_batch *b, size_t k);
GB_API int gb_batch_is_forest(const gb_batch *b);
/* The forest form's context (for gb_enable_timing, gb_kernel_times,
 * gb_launch_count, gb_stream; the batch owns it); NULL in the contexts form. */
GB_API gb_ctx *gb_batch_forest(gb_batch *b);
/* Accelerations (AoS, n_total x 3) and optionally potentials (n_total) of
 * every system at the current positions, concatenated like the state. */
GB_API int gb_batch_accel(gb_batch *b, double *a_aos, double *phi);

/* Initial state generated on the device: the reference's Plummer sphere
 * (Problem::initialize, problem.hpp:188-211, 245-292; G = M = a = 1) with one
 * counter-based random stream per particle. r_max = 0 keeps the reference's
 * radius cap (mass fraction below 1 - eps, eps from the config); r_max > 0
 * caps radii at r_max instead. Same distribution as the reference, not the
 * same numbers. Replaces the state like gb_upload; gb_download reads it. */
GB_API int gb_init_plummer(gb_ctx *ctx, size_t n, uint64_t seed, double r_max);

/* The adaptive-depth stress workload generated on the device (no counterpart
 * in the reference): `clusters` (1..8) equal-mass Plummer clusters, each with
 * its scale radius uniform in [0.01, 0.1], its centre uniform in [0, 1)^3, a
 * Gaussian bulk velocity (sigma 0.3 per component) and internal Plummer
 * velocities of its own mass and radius (G = 1), radii capped at r_max scale
 * radii, plus round(background n) particles uniform in [0, 1)^3 at rest;
 * total mass 1 in equal masses. The same counter-based streams as
 * gb_init_plummer. params (may be NULL) receives 8 doubles per cluster:
 * centre[3], scale radius, bulk velocity[3], particle count. Replaces the
 * state like gb_upload. */
GB_API int gb_init_clustered(gb_ctx *ctx, size_t n, uint64_t seed, int clusters, double background, double r_max,
                             double *params);

/* preprocess: copy n particles (AoS doubles) to the device. n may be 0. */
GB_API int gb_upload(gb_ctx *ctx, const double *x_aos, const double *v_aos, size_t n);
/* postprocess: copy the current state back (AoS doubles, n entries each). */
GB_API int gb_download(gb_ctx *ctx, double *x_aos, double *v_aos);

/* solve: one classical RK4 step of size dt (solver_ref.hpp:36-104); four
 * force evaluations, tree rebuilt at every stage. Asynchronous with respect to
 * the host; errors found on the device are reported by this call or the next
 * gb_sync / gb_download. */
GB_API int gb_rk4_step(gb_ctx *ctx, double dt);

/* One FMM force evaluation (SolverRef::acceleration, solver_ref.hpp:164-177)
 * at the current positions; a_aos (may be NULL) receives n accelerations (AoS
 * doubles). phi may be NULL; when given it receives n potentials per unit mass
 * in the accelerations' convention a = -grad phi: the softened near-field sum
 * -G m sum_{j != i} (r^2 + eps^2)^-1/2 (FP64) plus the far field from the local
 * expansions, which like the reference's far field carries no G (times G in
 * GB_MODE_ACCURATE, without the softening correction the accelerations get).
 * The reference has no potential; this output has no counterpart there. */
GB_API int gb_accel(gb_ctx *ctx, double *a_aos, double *phi);

/* Conserved quantities of the current state, for energy-drift checks (no
 * counterpart in the reference, which computes no potential). The potential
 * comes from one FMM evaluation of the current positions (gb_accel's phi);
 * sums in FP64 with a fixed reduction order (deterministic). */
typedef struct gb_conserved {
    double kinetic;             /* 1/2 m sum |v|^2 */
    double potential;           /* 1/2 m sum phi_i */
    double total;               /* kinetic + potential */
    double momentum[3];         /* m sum v */
    double angular_momentum[3]; /* m sum x cross v */
} gb_conserved;
GB_API int gb_get_conserved(gb_ctx *ctx, gb_conserved *out);
/* The conserved quantities of every system of a batch: out[k] for system k
 * (nsys entries). */
GB_API int gb_batch_conserved(gb_batch *b, gb_conserved *out);

/* FP64 direct softened sum on the GPU for the listed targets of the current
 * positions (the accuracy oracle; SolverRefNaive::acceleration,
 * solver_ref_naive.hpp:103-119). targets may be NULL for all particles.
 * a_aos receives ntargets (or n) accelerations. */
GB_API int gb_direct_accel(gb_ctx *ctx, const int64_t *targets, size_t ntargets, double *a_aos);

/* No counterpart in the reference. The same FP64 direct softened sum as
 * gb_direct_accel, for callers that cannot allocate GPU memory (hosts that own
 * every device allocation through their own pool, runtimes that forbid
 * cudaMalloc after start-up, plugins limited to the buffers they are handed).
 * It creates no context and calls no cudaMalloc/cudaFree or allocating
 * library routine: every input and output is the caller's device memory.
 *   x_dev        n positions, AoS doubles, device memory
 *   targets_dev  ntargets particle indices in [0, n) (device memory), or NULL
 *                for all n particles; an index outside [0, n) yields NaN
 *   a_dev        ntargets (or n) accelerations, AoS doubles, device memory
 *   stream       cudaStream_t to run on (NULL: the legacy default stream)
 * The kernels run on the calling thread's current device and are only
 * queued: results are ready once `stream` reaches this point. Its scratch
 * is one fixed 16 MiB device array inside the library, reserved on every
 * GPU that loads it until the process exits; at most 699,050 targets fit
 * (GB_ERR_CAPACITY beyond that). The first call on a device (and the first
 * after cudaDeviceReset gave it a new context) looks up that array's address
 * and should come before any stream capture. All calls share the array, so
 * calls that overlap on the GPU (other streams, other host threads) race;
 * order them on one stream. No targets (ntargets == 0 with a list, or n == 0
 * without one) is a no-op; a target list with n == 0 is GB_ERR_INVALID. A
 * CUDA error already pending on the calling thread when the call starts is
 * left pending and the call returns GB_ERR_CUDA without queueing anything. */
GB_API int gb_direct_accel_noalloc(const double *x_dev, size_t n, const int64_t *targets_dev, size_t ntargets, double G,
                                   double m, double eps, double *a_dev, void *stream);

/* Launch and tree parameters a tuner may change (no counterpart in the
 * reference). None changes the method: the launch shapes give bit-identical
 * results, the slice length changes only the FP32 summation order of long
 * near-field lists, and leaf_s applies to GB_MODE_ACCURATE alone (the
 * reference mode keeps the reference's tree for the config's s).
 * vipp_gb300/autotune.py measures candidates per size bucket and writes a
 * cache file; gb_upload applies the cache entry named by the environment
 * variable VIPP_GB_TUNE_FILE for the context's configuration and the uploaded
 * particle count, where the file has one. */
typedef struct gb_tuning {
    int p2p_blocks;      /* P2P blocks per SM when the near field runs alone, 1..16 (default 8) */
    int p2p_blocks_conc; /* P2P blocks per SM launched beside the far field, 0..16 (default 8) */
    int p2p_slice;       /* near-field sources per P2P work item, 1024..65536 (default 8192) */
    int m2l_ctas_pct;    /* tensor-core M2L CTAs, percent of the SMs, 10..100 (default 100) */
    int serial;          /* 1: the near field after the far field on one stream (default 0) */
    int leaf_s;          /* GB_MODE_ACCURATE: leaf parameter used instead of the config's s
                            (0: the config's s) */
    int p2p_occupancy;   /* mixed P2P kernel build: 8 (registers budgeted for 8 blocks
                            per SM, default; 0 means 8) or 6 (80 registers, more work
                            in flight per warp); same results either way */
} gb_tuning;
GB_API int gb_set_tuning(gb_ctx *ctx, const gb_tuning *t);
GB_API int gb_get_tuning(const gb_ctx *ctx, gb_tuning *out);
/* The entry of a tuning cache file for cfg's p, precision, mode and M2L split
 * (GB_FLAG_M2L_BF16) and n's size bucket floor(log2 n). The file holds one
 * entry per line as key=value tokens (p, precision, mode, m2l_bf16, log2n,
 * then the gb_tuning fields by name); '#' starts a comment. GB_OK with *out
 * filled, GB_ERR_STATE when the file has no matching entry, GB_ERR_INVALID
 * when it cannot be read or an entry is malformed. No GPU is needed. */
GB_API int gb_tuning_lookup(const char *path, const gb_config *cfg, size_t n, gb_tuning *out);

/* Checkpoints: the state that restarts a run. The reference keeps none (its
 * ENABLE_PRINT build writes the positions of a run as text,
 * gravity/include/benchmark.hpp:15-20, 46-58). A step depends only on the
 * positions, velocities and configuration, so a run restarted from a
 * checkpoint continues bit-identically to the run that wrote it.
 * File layout (little-endian; 8-byte words after the header):
 *   header, 128 bytes: 0 char[8] "VIPPGBCK", 8 uint32 version (1),
 *     12 uint32 header bytes (128), 16 uint64 n, 24 uint64 nsys,
 *     32 int64 steps, 40 double t, 48 int32 p, 52 int32 s, 56 int32 precision,
 *     60 int32 mode, 64 int32 flags, 68 int32 leaf_s, 72 double eps,
 *     80 double G, 88 double m, 96..127 zero;
 *   uint64 seg_offsets[nsys + 1]; double m_per_system[nsys];
 *   double x[3n]; double v[3n] (AoS, the caller's particle order);
 *   uint64 check word: FNV-1a over every preceding 8-byte word, one word per
 *     round (offset basis 0xcbf29ce484222325, prime 0x100000001b3).
 * Files are written under path + ".tmp" and renamed over path. */
typedef struct gb_checkpoint_info {
    uint64_t n;      /* particles of all systems */
    uint64_t nsys;   /* systems (1 for a context) */
    int64_t steps;   /* RK4 steps taken since the state was set */
    double t;        /* simulated time, as given to the save */
    gb_config cfg;   /* the writer's p, s, eps, G, m, precision, flags and mode
                        (device: 0 on read) */
    int32_t leaf_s;  /* leaf parameter in effect (s, or the tuning's leaf_s in
                        accurate mode) */
} gb_checkpoint_info;

enum gb_checkpoint_flags {
    GB_CHECKPOINT_ANY_CONFIG = 1  /* load: skip the configuration check */
};

/* Host only (no GPU). Write a checkpoint from host arrays: seg_offsets
 * (nsys + 1 entries from 0 to n, not decreasing; NULL for one system),
 * m_per_system (NULL: info->cfg.m for every system), x_aos and v_aos (3n
 * each). Read fills *info from the header; when any array is given it reads
 * the whole body, verifies the check word and fills the arrays given:
 * seg_offsets (nsys + 1) and m_per_system (nsys) when nsys <= nsys_cap, x_aos
 * and v_aos (3n) when n <= n_cap. A malformed, truncated or corrupt file or a
 * bad argument is GB_ERR_INVALID, described by gb_last_error(NULL). */
GB_API int gb_checkpoint_write(const char *path, const gb_checkpoint_info *info, const uint64_t *seg_offsets,
                               const double *m_per_system, const double *x_aos, const double *v_aos);
GB_API int gb_checkpoint_read(const char *path, gb_checkpoint_info *info, uint64_t *seg_offsets,
                              double *m_per_system, size_t nsys_cap, double *x_aos, double *v_aos, size_t n_cap);

/* Save the context's state, its step count and the time t (GB_ERR_STATE
 * before an upload). Load replaces the context's state as gb_upload does and
 * restores the step count; *t (may be NULL) receives the saved time. The file
 * must hold one system, and unless flags has GB_CHECKPOINT_ANY_CONFIG its p,
 * s, eps, G, m, precision, mode, leaf_s and result-changing flags
 * (GB_FLAG_P2P_NEWTON, GB_FLAG_M2L_CUDA_CORES, GB_FLAG_M2L_BF16) must equal
 * the context's (GB_ERR_INVALID otherwise; the state is then unchanged). */
GB_API int gb_checkpoint_save(gb_ctx *ctx, const char *path, double t);
GB_API int gb_checkpoint_load(gb_ctx *ctx, const char *path, int flags, double *t);
/* The same for a batch: the file holds the batch's systems. Load requires the
 * batch's segment offsets, and (unless GB_CHECKPOINT_ANY_CONFIG) its masses
 * and configuration. */
GB_API int gb_batch_checkpoint_save(gb_batch *b, const char *path, double t);
GB_API int gb_batch_checkpoint_load(gb_batch *b, const char *path, int flags, double *t);

/* Block until all queued work finished; reports deferred device errors. */
GB_API int gb_sync(gb_ctx *ctx);
GB_API int gb_get_stats(gb_ctx *ctx, gb_stats *out);
/* Batch statistics: the forest's (every system's cells, pairs and ranges
 * together), or the contexts' summed (depth: the deepest). */
GB_API int gb_batch_stats(gb_batch *b, gb_stats *out);
/* Kernel launches queued by the batch so far (all its contexts). */
GB_API int64_t gb_batch_launch_count(const gb_batch *b);

/* Tree dump of the last force evaluation, for the parity tests. Cells are
 * numbered level by level, and within a level in the reference's child order
 * (octant bit = 1 for the lower half, ties to the upper half), so that cell
 * order within a level equals the reference's path order.
 *   level[c], parent[c] (-1 root), first_child[c] (-1 leaf), path[c] (3 bits
 *   per level, level-1 digit most significant), box_min/box_max[3c..3c+2],
 *   pt_begin[c]..pt_end[c] index into order[] (original particle indices in
 *   tree order; within a leaf ascending, as the reference inserts them).
 * Lists (CSR over cells, entries are cell numbers in the reference's order):
 *   m2l (solver_ref.hpp:144), p2p_own (the entries a cell adds itself,
 *   solver_ref.hpp:140, 150; the full p2p list is the concatenation over the
 *   ancestors from the root), coll (solver_ref.hpp:138, 152).
 * Call with all array pointers NULL to get the sizes in *ncells and
 * *list_sizes[3]. */
GB_API int gb_tree_dump(gb_ctx *ctx, int64_t *ncells, int64_t *list_sizes, int32_t *level, int64_t *parent,
                 int64_t *first_child, uint64_t *path, double *box_min, double *box_max, int64_t *pt_begin,
                 int64_t *pt_end, int64_t *order, int64_t *m2l_off, int64_t *m2l, int64_t *p2p_off,
                 int64_t *p2p_own, int64_t *coll_off, int64_t *coll);

/* Kernel timing: when enabled, the context brackets each kernel class with
 * CUDA events on its stream and accumulates milliseconds and launch counts;
 * while it is on, the classes run one after another on one stream (no
 * near/far overlap) and every kernel is launched directly (no step graph).
 * Classes: 0 tree+lists, 1 operators, 2 P2M+M2M, 3 M2L, 4 L2L+L2P, 5 P2P,
 * 6 RK4+finalize, 7 softening correction (accurate mode). gb_kernel_times fills up to n entries of ms and launches
 * and resets the accumulators. */
GB_API int gb_enable_timing(gb_ctx *ctx, int on);
GB_API int gb_kernel_times(gb_ctx *ctx, double *ms, int64_t *launches, int n);

/* The context's CUDA stream (a cudaStream_t), so callers can order their own
 * work or record events around the context's kernels. */
GB_API void *gb_stream(gb_ctx *ctx);

/* Number of kernel launches issued by the context since creation. */
GB_API int64_t gb_launch_count(const gb_ctx *ctx);

/* Library version string. */
GB_API const char *gb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* VIPP_GB300_H */
