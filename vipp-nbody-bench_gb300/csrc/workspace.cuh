// Device workspace of one solver context and the stage entry points.
//
// HBM layout (N particles, C cells, S non-leaf cells, K = (p+1)^2):
//   state, original particle order, FP64 SoA planes [3][N]:
//     x, v (current), x0, v0 (step start), xo, vo (RK4 accumulators) [3][N];
//     acc [N][3] (as returned to the caller)
//   per evaluation, tree (Morton) order:
//     keys/perm (u64/u32 ping-pong pairs), xs [3][N] FP64 positions,
//     ph/pl float4 hi/lo split of the positions (mixed P2P),
//     near/far [3][N] partial accelerations (FP32 or FP64)
//   cells (level by level, path order inside a level, 8 siblings adjacent):
//     begin/end/parent/child/level/path/coord, box [6C], centre [3C],
//     M and L scaled real-basis expansions [C][K] (FP32 or FP64),
//     m2l_src [C][216] source cell per (parent-neighbour, octant) slot,
//     p2p_own/coll [C][27] + counts
//   leaves: list, near-field source ranges (CSR of uint2), P2P work chunks
//   operators: 343 M2L offsets + 8 M2M + 8 L2L real matrices [K][K],
//     stored input-major (op[c*K + r]) in FP64 and FP32.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "harmonics.cuh"
#include "prims.cuh"

namespace gb {

enum TimerClass { kTTree = 0, kTOps = 1, kTUp = 2, kTM2L = 3, kTDown = 4, kTP2P = 5, kTRK4 = 6, kTSoft = 7, kNumTimers = 8 };

struct Workspace {
    // configuration of the evaluation
    int p = 4, K = 25, T = 90;  // T = floor(sqrt(8) s)
    double eps = 0, G = 1, m = 1;
    bool mixed = false;
    bool p2p_newton = false;  // one Newton step after the FP32 rsqrt
    bool m2l_tensor = false;  // tcgen05 M2L (mixed precision only)
    bool m2l_bf16 = false;    // its split: bf16 hi/lo (kind::f16), else 3 x tf32
    bool accurate = false;    // accurate mode: far field times G plus the softening correction (soften.cu)
    cudaStream_t st = nullptr;
    cudaStream_t st2 = nullptr;         // near field, concurrent with the far field on st
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaStream_t st3 = nullptr;         // accurate mode: the softening correction, concurrent with the far field
    cudaEvent_t ev_fork3 = nullptr, ev_join3 = nullptr;
    bool serial = false;                // near field on st after the far field
    int sort_levels = 10;               // key levels the radix sort orders (grown on demand, up to 21)
    unsigned sort_spin_max = kSortSpinMax;  // look-back polls before a wait gives up (tests lower it)
    int64_t launches = 0;
    int num_sms = 152;
    // tuning knobs (gb_set_tuning / the tuning cache; the defaults are the measured best at 4M)
    unsigned p2p_blocks = 8;        // P2P blocks per SM when it runs alone (or after the far field)
    unsigned p2p_blocks_conc = 8;   // P2P blocks per SM launched beside the far field
    int p2p_occ = 8;                // blocks per SM the mixed P2P kernel's registers are budgeted for (8 or 6)
    unsigned p2p_slice = kSliceSources;  // near-field sources per P2P work item
    int m2l_ctas_pct = 100;         // tensor-core M2L CTAs, percent of the SMs (one persistent CTA per SM)

    // forest of independent systems (the batched form; nsys == 1: one tree).
    // Systems keep their particles contiguous in input and tree order, so
    // seg[k] .. seg[k+1] are system k's positions in both; cells are numbered
    // level by level over the whole forest, system by system inside a level
    // (roots: cells 0 .. nsys-1).
    int nsys = 1;
    unsigned *seg = nullptr;        // [nsys + 1] (device)
    int *psys = nullptr;            // [N] system of each particle position
    int *c_sys = nullptr;           // [C] system of each cell
    double2 *sys_par = nullptr;     // [nsys] particle mass and G times it
    uint64_t *mkeys = nullptr;      // [N] Morton keys in input order (the sort orders (system, key) words)
    int sys_bits = 0;               // bits of a system index in the sort word
    int2 *etile = nullptr;          // [s_cap] M2M/L2L tiles: first split entry, entries (<= 64, one system)
    int *oct_list = nullptr;        // [C / 8] M2L target octets grouped by system
    int4 *otile = nullptr;          // [C / 8 + nsys] M2L tiles: system, first list entry, octets
    unsigned *ocnt = nullptr;       // [3 nsys + 1] octets per system, list offsets, fill cursors
    bool forest() const { return seg != nullptr; }
    // key levels a sort word holds beside the system index (3 bits a level)
    int sort_levels_cap() const { return forest() ? (64 - sys_bits) / 3 < kMaxLevel ? (64 - sys_bits) / 3 : kMaxLevel : kMaxLevel; }

    // capacities
    unsigned n_cap = 0;   // particles
    unsigned s_cap = 0;   // split entries (non-leaf cells)
    unsigned c_cap = 0;   // cells = 1 + 8 s_cap
    unsigned r_cap = 0;   // near-field source ranges
    unsigned ch_cap = 0;  // P2P chunks
    int k_cap = 0;        // K the expansion buffers were sized for
    unsigned n = 0;       // current particle count

    // state (original order)
    double *x = nullptr, *v = nullptr, *x0 = nullptr, *v0 = nullptr, *xo = nullptr, *vo = nullptr, *acc = nullptr;
    double *phi = nullptr;  // optional potential (original order)
    double *staging = nullptr;  // AoS staging [3N] for host copies
    double *bbox_part = nullptr; // [6 * 2 * num_sms] bounding-box partials

    // per evaluation, tree order
    uint64_t *keys0 = nullptr, *keys1 = nullptr;
    unsigned *perm0 = nullptr, *perm1 = nullptr;
    uint64_t *keys = nullptr;  // points at the sorted buffer
    unsigned *perm = nullptr;
    unsigned *inv = nullptr;                // [N] tree position of particle i (perm[inv[i]] = i)
    double *xs = nullptr;                   // [3][N]
    float4 *ph = nullptr, *pl = nullptr;    // hi/lo positions, w = mass (hi) / 0
    void *nearf = nullptr, *farf = nullptr; // [3][N] of FP32 or FP64
    double *phis = nullptr;                 // potential parts, tree order [2][N]: near, far (optional)
    double *diag = nullptr;                 // reduction partials of the conserved sums
    unsigned *cnt = nullptr, *off = nullptr;  // [N+1]

    // split entries
    uint64_t *ent0 = nullptr, *ent1 = nullptr, *ent = nullptr;
    int *split_cell = nullptr;

    // cells
    int *c_begin = nullptr, *c_end = nullptr, *c_parent = nullptr, *c_child = nullptr, *c_level = nullptr;
    uint64_t *c_path = nullptr;
    int *c_coord = nullptr;     // [3C]
    double *c_box = nullptr;    // [6C] min xyz, max xyz
    double *c_ctr = nullptr;    // [3C]
    void *Mexp = nullptr, *Lexp = nullptr;  // [C][K]
    int *m2l_src = nullptr;     // [C][216]
    int *p2p_own = nullptr, *p2p_cnt = nullptr;  // [C][27], [C]
    void *smom = nullptr;       // accurate mode: [C] moment records (soften.cu)
    void *smom_oct = nullptr;   // [C][8] octant moment records of the leaves
    void *staylor = nullptr;    // [C][13] leaf-centre value, J and potential of the far levels' correction
    void *soft_corr = nullptr;  // [3][N] the correction, tree order (computed beside the far field)
    unsigned soft_corr_cap = 0; // particles soft_corr is sized for (doubles)
    unsigned soft_cap = 0;      // cells the three are sized for (0: not allocated)
    bool soft_mixed = false;    // their element type
    int *coll = nullptr, *coll_cnt = nullptr;    // [C][27], [C]
    unsigned *flag = nullptr, *flag_off = nullptr;  // [C+1]

    // leaves
    int *leaves = nullptr;            // [C]
    unsigned *rng_cnt = nullptr;      // [C] ranges per leaf before merging (then capacity offsets)
    unsigned *rng_off = nullptr;      // [C+1]
    unsigned *rng_len = nullptr;      // [C] ranges per leaf after merging
    uint2 *ranges = nullptr;          // [r_cap]
    unsigned *chunk_cnt = nullptr, *chunk_off = nullptr;  // [C]
    int4 *chunks = nullptr;           // [ch_cap] work items (leaf, first target, packed sizes, partial slot)
    unsigned *src_total = nullptr;    // [C] near-field sources per leaf
    unsigned *part_cnt = nullptr, *part_off = nullptr;  // [C+1] partial-sum slots per leaf
    void *part = nullptr;             // [part_cap][3][32] partial sums of split items (FP32 or FP64)
    unsigned part_cap = 0;
    unsigned *queue = nullptr;        // P2P work-queue counter

    // operators
    double *ops_d = nullptr;  // [(343+16) K K]
    float *ops_f = nullptr;
    float *zf = nullptr;      // mixed forms: [nsys][359][(2p+1)^2] Z tables of the FP32 operators (fmm.cu)
    void *m2l_tab = nullptr;  // offset-independent factors of the M2L operator entries (fmm.cu)
    float *bimg = nullptr;    // tensor-core M2L operator images (m2l_tc.cu)
    float *ms_tc = nullptr;   // tensor-core M2L split expansions, 2 ms_rows ms_kp floats (m2l_tc.cu)
    unsigned ms_rows = 0;     // c_cap + kZeroRows: the last rows are zero
    int ms_kp = 0;
    bool ms_bf16 = false;     // the split form tmap_ms was encoded for
    CUtensorMap tmap_ms{};    // TMA map of ms_tc

    // device-side info and device-resident counters
    TreeInfo *info = nullptr;
    unsigned *d_counts = nullptr;  // [kNumCounts]: 0 n, 1 S, 2 C, 3 leaves, 4 ranges, 5 items,
                                   // 6 S requested, 7 items requested, 8 partial slots,
                                   // 9 key levels a deeper sort needs (0: enough)
    TreeInfo *h_info = nullptr;    // pinned mirror

    SortTemp sort;
    ScanTemp scan;

    // timing
    bool timing = false;
    double t_ms[kNumTimers] = {};
    int64_t t_launch[kNumTimers] = {};
};

constexpr int kNumCounts = 16;

// Grid of a grid-stride kernel: the full-GPU size, capped by an upper bound of
// the work (from the buffer capacities) so that small systems launch small
// grids and several systems' kernels can share the GPU.
inline unsigned capped_grid(unsigned full, size_t work_bound) {
    const size_t b = work_bound < 1 ? 1 : work_bound;
    return b < full ? static_cast<unsigned>(b) : full;
}
inline size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }
// per-cell systems of a forest, or null for one tree
inline const int *forest_cells(const Workspace &ws) { return ws.forest() ? ws.c_sys : nullptr; }
constexpr int kM2LTileTC = 128;  // target octets per tensor-core M2L tile (m2l_tc.cu)
constexpr int kZeroRows = 32;    // zero rows after the split expansions (one per row quad of a tile)
constexpr int kM2LTileCC = 64;   // per CUDA-core M2L tile (fmm.cu)
constexpr int kOpM2M = 343;  // op index of M2M octant 0
constexpr int kOpL2L = 351;  // op index of L2L octant 0
constexpr int kNumOps = 359;

// stages (all asynchronous on ws.st)
void build_tree(Workspace &ws);               // bbox, keys, sort, cells, leaves, lists, near-field ranges
void forest_tiles(Workspace &ws, int rows);   // forest: M2M/L2L tiles and M2L tiles of `rows` octets per system
void build_operators(Workspace &ws);          // 359 translation matrices for the current root box
size_t m2l_table_bytes(int p);
inline size_t zf_table_floats(int p) { return static_cast<size_t>(kNumOps) * (2 * p + 1) * (2 * p + 1); }  // per system
void build_m2l_table(Workspace &ws);          // fill m2l_tab for ws.p (once per p, outside step graphs)
void upward_pass(Workspace &ws);              // P2M + M2M
void m2l_pass(Workspace &ws);                 // M2L into L (CUDA cores)
void m2l_pass_tc(Workspace &ws);              // M2L into L (tensor cores, mixed)
bool m2l_tc_supported(int p);
size_t m2l_tc_image_floats(int p);
int m2l_tc_row_floats(int p);
const char *m2l_tc_encode(Workspace &ws);     // (re)build tmap_ms; nullptr or an error message
void downward_pass(Workspace &ws);            // L2L + L2P into far
void soften_pass(Workspace &ws);              // accurate mode: far = G (far + softening correction)
void soften_corr(Workspace &ws);              // the same correction into soft_corr (no far-field input)
void soften_apply(Workspace &ws);             // far = G (far + soft_corr)
void soften_phi(Workspace &ws, double *farphi); // accurate mode: the far potential's correction (tree order)
size_t soften_taylor_values();                // per-leaf values of the far levels' correction
size_t soften_cell_bytes(bool mixed);         // bytes of one moment record
void p2p_pass(Workspace &ws, unsigned per_sm); // near-field kernel over the queue, per_sm blocks per SM
void p2p_finish(Workspace &ws);               // add the slices of split items: near complete
void finalize_accel(Workspace &ws, double *acc_orig);  // acc[perm] = near + far
// diagnostics after an evaluation (tree order, FP64): far-field potential of the
// local expansions (no G, like the far-field acceleration) and the near-field
// softened potential sum (times G m, i == j excluded)
void far_potential(Workspace &ws, double *farphi);
void near_potential(Workspace &ws, double *nearphi);
void potential_orig(Workspace &ws, double *phi_orig);    // phi[perm] = -(near + far), needs ws.phis [2N]
void conserved_sums(Workspace &ws, const double *phi_orig, double *sums8);  // see diag.cu
size_t diag_scratch_doubles();
void generate_plummer(Workspace &ws, unsigned n, uint64_t seed, double x0_max, double r_max, double x_scale = 1.0,
                      double v_scale = 1.0);  // ic.cu
// forest: system k's particles are stream family seeds[k] scaled by scales[k] (positions, velocities)
void generate_plummer_forest(Workspace &ws, const uint64_t *seeds, const double2 *scales, double x0_max, double r_max);
// clusters (<= 8) Plummer clusters + a uniform background fraction (ic.cu);
// params (may be null): 8 doubles per cluster, centre[3], radius, bulk[3], size
int generate_clustered(Workspace &ws, unsigned n, uint64_t seed, int clusters, double background, double r_max,
                       double *params);
void direct_sum(Workspace &ws, const double *x_orig, const long long *targets, unsigned nt, double *out_soa,
                double *part, unsigned nsplit);  // part: [nsplit][3][nt] scratch

// timing helpers
void timer_begin(Workspace &ws, int cls);
void timer_end(Workspace &ws, int cls);

#ifdef __CUDACC__
// Cell centre relative to the root-box centre as an FP32 hi/lo pair, to
// re-centre the FP32 hi/lo particle positions ph/pl on a cell:
// (ph - c.h) + (pl - c.l) keeps ~1e-7 of the cell's neighbourhood.
struct RootC {
    float hx, hy, hz, lx, ly, lz;
};

__device__ __forceinline__ RootC leaf_centre(const double *c_ctr, int c, const TreeInfo *info) {
    RootC r;
    const double d0 = c_ctr[3 * c] - info->root_c[0];
    const double d1 = c_ctr[3 * c + 1] - info->root_c[1];
    const double d2 = c_ctr[3 * c + 2] - info->root_c[2];
    r.hx = static_cast<float>(d0), r.hy = static_cast<float>(d1), r.hz = static_cast<float>(d2);
    r.lx = static_cast<float>(d0 - r.hx), r.ly = static_cast<float>(d1 - r.hy), r.lz = static_cast<float>(d2 - r.hz);
    return r;
}
#endif

}  // namespace gb
