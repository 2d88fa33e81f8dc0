// Adaptive octree, interaction lists and near-field source ranges, built in
// parallel and bit-exact with the reference's serial insertion
// (gravity/include/octree.hpp:79-191, solver_ref.hpp:115-162).
//
// Why this reproduces the reference tree:
//  * A reference cell splits exactly when more than T = floor(sqrt(8) s)
//    particles fall into it (octree.hpp:83, 143-147); membership does not
//    depend on insertion order.
//  * Child boxes are recursive FP64 midpoints (hi + lo) / 2 of the padded
//    bounding box (octree.hpp:169-176, fmm.hpp:403-405); a particle goes to the
//    first child whose closed box holds it, so it takes the lower half of an
//    axis iff coordinate < mid. k_keys walks 21 levels of exactly these
//    midpoints and records the child offset of every level (bit set = lower
//    half), so particles of one cell share the key prefix of that cell.
//  * After a stable sort, position i starts a level-L run iff its key differs
//    from key[i-1] at or above level L, and that run holds more than T
//    particles iff key[i+T] still shares the level-L prefix. The split cells
//    are therefore found for all levels at once (k_split_count).
//  * Lists: by induction over calc_link, a cell's colleagues are the non-leaf
//    same-level cells within one cell of it, and its cousins are the children
//    of its parent's colleagues; every list is ordered by (parent's list
//    order, child offset), which is the cell path order — the order of cell
//    numbers inside a level here.
#include <cfloat>

#include "workspace.cuh"

namespace gb {

namespace {

constexpr int kTB = 256;

// Order-preserving map of finite doubles to signed integers (an involution):
// negative values get their magnitude bits flipped, so integer order is the
// order of the values (-0 just below +0). Min and max then run on the integer
// pipe instead of GB300's narrow FP64 pipe.
__device__ __forceinline__ long long ord_key(long long b) { return b ^ ((b >> 63) & 0x7fffffffffffffffLL); }

__global__ void k_bbox_partial(const double *__restrict__ x, unsigned n, double *__restrict__ part, TreeInfo *info) {
    const long long kmax = ord_key(__double_as_longlong(DBL_MAX)), kmin = ord_key(__double_as_longlong(-DBL_MAX));
    long long kn[3] = {kmax, kmax, kmax}, kx[3] = {kmin, kmin, kmin};
    bool bad = false;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const long long b = __double_as_longlong(x[static_cast<size_t>(a) * n + i]);
            const bool fin = ((b >> 52) & 0x7ff) != 0x7ff;  // non-finite values are skipped, as fmin / fmax do NaN
            bad |= !fin;
            const long long k = ord_key(b);
            if (fin) kn[a] = min(kn[a], k), kx[a] = max(kx[a], k);
        }
    }
    if (bad) atomicOr(&info->err, kDevNonFinite);
    double mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // +-0 compare equal as doubles: either is the box's bound (the padding makes them the same)
        mn[a] = __longlong_as_double(ord_key(kn[a]));
        mx[a] = __longlong_as_double(ord_key(kx[a]));
    }
    __shared__ double red[6][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o; o >>= 1) {
            mn[a] = fmin(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmax(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
        if (lane == 0) red[a][w] = mn[a], red[3 + a][w] = mx[a];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int q = threadIdx.x;
        double r = q < 3 ? DBL_MAX : -DBL_MAX;
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) r = q < 3 ? fmin(r, red[q][k]) : fmax(r, red[q][k]);
        part[q * gridDim.x + blockIdx.x] = r;
    }
}

__device__ void set_root_box(TreeInfo *info, const double *mn, const double *mx);

// One block of kTB threads; min and max do not depend on the order of the
// partials, so the parallel reduction gives the same box as a serial one.
__global__ void __launch_bounds__(kTB) k_bbox_final(const double *__restrict__ part, int nb, TreeInfo *info) {
    __shared__ double red[6][kTB / 32];
    double v[6];
#pragma unroll
    for (int a = 0; a < 3; ++a) v[a] = DBL_MAX, v[3 + a] = -DBL_MAX;
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
        for (int a = 0; a < 3; ++a) v[a] = fmin(v[a], part[a * nb + b]), v[3 + a] = fmax(v[3 + a], part[(3 + a) * nb + b]);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        for (int o = 16; o; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, v[q], o);
            v[q] = q < 3 ? fmin(v[q], u) : fmax(v[q], u);
        }
        if (lane == 0) red[q][w] = v[q];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double mn[3], mx[3];
    for (int a = 0; a < 3; ++a) {
        mn[a] = DBL_MAX, mx[a] = -DBL_MAX;
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) mn[a] = fmin(mn[a], red[a][k]), mx[a] = fmax(mx[a], red[3 + a][k]);
    }
    set_root_box(info, mn, mx);
}

// Root box (padded by Problem::OCTREE_WIDTH_PADDING, problem.hpp:167) and
// the key parameters derived from it, from the particles' min and max.
__device__ void set_root_box(TreeInfo *info, const double *mn, const double *mx) {
    const double pad = 1e-5;
    double S = 0, margin = 0;
    for (int a = 0; a < 3; ++a) {
        info->root_min[a] = mn[a] - pad;
        info->root_max[a] = mx[a] + pad;
        info->H[a] = info->root_max[a] - info->root_min[a];
        S = fmax(S, info->H[a]);
        info->key_scale[a] = ldexp(1.0, kMaxLevel) / info->H[a];
        // Recursive FP64 midpoints stray from the ideal ones by at most
        // 21/2 ulp(max|bound|) and u = (x - lo) 2^21 / H carries about one more
        // ulp; in key units that is < 12 * 2^-52 * 2^21 * max|bound| / H.
        const double big = fmax(fabs(info->root_min[a]), fabs(info->root_max[a]));
        margin = fmax(margin, 64.0 * ldexp(big / info->H[a], -31) + ldexp(1.0, -30));
    }
    info->S = S;
    info->key_margin = margin;
    for (int a = 0; a < 3; ++a) {
        info->key_scale32[a] = ldexp(info->key_scale[a], 32);
        info->key_off32[a] = -info->root_min[a] * info->key_scale32[a];
        info->root_c[a] = (info->root_min[a] + info->root_max[a]) / 2;
    }
    info->key_mfrac = static_cast<unsigned long long>(ceil(ldexp(margin, 32))) + 1;
}

// Forest: one block per system, the same box as k_bbox_partial/final give
// for that system alone (min and max are exact), plus the system's particle
// mass and G m. An empty system gets the box of the origin (no particle
// uses it).
__global__ void __launch_bounds__(kTB) k_bbox_sys(const double *__restrict__ x, unsigned n, const unsigned *__restrict__ seg,
                                                  const double2 *__restrict__ sys_par, TreeInfo *info) {
    const int sidx = blockIdx.x;
    const unsigned b = seg[sidx], e = seg[sidx + 1];
    const long long kmax = ord_key(__double_as_longlong(DBL_MAX)), kmin = ord_key(__double_as_longlong(-DBL_MAX));
    long long kn[3] = {kmax, kmax, kmax}, kx[3] = {kmin, kmin, kmin};
    bool bad = false;
    for (unsigned i = b + threadIdx.x; i < e; i += blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const long long bits = __double_as_longlong(x[static_cast<size_t>(a) * n + i]);
            const bool fin = ((bits >> 52) & 0x7ff) != 0x7ff;
            bad |= !fin;
            const long long k = ord_key(bits);
            if (fin) kn[a] = min(kn[a], k), kx[a] = max(kx[a], k);
        }
    }
    if (bad) atomicOr(&info->err, kDevNonFinite);
    __shared__ long long red[6][kTB / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o; o >>= 1) {
            kn[a] = min(kn[a], __shfl_xor_sync(0xffffffffu, kn[a], o));
            kx[a] = max(kx[a], __shfl_xor_sync(0xffffffffu, kx[a], o));
        }
        if (lane == 0) red[a][w] = kn[a], red[3 + a][w] = kx[a];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double mn[3], mx[3];
    for (int a = 0; a < 3; ++a) {
        long long lo = red[a][0], hi = red[3 + a][0];
        for (int k = 1; k < kTB / 32; ++k) lo = min(lo, red[a][k]), hi = max(hi, red[3 + a][k]);
        // +-0 compare equal as doubles: either is the bound (the padding makes them the same)
        mn[a] = e > b ? __longlong_as_double(ord_key(lo)) : 0.0;
        mx[a] = e > b ? __longlong_as_double(ord_key(hi)) : 0.0;
    }
    TreeInfo *si = info + sidx;
    set_root_box(si, mn, mx);
    si->m = sys_par[sidx].x;
    si->gm = sys_par[sidx].y;
}

// Spread the 21 low bits of v to every third bit.
__device__ __forceinline__ uint64_t spread3(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// Child offsets of 21 levels of recursive midpoints (see file comment).
__device__ __forceinline__ uint64_t morton_key(const double *p, const TreeInfo *__restrict__ info) {
    // Fast path: every split decision of the 21 levels compares x with a
    // midpoint that sits at an integer of u = (x - lo) 2^21 / H up to the
    // rounding bounded by key_margin, so away from integers the child offsets
    // are the complemented bits of floor(u). u is taken in 32.32 fixed point,
    // q = trunc(fma(x, 2^32 scale, -lo 2^32 scale)): one FMA and one
    // conversion on the FP64 pipe, the rest integer. The FMA's error (about one
    // ulp of max|bound| in key units, plus 2^-33) lies well inside key_margin,
    // which allows 64 such ulps.
    {
        const unsigned long long mf = info->key_mfrac;
        bool ok = info->key_margin < 0.25;
        uint64_t k[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const long long q = __double2ll_rz(fma(p[a], info->key_scale32[a], info->key_off32[a]));
            const unsigned long long fr = static_cast<unsigned long long>(q) & 0xffffffffull;
            ok &= q >= 0 && q < (1LL << 53) && fr > mf && fr < (1ull << 32) - mf;
            k[a] = ok ? (~static_cast<uint64_t>(q >> 32)) & 0x1fffffull : 0;
        }
        if (ok) return spread3(k[0]) | (spread3(k[1]) << 1) | (spread3(k[2]) << 2);
    }
    double lo[3] = {info->root_min[0], info->root_min[1], info->root_min[2]};
    double hi[3] = {info->root_max[0], info->root_max[1], info->root_max[2]};
    uint64_t key = 0;
    for (int L = 1; L <= kMaxLevel; ++L) {
        unsigned dig = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double mid = (hi[a] + lo[a]) / 2;
            if (p[a] < mid) {
                dig |= 1u << a;
                hi[a] = mid;
            } else {
                lo[a] = mid;
            }
        }
        key = (key << 3) | dig;
    }
    return key;
}

__global__ void k_keys(const double *__restrict__ x, unsigned n, const TreeInfo *__restrict__ info,
                       uint64_t *__restrict__ keys, unsigned *__restrict__ perm, SortZero z) {
    sort_temp_zero(z);  // for the key sort that follows
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double p[3] = {x[i], x[static_cast<size_t>(n) + i], x[2 * static_cast<size_t>(n) + i]};
    keys[i] = morton_key(p, info);
    perm[i] = i;
}

// Forest: the Morton key of particle i in its own system's root box (kept in
// mkeys) and the sort word (system << 3 sorted | top `sorted` levels of the
// key), so that one stable sort orders every system's particles as a sort of
// that system alone would, systems in order.
__global__ void k_keys_forest(const double *__restrict__ x, unsigned n, const TreeInfo *__restrict__ info,
                              const int *__restrict__ psys, int sorted, uint64_t *__restrict__ words,
                              unsigned *__restrict__ perm, uint64_t *__restrict__ mkeys, SortZero z) {
    sort_temp_zero(z);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double p[3] = {x[i], x[static_cast<size_t>(n) + i], x[2 * static_cast<size_t>(n) + i]};
    const int sidx = psys[i];
    const uint64_t key = morton_key(p, info + sidx);
    mkeys[i] = key;
    words[i] = (static_cast<uint64_t>(sidx) << (3 * sorted)) | (key >> path_shift(sorted));
    perm[i] = i;
}

// Forest: the Morton keys in sorted order.
__global__ void k_forest_morton(const uint64_t *__restrict__ mkeys, const unsigned *__restrict__ perm, unsigned n,
                                uint64_t *__restrict__ keys) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) keys[j] = mkeys[perm[j]];
}

// Keys are sorted on their top `sorted` levels only (particles inside a leaf
// are put in index order afterwards, so deeper key bits never matter while no
// cell of level `sorted` has to split). A run whose level-`sorted` prefix
// still holds more than T particles asks for a deeper sort through counts[9].
// A forest (psys, seg non-null) treats each system's positions [seg[s],
// seg[s+1]) as a tree of its own: a system's first particle starts runs of
// every level, and no run reaches into the next system. Its sort words hold
// at most sorted_cap key levels; a system that needs more is an error.
__global__ void k_split_count(const uint64_t *__restrict__ keys, unsigned n, int T, int sorted, int sorted_cap,
                              const int *__restrict__ psys, const unsigned *__restrict__ seg, unsigned *__restrict__ cnt,
                              unsigned *counts, TreeInfo *info) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned sb = psys ? seg[psys[i]] : 0u, se = psys ? seg[psys[i] + 1] : n;
    const int Ls = i == sb ? 0 : first_diff_level(keys[i - 1], keys[i]);
    int Lm = -1;
    if (static_cast<unsigned long long>(i) + T < se) {
        Lm = first_diff_level(keys[i], keys[i + T]) - 1;
        if (Lm >= sorted && sorted < sorted_cap) {
            atomicMax(&counts[9], static_cast<unsigned>(min(sorted + 6, sorted_cap)));
            Lm = sorted - 1;
        } else if (Lm >= sorted && sorted < kMaxLevel) {  // a forest system deeper than its sort word
            atomicOr(&info->err, kDevForestDepth);
            Lm = sorted - 1;
        } else if (Lm >= kMaxLevel) {  // a deepest-level cell would still split
            atomicOr(&info->err, kDevDepth);
            Lm = kMaxLevel - 1;
        }
    }
    cnt[i] = Lm >= Ls ? static_cast<unsigned>(Lm - Ls + 1) : 0u;
}

// Split entries (level << 32 | first particle) at their scanned offsets. On
// an overflow of the split buffer or a too shallow key sort (seen by thread
// 0, which zeroes the count) the attempt builds a root-only tree (nothing
// addresses past a buffer) and the host repeats it.
__global__ void k_split_emit(const uint64_t *__restrict__ keys, unsigned n, int T, int sorted, const int *__restrict__ psys,
                             const unsigned *__restrict__ seg, const unsigned *__restrict__ off, unsigned *counts,
                             unsigned s_cap, uint64_t *__restrict__ ent, TreeInfo *info, SortZero z) {
    sort_temp_zero(z);  // for the entry sort that follows (the key sort is done with them)
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned total = counts[1];
    const bool over = total > s_cap || counts[9] != 0;
    if (i == 0) {
        counts[6] = total;  // requested size, kept for the host when it overflows
        if (over) atomicOr(&info->err, kDevCapacity), counts[1] = 0;
    }
    // a block that reads counts[1] after thread 0 zeroed it sees 0 and also writes nothing
    if (i >= n || over || total == 0) return;
    const unsigned sb = psys ? seg[psys[i]] : 0u, se = psys ? seg[psys[i] + 1] : n;
    const int Ls = i == sb ? 0 : first_diff_level(keys[i - 1], keys[i]);
    int Lm = -1;
    // (sorted - 1 caps Lm only where k_split_count reported an error)
    if (static_cast<unsigned long long>(i) + T < se)
        Lm = min(first_diff_level(keys[i], keys[i + T]) - 1, min(kMaxLevel, sorted) - 1);
    unsigned o = off[i];
    for (int L = Ls; L <= Lm; ++L, ++o)
        if (o < s_cap) ent[o] = (static_cast<uint64_t>(L) << 32) | i;
}

__device__ unsigned lower_bound_ent(const uint64_t *ent, unsigned lo, unsigned hi, uint64_t v) {
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (ent[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// first j in [lo, hi) with (keys[j] >> sh) >= v
__device__ unsigned lower_bound_pre(const uint64_t *keys, unsigned lo, unsigned hi, int sh, uint64_t v) {
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if ((keys[mid] >> sh) < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__device__ void path_geometry(uint64_t path, int L, const TreeInfo *info, double *box, double *ctr, int *coord);

// One warp: lane L finds level L's split entries (ent is sorted by level),
// then the cell counts and starts of every level follow by a warp scan.
// A forest has nroots roots at level 0 (cells 0 .. nroots-1, set up by
// k_roots); one tree has the root cell set up here.
__global__ void k_level_table(const uint64_t *__restrict__ ent, unsigned *counts, TreeInfo *info, unsigned n, int T, int nroots,
                              int *c_begin, int *c_end, int *c_parent, int *c_child, int *c_level, uint64_t *c_path,
                              int *c_coord, double *c_box, double *c_ctr, int *p2p_own, int *p2p_cnt, int *coll,
                              int *coll_cnt) {
    static_assert(kMaxLevel + 2 <= 32, "one lane per level");
    const int L = static_cast<int>(threadIdx.x);
    if (L >= 32) return;
    const unsigned S = counts[1];
    unsigned split = 0;
    if (L <= kMaxLevel) {
        const unsigned a = lower_bound_ent(ent, 0, S, static_cast<uint64_t>(L) << 32);
        const unsigned b = lower_bound_ent(ent, 0, S, static_cast<uint64_t>(L + 1) << 32);
        info->split_start[L] = static_cast<int>(a);
        info->split_count[L] = static_cast<int>(b - a);
        split = b - a;
    }
    // cells of level L: 1 at the root, 8 per split cell of level L - 1
    const unsigned below = __shfl_up_sync(0xffffffffu, split, 1);
    const bool lv = L <= kMaxLevel + 1;
    const int cnt = !lv ? 0 : (L == 0 ? nroots : 8 * static_cast<int>(below));
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (L >= o) incl += y;
    }
    if (lv) info->level_count[L] = cnt, info->level_start[L] = incl - cnt;
    const int start = __shfl_sync(0xffffffffu, incl, kMaxLevel + 1);  // all cells
    const int start2 = __shfl_sync(0xffffffffu, incl - cnt, 2);
    const unsigned nonempty = __ballot_sync(0xffffffffu, lv && cnt > 0);
    if (L == 0) {
        const int depth = 31 - __clz(static_cast<int>(nonempty));
        info->ncells = start;
        info->nsplit_total = static_cast<int>(S);
        info->nleaves = start - static_cast<int>(S);
        info->depth = depth;
        info->n_targets_m2l = depth >= 2 ? start - start2 : 0;
        counts[2] = static_cast<unsigned>(start);
        counts[3] = static_cast<unsigned>(start) - S;
        if (nroots != 1) return;
        // the root cell
        c_begin[0] = 0;
        c_end[0] = static_cast<int>(n);
        c_parent[0] = -1;
        c_level[0] = 0;
        c_path[0] = 0;
        const bool split = static_cast<long long>(n) > T;
        c_child[0] = split ? 1 : -1;
        path_geometry(0, 0, info, c_box, c_ctr, c_coord);
        // calc_link at the root (solver_ref.hpp:148-154)
        if (split) {
            coll[0] = 0, coll_cnt[0] = 1, p2p_cnt[0] = 0;
        } else {
            p2p_own[0] = 0, p2p_cnt[0] = 1, coll_cnt[0] = 0;
        }
    }
}

__device__ void path_geometry(uint64_t path, int L, const TreeInfo *info, double *box, double *ctr, int *coord) {
    double lo[3] = {info->root_min[0], info->root_min[1], info->root_min[2]};
    double hi[3] = {info->root_max[0], info->root_max[1], info->root_max[2]};
    int c[3] = {0, 0, 0};
    for (int l = 1; l <= L; ++l) {
        const unsigned dig = static_cast<unsigned>(path >> (3 * (L - l))) & 7u;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double mid = (hi[a] + lo[a]) / 2;
            const int lower = (dig >> a) & 1;
            if (lower)
                hi[a] = mid;
            else
                lo[a] = mid;
            c[a] = 2 * c[a] + (1 - lower);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        box[a] = lo[a];
        box[3 + a] = hi[a];
        ctr[a] = (lo[a] + hi[a]) / 2;
        coord[a] = c[a];
    }
}


// Forest roots: cell k is system k's root, its particles seg[k] .. seg[k+1],
// its box the system's root box; calc_link at each root as at a single tree's
// (solver_ref.hpp:148-154).
__global__ void k_roots(const uint64_t *__restrict__ ent, const unsigned *__restrict__ seg, int nsys, int T,
                        const TreeInfo *__restrict__ info, int *c_begin, int *c_end, int *c_parent, int *c_child,
                        int *c_level, uint64_t *c_path, int *c_coord, double *c_box, double *c_ctr, int *c_sys,
                        int *p2p_own, int *p2p_cnt, int *coll, int *coll_cnt) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nsys; r += gridDim.x * blockDim.x) {
        const unsigned b = seg[r], e = seg[r + 1];
        c_begin[r] = static_cast<int>(b);
        c_end[r] = static_cast<int>(e);
        c_parent[r] = -1;
        c_level[r] = 0;
        c_path[r] = 0;
        c_sys[r] = r;
        const bool split = static_cast<long long>(e) - b > T;
        int fc = -1;
        if (split) {  // its level-0 split entry is (0, b); the entries of level 0 are in system order
            const unsigned a = static_cast<unsigned>(info->split_start[0]);
            const unsigned rk = lower_bound_ent(ent, a, a + static_cast<unsigned>(info->split_count[0]), b) - a;
            fc = info->level_start[1] + 8 * static_cast<int>(rk);
        }
        c_child[r] = fc;
        path_geometry(0, 0, info + r, c_box + 6 * static_cast<size_t>(r), c_ctr + 3 * static_cast<size_t>(r),
                      c_coord + 3 * static_cast<size_t>(r));
        const size_t o = static_cast<size_t>(r) * kNbrCap;
        if (split) {
            coll[o] = r, coll_cnt[r] = 1, p2p_cnt[r] = 0;
        } else {
            p2p_own[o] = r, p2p_cnt[r] = 1, coll_cnt[r] = 0;
        }
    }
}

// One thread per (split cell, child octant): the 8 threads of a split cell
// find its number and particle range (the same searches, in one warp), then
// each its child's range, links and geometry.
// In a forest (psys non-null) the searches stay inside the entry's system,
// whose root is cell psys[i], and every child records its system.
__global__ void k_cells(const uint64_t *__restrict__ ent, const unsigned *counts, const uint64_t *__restrict__ keys,
                        unsigned n, int T, const TreeInfo *__restrict__ info, const int *__restrict__ psys,
                        const unsigned *__restrict__ seg, int *split_cell, int *c_begin, int *c_end, int *c_parent,
                        int *c_child, int *c_level, uint64_t *c_path, int *c_coord, double *c_box, double *c_ctr,
                        int *c_sys) {
    const unsigned S = counts[1];
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < 8u * S; t += gridDim.x * blockDim.x) {
        const unsigned e = t >> 3;
        const int o = static_cast<int>(t & 7u);
        const int L = static_cast<int>(ent[e] >> 32);
        const unsigned i = static_cast<unsigned>(ent[e] & 0xffffffffu);
        const unsigned r = e - static_cast<unsigned>(info->split_start[L]);
        const int sh = path_shift(L);
        const uint64_t pre = L == 0 ? 0 : (keys[i] >> sh);
        const int sidx = psys ? psys[i] : 0;
        const unsigned sb = psys ? seg[sidx] : 0u, se = psys ? seg[sidx + 1] : n;
        int own = sidx;
        if (L > 0) {
            const int shp = path_shift(L - 1);
            const unsigned ip = lower_bound_pre(keys, sb, i, shp, keys[i] >> shp);
            const unsigned a = static_cast<unsigned>(info->split_start[L - 1]);
            const unsigned b = a + static_cast<unsigned>(info->split_count[L - 1]);
            const unsigned rp = lower_bound_ent(ent, a, b, (static_cast<uint64_t>(L - 1) << 32) | ip) - a;
            own = info->level_start[L] + 8 * static_cast<int>(rp) + static_cast<int>(pre & 7u);
        }
        if (o == 0) split_cell[e] = own;
        const unsigned pe = L == 0 ? se : lower_bound_pre(keys, i + 1, se, sh, pre + 1);
        const int shc = path_shift(L + 1);
        const unsigned a1 = static_cast<unsigned>(info->split_start[L + 1]);
        const unsigned b1 = a1 + static_cast<unsigned>(info->split_count[L + 1]);
        {
            // [i, pe) is sorted on the child prefix, so each child's bounds are
            // lower bounds over the whole range
            const uint64_t cpath = (pre << 3) | static_cast<uint64_t>(o);
            const unsigned cb = o == 0 ? i : lower_bound_pre(keys, i, pe, shc, cpath);
            const unsigned ce = o == 7 ? pe : lower_bound_pre(keys, i, pe, shc, cpath + 1);
            const int c = info->level_start[L + 1] + 8 * static_cast<int>(r) + o;
            c_begin[c] = static_cast<int>(cb);
            c_end[c] = static_cast<int>(ce);
            c_parent[c] = own;
            c_level[c] = L + 1;
            c_path[c] = cpath;
            int fc = -1;
            if (static_cast<long long>(ce) - cb > T && L + 1 <= kMaxLevel - 1) {
                const unsigned rc = lower_bound_ent(ent, a1, b1, (static_cast<uint64_t>(L + 1) << 32) | cb) - a1;
                fc = info->level_start[L + 2] + 8 * static_cast<int>(rc);
            }
            c_child[c] = fc;
            if (c_sys) c_sys[c] = sidx;
            path_geometry(cpath, L + 1, info + sidx, c_box + 6 * static_cast<size_t>(c), c_ctr + 3 * static_cast<size_t>(c),
                          c_coord + 3 * static_cast<size_t>(c));
        }
    }
}

__global__ void k_leaf_flags(const int *__restrict__ c_child, const unsigned *counts, unsigned *flag) {
    const unsigned C = counts[2];
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) flag[c] = c_child[c] < 0;
}

// The leaves in cell order by one block (smaller trees: one launch instead of
// flags, scan and compaction).
__global__ void __launch_bounds__(1024) k_leaf_list(const int *__restrict__ c_child, const unsigned *counts, int *leaves) {
    __shared__ unsigned wsum[32];
    const unsigned C = counts[2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned base = 0;
    for (unsigned start = 0; start < C; start += 4 * blockDim.x) {
        const unsigned c0 = start + 4 * threadIdx.x;
        unsigned f[4], s = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            f[j] = (c0 + j < C && c_child[c0 + j] < 0) ? 1u : 0u;
            s += f[j];
        }
        unsigned incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        if (w == 0) {
            unsigned v = lane < nw ? wsum[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += y;
            }
            if (lane < nw) wsum[lane] = v;
        }
        __syncthreads();
        unsigned pos = base + (w ? wsum[w - 1] : 0u) + incl - s;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (f[j]) leaves[pos++] = static_cast<int>(c0 + j);
        base += wsum[nw - 1];
        __syncthreads();  // wsum is reused by the next chunk
    }
}

__global__ void k_leaf_compact(const unsigned *__restrict__ flag, const unsigned *__restrict__ off, const unsigned *counts,
                               int *leaves) {
    const unsigned C = counts[2];
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x)
        if (flag[c]) leaves[off[c]] = static_cast<int>(c);
}

// Within a leaf the reference keeps insertion order, i.e. ascending particle
// index (octree.hpp:143-145). Rank sort of each leaf's permutation slice.
__global__ void k_leaf_sort(const int *__restrict__ leaves, const unsigned *counts, const int *__restrict__ c_begin,
                            const int *__restrict__ c_end, int T, unsigned *perm) {
    extern __shared__ unsigned sh[];  // per warp: 2 (T + 1)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned *in = sh + static_cast<size_t>(w) * 2 * (T + 1), *out = in + (T + 1);
    const unsigned NL = counts[3];
    for (unsigned li = blockIdx.x * nw + w; li < NL; li += gridDim.x * nw) {  // a warp per leaf
        const int c = leaves[li];
        const int b = c_begin[c], e = c_end[c], len = e - b;
        if (len < 2 || len > T) continue;  // uniform per warp
        for (int k = lane; k < len; k += 32) in[k] = perm[b + k];
        __syncwarp();
        for (int k = lane; k < len; k += 32) {
            const unsigned v = in[k];
            int rank = 0;
            for (int q = 0; q < len; ++q) rank += in[q] < v;
            out[rank] = v;
        }
        __syncwarp();
        for (int k = lane; k < len; k += 32) perm[b + k] = out[k];
        __syncwarp();
    }
}

// Positions in tree order; the FP32 hi/lo pairs relative to the root-box
// centre (a forest: the system's, with the system's particle mass).
__global__ void k_gather(const double *__restrict__ x, unsigned n, const unsigned *__restrict__ perm,
                         const TreeInfo *__restrict__ info_all, const int *__restrict__ psys, float mass_f,
                         double *__restrict__ xs, float4 *__restrict__ ph, float4 *__restrict__ pl, unsigned *__restrict__ inv) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const TreeInfo *info = psys ? info_all + psys[j] : info_all;
    if (psys) mass_f = static_cast<float>(info->m);
    const unsigned i = perm[j];
    inv[i] = j;
    double d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double v = x[static_cast<size_t>(a) * n + i];
        xs[static_cast<size_t>(a) * n + j] = v;
        d[a] = v - info->root_c[a];
    }
    const float hx = static_cast<float>(d[0]), hy = static_cast<float>(d[1]), hz = static_cast<float>(d[2]);
    ph[j] = make_float4(hx, hy, hz, mass_f);
    pl[j] = make_float4(static_cast<float>(d[0] - hx), static_cast<float>(d[1] - hy), static_cast<float>(d[2] - hz), 0.f);
}

// One warp per non-leaf cell P: its 27 same-level neighbours, then for each of
// its 8 children the colleague, own-p2p and M2L entries (solver_ref.hpp:129-147).
// In a forest a level holds the systems' cells in system order, path order
// inside each: neighbours are searched by (system, path).
__global__ void k_lists(const uint64_t *__restrict__ ent, const unsigned *counts, const int *__restrict__ split_cell,
                        const TreeInfo *__restrict__ info, const int *__restrict__ c_child,
                        const uint64_t *__restrict__ c_path, const int *__restrict__ c_coord, const int *__restrict__ c_sys,
                        int *m2l_src, int *p2p_own, int *p2p_cnt, int *coll, int *coll_cnt, unsigned long long *m2l_pairs) {
    __shared__ int nb[8][32], ord[8][32], nord[8];
    __shared__ int uch[8][27 * 8];  // per neighbour (in order) and octant: child u, or ~u if u is a leaf
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned S = counts[1];
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    unsigned long long pairs = 0;  // M2L pairs of this lane's cells, added once per warp below
    for (unsigned e = blockIdx.x * (blockDim.x >> 5) + w; e < S; e += warps) {
        const int L = static_cast<int>(ent[e] >> 32);
        const int P = split_cell[e];
        const int fcP = c_child[P];
        int q = -1;
        if (lane < 27) {
            const int d[3] = {lane % 3 - 1, (lane / 3) % 3 - 1, lane / 9 - 1};
            int qc[3];
            bool in = true;
            const int lim = 1 << L;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                qc[a] = c_coord[3 * P + a] + d[a];
                in &= qc[a] >= 0 && qc[a] < lim;
            }
            if (in) {
                uint64_t path = 0;
                for (int l = 1; l <= L; ++l) {
                    unsigned dig = 0;
#pragma unroll
                    for (int a = 0; a < 3; ++a) dig |= static_cast<unsigned>(1 - ((qc[a] >> (L - l)) & 1)) << a;
                    path = (path << 3) | dig;
                }
                const int sP = cell_system(c_sys, P);
                int lo = info->level_start[L], hi = lo + info->level_count[L];
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    const int sm = cell_system(c_sys, mid);
                    if (sm < sP || (sm == sP && c_path[mid] < path))
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                if (lo < info->level_start[L] + info->level_count[L] && cell_system(c_sys, lo) == sP && c_path[lo] == path &&
                    c_child[lo] >= 0)
                    q = lo;
            }
        }
        nb[w][lane] = q;
        __syncwarp();
        // order the existing neighbours by cell number (= path order)
        if (lane < 27 && q >= 0) {
            int rank = 0;
            for (int k = 0; k < 27; ++k) {
                const int o = nb[w][k];
                rank += (o >= 0 && o < q);
            }
            ord[w][rank] = lane;
        }
        const unsigned ballot = __ballot_sync(0xffffffffu, lane < 27 && q >= 0);
        if (lane == 0) nord[w] = __popc(ballot);
        // every child's 216 M2L slots start empty
        for (int k = lane; k < 8 * kM2LSlots; k += 32) m2l_src[static_cast<size_t>(fcP + k / kM2LSlots) * kM2LSlots + k % kM2LSlots] = -1;
        __syncwarp();
        // the neighbours' children, loaded once by the whole warp
        for (int idx = lane; idx < 8 * nord[w]; idx += 32) {
            const int u = c_child[nb[w][ord[w][idx >> 3]]] + (idx & 7);
            uch[w][idx] = c_child[u] >= 0 ? u : ~u;
        }
        __syncwarp();
        if (lane < 8) {
            const int c = fcP + lane;
            const int uc[3] = {1 - (lane & 1), 1 - ((lane >> 1) & 1), 1 - ((lane >> 2) & 1)};
            const bool cleaf = c_child[c] < 0;
            int ncoll = 0, np2p = 0;
            unsigned nm2l = 0;
            for (int k = 0; k < nord[w]; ++k) {
                const int dd = ord[w][k];
                const int d[3] = {dd % 3 - 1, (dd / 3) % 3 - 1, dd / 9 - 1};
                for (int o = 0; o < 8; ++o) {
                    const int code = uch[w][8 * k + o];
                    const int u = code >= 0 ? code : ~code;
                    const bool usplit = code >= 0;
                    const int uo[3] = {1 - (o & 1), 1 - ((o >> 1) & 1), 1 - ((o >> 2) & 1)};
                    bool adj = true;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const int off = 2 * d[a] + uo[a] - uc[a];
                        adj &= off >= -1 && off <= 1;
                    }
                    if (adj) {
                        if (!cleaf && usplit)
                            coll[static_cast<size_t>(c) * kNbrCap + ncoll++] = u;
                        else
                            p2p_own[static_cast<size_t>(c) * kNbrCap + np2p++] = u;
                    } else {
                        m2l_src[static_cast<size_t>(c) * kM2LSlots + dd * 8 + o] = u;
                        ++nm2l;
                    }
                }
            }
            coll_cnt[c] = ncoll;
            p2p_cnt[c] = np2p;
            if (L + 1 >= 2) pairs += nm2l;
        }
        __syncwarp();
    }
    // one atomic per warp: the same counter from every cell serialised the kernel
#pragma unroll
    for (int o = 16; o; o >>= 1) pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    if (lane == 0 && pairs) atomicAdd(m2l_pairs, pairs);
}

// Near-field source ranges of every leaf: the own-p2p entries of its
// ancestors from the root down, then its own (the inherited list of
// solver_ref.hpp:126 followed by the cell's additions). Each entry is a
// subtree, i.e. a contiguous particle range in tree order.
__global__ void k_rng_count(const int *__restrict__ leaves, const unsigned *counts, const int *__restrict__ c_parent,
                            const int *__restrict__ c_begin, const int *__restrict__ c_end,
                            const int *__restrict__ p2p_own, const int *__restrict__ p2p_cnt, unsigned *rng_cnt,
                            unsigned *chunk_cnt, unsigned *src_total, unsigned *part_cnt, unsigned slice) {
    const unsigned NL = counts[3];
    for (unsigned li = blockIdx.x * blockDim.x + threadIdx.x; li < NL; li += gridDim.x * blockDim.x) {
        const int c = leaves[li];
        const int nt = c_end[c] - c_begin[c];
        unsigned tot = 0;
        unsigned long long srcs = 0;
        if (nt > 0)
            for (int a = c; a >= 0; a = c_parent[a]) {
                tot += static_cast<unsigned>(p2p_cnt[a]);
                for (int q = 0; q < p2p_cnt[a]; ++q) {
                    const int u = p2p_own[static_cast<size_t>(a) * kNbrCap + q];
                    srcs += static_cast<unsigned>(c_end[u] - c_begin[u]);
                }
            }
        rng_cnt[li] = tot;
        const unsigned ns = nt > 0 ? static_cast<unsigned>(slice_count(srcs, slice)) : 1u;
        chunk_cnt[li] = static_cast<unsigned>(chunk_count(nt)) * ns;
        part_cnt[li] = ns > 1 ? static_cast<unsigned>(chunk_count(nt)) * ns : 0u;
        src_total[li] = static_cast<unsigned>(srcs < 0xffffffffull ? srcs : 0xffffffffull);
    }
}

// Thread 0 first checks the near-field totals against the buffers: on any
// overflow the evaluation queues no P2P work item at all (this kernel may still
// address items whose partial-sum slot lies past part_cap, and the P2P kernels
// run before the host sees the flag, grows the buffers and repeats the
// evaluation).
__global__ void k_rng_fill(const int *__restrict__ leaves, unsigned *counts, unsigned r_cap, unsigned ch_cap,
                           const int *__restrict__ c_parent, const int *__restrict__ c_begin, const int *__restrict__ c_end,
                           const int *__restrict__ p2p_own, const int *__restrict__ p2p_cnt,
                           const unsigned *__restrict__ rng_off, unsigned *rng_len, uint2 *ranges,
                           const unsigned *__restrict__ chunk_off, int4 *chunks, const unsigned *__restrict__ src_total,
                           const unsigned *__restrict__ part_off, unsigned part_cap, TreeInfo *info, unsigned slice) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counts[7] = counts[5];  // requested sizes, kept for the host when they overflow
        const bool over = counts[4] > r_cap || counts[5] > ch_cap || counts[8] > part_cap;
        if (over) atomicOr(&info->err, kDevCapacity);
        counts[5] = over ? 0u : counts[5];
        info->n_p2p_chunks = static_cast<int>(counts[5]);
    }
    const unsigned NL = counts[3];
    unsigned long long pairs = 0, nranges = 0;  // this thread's totals, added once per warp below
    for (unsigned li = blockIdx.x * blockDim.x + threadIdx.x; li < NL; li += gridDim.x * blockDim.x) {
        const int c = leaves[li];
        const int b = c_begin[c], e = c_end[c];
        if (e == b) {
            rng_len[li] = 0;
            continue;
        }
        int anc[kMaxLevel + 2];
        int na = 0;
        for (int a = c; a >= 0 && na < kMaxLevel + 2; a = c_parent[a]) anc[na++] = a;
        const unsigned base = rng_off[li];
        unsigned k = 0;
        unsigned long long srcs = 0;
        uint2 last = make_uint2(0, 0);
        bool have = false, overflow = false;
        for (int t = na - 1; t >= 0; --t) {
            const int a = anc[t];
            for (int q = 0; q < p2p_cnt[a]; ++q) {
                const int u = p2p_own[static_cast<size_t>(a) * kNbrCap + q];
                const unsigned ub = static_cast<unsigned>(c_begin[u]), ue = static_cast<unsigned>(c_end[u]);
                if (ue == ub) continue;
                srcs += ue - ub;
                if (have && last.y == ub) {
                    last.y = ue;
                } else {
                    if (have) {
                        if (base + k < r_cap)
                            ranges[base + k] = last;
                        else
                            overflow = true;
                        ++k;
                    }
                    last = make_uint2(ub, ue);
                    have = true;
                }
            }
        }
        if (have) {
            if (base + k < r_cap)
                ranges[base + k] = last;
            else
                overflow = true;
            ++k;
        }
        rng_len[li] = overflow ? 0u : k;  // never let P2P read past the buffer
        const unsigned cb = chunk_off[li];
        const int nch = chunk_count(e - b);
        const int ns = slice_count(src_total[li], slice);
        for (int q = 0; q < nch; ++q) {
            int off, len;
            chunk_at(e - b, q, off, len);
            for (int sl = 0; sl < ns; ++sl) {
                const unsigned it = cb + static_cast<unsigned>(q * ns + sl);
                // split items keep their partial sums in part[pslot]
                const unsigned pslot = ns > 1 ? part_off[li] + static_cast<unsigned>(q * ns + sl) : 0xffffffffu;
                if (ns > 1 && pslot >= part_cap) overflow = true;
                if (it < ch_cap)
                    chunks[it] = make_int4(static_cast<int>(li), b + off, item_pack(len, sl, ns), static_cast<int>(pslot));
                else
                    overflow = true;
            }
        }
        if (overflow) atomicOr(&info->err, kDevCapacity);
        pairs += static_cast<unsigned long long>(e - b) * srcs;
        nranges += k;
    }
    // one atomic per warp and counter (per-leaf atomics on two addresses serialised the kernel)
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
        nranges += __shfl_xor_sync(0xffffffffu, nranges, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (pairs) atomicAdd(reinterpret_cast<unsigned long long *>(&info->p2p_pairs), pairs);
        if (nranges) atomicAdd(reinterpret_cast<unsigned long long *>(&info->p2p_ranges), nranges);
    }
}

// Start of an evaluation (one block): TreeInfo and the device counters zeroed,
// counts[0] = n, the near-field work queue emptied; a kernel rather than host
// copies or memsets, so the whole evaluation is one short graph section.
__global__ void k_eval_begin(TreeInfo *info, unsigned *counts, unsigned n, unsigned *queue) {
    static_assert(sizeof(TreeInfo) % sizeof(unsigned) == 0, "TreeInfo in words");
    unsigned *iw = reinterpret_cast<unsigned *>(info);
    for (unsigned k = threadIdx.x; k < sizeof(TreeInfo) / sizeof(unsigned); k += blockDim.x) iw[k] = 0;
    for (unsigned k = threadIdx.x; k < static_cast<unsigned>(kNumCounts); k += blockDim.x) counts[k] = k == 0 ? n : 0u;
    if (threadIdx.x == 0) *queue = 0;
}

inline unsigned grid_for(unsigned n, int tb) { return (n + tb - 1) / tb; }

// ---------------------------------------------------------------- forest tiles
// The M2M/L2L and M2L kernels apply one operator to a tile of cells, and a
// forest's operators are per system (each system has its own root box), so
// every tile holds cells of one system. M2M/L2L tiles: runs of one level's
// split entries of one system (the entries of a level ascend by particle,
// hence by system) cut into tiles of kEntTile. M2L tiles: the target octets
// (8 sibling cells at level >= 2) of one system, listed system by system, cut
// into tiles of `rows` octets.
constexpr int kEntTile = 64;

__device__ __forceinline__ int ent_system(const uint64_t *ent, const int *psys, unsigned e) {
    return psys[static_cast<unsigned>(ent[e] & 0xffffffffu)];
}

// first e in [lo, hi) whose system is >= sv
__device__ unsigned lower_bound_system(const uint64_t *ent, const int *psys, unsigned lo, unsigned hi, int sv) {
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (ent_system(ent, psys, mid) < sv)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_etile_flag(const uint64_t *__restrict__ ent, const unsigned *counts, const int *__restrict__ psys,
                             const TreeInfo *__restrict__ info, unsigned *flag) {
    const unsigned S = counts[1];
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < S; e += gridDim.x * blockDim.x) {
        const int L = static_cast<int>(ent[e] >> 32);
        const unsigned rs = lower_bound_system(ent, psys, static_cast<unsigned>(info->split_start[L]), e, ent_system(ent, psys, e));
        flag[e] = (e - rs) % kEntTile == 0 ? 1u : 0u;
    }
}

__global__ void k_etile_fill(const uint64_t *__restrict__ ent, const unsigned *counts, const int *__restrict__ psys,
                             const unsigned *__restrict__ flag, const unsigned *__restrict__ off, TreeInfo *info, int2 *etile) {
    const unsigned S = counts[1];
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < S; e += gridDim.x * blockDim.x) {
        const int L = static_cast<int>(ent[e] >> 32);
        const unsigned a = static_cast<unsigned>(info->split_start[L]), b = a + static_cast<unsigned>(info->split_count[L]);
        if (flag[e]) {
            const unsigned re = lower_bound_system(ent, psys, e, b, ent_system(ent, psys, e) + 1);
            etile[off[e]] = make_int2(static_cast<int>(e), static_cast<int>(min(re - e, static_cast<unsigned>(kEntTile))));
        }
        if (e == a) info->etile_start[L] = static_cast<int>(off[e]);
        if (e + 1 == b) info->etile_end[L] = static_cast<int>(off[e] + flag[e]);
    }
}

__global__ void k_oct_count(const TreeInfo *__restrict__ info, const int *__restrict__ c_sys, unsigned *ocnt) {
    const int base = info->level_start[2], O = info->n_targets_m2l / 8;
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < O; o += gridDim.x * blockDim.x) atomicAdd(&ocnt[c_sys[base + 8 * o]], 1u);
}

// Exclusive scan of one value per thread over a block of 1024 threads.
__device__ unsigned block_scan_excl(unsigned v, unsigned *wsum, unsigned &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        unsigned x = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        wsum[lane] = x;
    }
    __syncthreads();
    const unsigned r = (w ? wsum[w - 1] : 0u) + incl - v;
    total = wsum[31];
    __syncthreads();
    return r;
}

// One block of 1024 threads, each a contiguous range of systems: list
// offsets, tiles, and the fill cursors zeroed.
__global__ void __launch_bounds__(1024) k_oct_plan(int nsys, int rows, unsigned *ocnt, TreeInfo *info, int4 *otile) {
    __shared__ unsigned wsum[32];
    const int per = (nsys + 1023) / 1024;
    const int s0 = min(nsys, static_cast<int>(threadIdx.x) * per), s1 = min(nsys, s0 + per);
    unsigned octs = 0, tiles = 0;
    for (int s = s0; s < s1; ++s) octs += ocnt[s], tiles += (ocnt[s] + rows - 1) / rows;
    unsigned tot_o, tot_t;
    unsigned oo = block_scan_excl(octs, wsum, tot_o);
    unsigned to = block_scan_excl(tiles, wsum, tot_t);
    for (int s = s0; s < s1; ++s) {
        const unsigned c = ocnt[s];
        ocnt[nsys + s] = oo;
        ocnt[2 * nsys + s] = 0;
        for (unsigned k = 0; k * rows < c; ++k)
            otile[to++] = make_int4(s, static_cast<int>(oo + k * rows), static_cast<int>(min(static_cast<unsigned>(rows), c - k * rows)), 0);
        oo += c;
    }
    if (threadIdx.x == 0) info->n_otiles = static_cast<int>(tot_t);
}

__global__ void k_oct_fill(const TreeInfo *__restrict__ info, const int *__restrict__ c_sys, int nsys, unsigned *ocnt,
                           int *oct_list) {
    const int base = info->level_start[2], O = info->n_targets_m2l / 8;
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < O; o += gridDim.x * blockDim.x) {
        const int sidx = c_sys[base + 8 * o];
        oct_list[ocnt[nsys + sidx] + atomicAdd(&ocnt[2 * nsys + sidx], 1u)] = o;
    }
}

}  // namespace

void forest_tiles(Workspace &ws, int rows) {
    cudaStream_t st = ws.st;
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 4, ceil_div(ws.c_cap, kTB));
    k_etile_flag<<<gs, kTB, 0, st>>>(ws.ent, ws.d_counts, ws.psys, ws.info, ws.flag);
    scan_exclusive_u32(ws.flag, ws.flag_off, ws.s_cap, ws.d_counts + 1, ws.d_counts + 10, ws.scan, st, &ws.launches);
    k_etile_fill<<<gs, kTB, 0, st>>>(ws.ent, ws.d_counts, ws.psys, ws.flag, ws.flag_off, ws.info, ws.etile);
    cudaMemsetAsync(ws.ocnt, 0, sizeof(unsigned) * ws.nsys, st);
    k_oct_count<<<gs, kTB, 0, st>>>(ws.info, ws.c_sys, ws.ocnt);
    k_oct_plan<<<1, 1024, 0, st>>>(ws.nsys, rows, ws.ocnt, ws.info, ws.otile);
    k_oct_fill<<<gs, kTB, 0, st>>>(ws.info, ws.c_sys, ws.nsys, ws.ocnt, ws.oct_list);
    ws.launches += 5;
}

void build_tree(Workspace &ws) {
    const unsigned n = ws.n;
    cudaStream_t st = ws.st;
    timer_begin(ws, kTTree);
    k_eval_begin<<<1, 128, 0, st>>>(ws.info, ws.d_counts, n, ws.queue);
    const bool forest = ws.forest();
    if (!forest) {
        const int nb = 2 * ws.num_sms;
        double *part = ws.bbox_part;
        k_bbox_partial<<<nb, kTB, 0, st>>>(ws.x, n, part, ws.info);
        k_bbox_final<<<1, kTB, 0, st>>>(part, nb, ws.info);
        const int kbit = 3 * (kMaxLevel - ws.sort_levels);
        k_keys<<<grid_for(n, kTB), kTB, 0, st>>>(ws.x, n, ws.info, ws.keys0, ws.perm0,
                                                 sort_zero_plan(ws.sort, n, kbit, 3 * kMaxLevel));
        ws.launches += 4;
        const int res = radix_sort_u64(ws.keys0, ws.perm0, ws.keys1, ws.perm1, n, nullptr, kbit, 3 * kMaxLevel, ws.sort, st,
                                       &ws.launches, &ws.info->err, kDevTimeout, true, ws.sort_spin_max);
        ws.keys = res ? ws.keys1 : ws.keys0;
        ws.perm = res ? ws.perm1 : ws.perm0;
    } else {
        // every system's box, then one sort of (system, key prefix) words and
        // the Morton keys gathered into sorted order (into the other key buffer)
        k_bbox_sys<<<ws.nsys, kTB, 0, st>>>(ws.x, n, ws.seg, ws.sys_par, ws.info);
        const int wbits = 3 * ws.sort_levels + ws.sys_bits;
        k_keys_forest<<<grid_for(n, kTB), kTB, 0, st>>>(ws.x, n, ws.info, ws.psys, ws.sort_levels, ws.keys0, ws.perm0,
                                                        ws.mkeys, sort_zero_plan(ws.sort, n, 0, wbits));
        ws.launches += 3;
        const int res = radix_sort_u64(ws.keys0, ws.perm0, ws.keys1, ws.perm1, n, nullptr, 0, wbits, ws.sort, st,
                                       &ws.launches, &ws.info->err, kDevTimeout, true, ws.sort_spin_max);
        ws.perm = res ? ws.perm1 : ws.perm0;
        ws.keys = res ? ws.keys0 : ws.keys1;
        k_forest_morton<<<grid_for(n, kTB), kTB, 0, st>>>(ws.mkeys, ws.perm, n, ws.keys);
        ws.launches += 1;
    }
    const int *psys = forest ? ws.psys : nullptr;
    const unsigned *seg = forest ? ws.seg : nullptr;
    // split cells of every level
    k_split_count<<<grid_for(n, kTB), kTB, 0, st>>>(ws.keys, n, ws.T, ws.sort_levels, forest ? ws.sort_levels_cap() : kMaxLevel,
                                                    psys, seg, ws.cnt, ws.d_counts, ws.info);
    scan_exclusive_u32(ws.cnt, ws.off, n, nullptr, ws.d_counts + 1, ws.scan, st, &ws.launches);
    k_split_emit<<<grid_for(n, kTB), kTB, 0, st>>>(ws.keys, n, ws.T, ws.sort_levels, psys, seg, ws.off, ws.d_counts,
                                                   ws.s_cap, ws.ent0, ws.info, sort_zero_plan(ws.sort, ws.s_cap, 32, 40));
    ws.launches += 2;
    const int re = radix_sort_u64(ws.ent0, nullptr, ws.ent1, nullptr, ws.s_cap, ws.d_counts + 1, 32, 40, ws.sort, st,
                                  &ws.launches, &ws.info->err, kDevTimeout, true, ws.sort_spin_max);
    ws.ent = re ? ws.ent1 : ws.ent0;
    k_level_table<<<1, 32, 0, st>>>(ws.ent, ws.d_counts, ws.info, n, ws.T, forest ? ws.nsys : 1, ws.c_begin, ws.c_end,
                                    ws.c_parent, ws.c_child, ws.c_level, ws.c_path, ws.c_coord, ws.c_box, ws.c_ctr,
                                    ws.p2p_own, ws.p2p_cnt, ws.coll, ws.coll_cnt);
    if (forest) {
        k_roots<<<grid_for(ws.nsys, kTB), kTB, 0, st>>>(ws.ent, ws.seg, ws.nsys, ws.T, ws.info, ws.c_begin, ws.c_end,
                                                        ws.c_parent, ws.c_child, ws.c_level, ws.c_path, ws.c_coord, ws.c_box,
                                                        ws.c_ctr, ws.c_sys, ws.p2p_own, ws.p2p_cnt, ws.coll, ws.coll_cnt);
        ws.launches += 1;
    }
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 4, ceil_div(ws.c_cap, 32));
    k_cells<<<capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.c_cap, 128)), 128, 0, st>>>(
        ws.ent, ws.d_counts, ws.keys, n, ws.T, ws.info, psys, seg, ws.split_cell, ws.c_begin, ws.c_end, ws.c_parent,
        ws.c_child, ws.c_level, ws.c_path, ws.c_coord, ws.c_box, ws.c_ctr, forest ? ws.c_sys : nullptr);
    if (ws.c_cap <= 65536u) {
        k_leaf_list<<<1, 1024, 0, st>>>(ws.c_child, ws.d_counts, ws.leaves);
        ws.launches -= 1;  // one launch in place of the two counted below
    } else {
        k_leaf_flags<<<gs, kTB, 0, st>>>(ws.c_child, ws.d_counts, ws.flag);
        scan_exclusive_u32(ws.flag, ws.flag_off, ws.c_cap, ws.d_counts + 2, nullptr, ws.scan, st, &ws.launches);
        k_leaf_compact<<<gs, kTB, 0, st>>>(ws.flag, ws.flag_off, ws.d_counts, ws.leaves);
    }
    {
        // a warp per leaf, up to 4 warps per block within 48 KB of shared memory
        const size_t per_warp = sizeof(unsigned) * 2 * (static_cast<size_t>(ws.T) + 1);
        const int nw = static_cast<int>(std::max<size_t>(1, std::min<size_t>(4, 49152 / per_warp)));
        const size_t smem = per_warp * nw;
        if (smem > 49152) cudaFuncSetAttribute(k_leaf_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        k_leaf_sort<<<capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.c_cap, 4)), 32 * nw, smem, st>>>(
            ws.leaves, ws.d_counts, ws.c_begin, ws.c_end, ws.T, ws.perm);
    }
    k_gather<<<grid_for(n, kTB), kTB, 0, st>>>(ws.x, n, ws.perm, ws.info, psys, static_cast<float>(ws.m), ws.xs, ws.ph,
                                               ws.pl, ws.inv);
    k_lists<<<gs, 256, 0, st>>>(ws.ent, ws.d_counts, ws.split_cell, ws.info, ws.c_child, ws.c_path, ws.c_coord,
                                forest ? ws.c_sys : nullptr, ws.m2l_src, ws.p2p_own, ws.p2p_cnt, ws.coll, ws.coll_cnt,
                                reinterpret_cast<unsigned long long *>(&ws.info->m2l_pairs));
    k_rng_count<<<gs, kTB, 0, st>>>(ws.leaves, ws.d_counts, ws.c_parent, ws.c_begin, ws.c_end, ws.p2p_own, ws.p2p_cnt,
                                    ws.rng_cnt, ws.chunk_cnt, ws.src_total, ws.part_cnt, ws.p2p_slice);
    {  // range, work-item and partial-slot offsets per leaf, one scan sequence
        ScanSet sc{};
        sc.in[0] = ws.rng_cnt, sc.out[0] = ws.rng_off, sc.total[0] = ws.d_counts + 4;
        sc.in[1] = ws.chunk_cnt, sc.out[1] = ws.chunk_off, sc.total[1] = ws.d_counts + 5;
        sc.in[2] = ws.part_cnt, sc.out[2] = ws.part_off, sc.total[2] = ws.d_counts + 8;
        scan_exclusive_multi(sc, 3, ws.c_cap, ws.d_counts + 3, ws.scan, st, &ws.launches);
    }
    k_rng_fill<<<gs, kTB, 0, st>>>(ws.leaves, ws.d_counts, ws.r_cap, ws.ch_cap, ws.c_parent, ws.c_begin, ws.c_end,
                                   ws.p2p_own, ws.p2p_cnt, ws.rng_off, ws.rng_len, ws.ranges, ws.chunk_off, ws.chunks,
                                   ws.src_total, ws.part_off, ws.part_cap, ws.info, ws.p2p_slice);
    ws.launches += 9;
    timer_end(ws, kTTree);
}

}  // namespace gb
