// C-ABI of the solver (include/vipp_gb300.h): context, memory management,
// the force evaluation sequence and the RK4 step.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <functional>
#include <thread>
#include <vector>

#include "../../include/vipp_gb300.h"
#include "checkpoint.h"
#include "direct.cuh"
#include "trace.h"
#include "workspace.cuh"

namespace gb {
cudaError_t upload_tables();
void rk4_begin(Workspace &ws);
void rk4_stage(Workspace &ws, int stage, double dt);
void rk4_restore(Workspace &ws);
void aos_to_soa(Workspace &ws, const double *aos, double *soa, unsigned n);
void soa_to_aos(Workspace &ws, const double *soa, double *aos, unsigned n);

struct PendingTimer {
    int cls;
    cudaEvent_t a, b;
};

}  // namespace gb

struct gb_ctx {
    gb_config cfg{};
    gb::Workspace ws;
    std::string err;
    bool have_state = false;
    long long state_steps = 0;  // RK4 steps since the state was set
    long long retries = 0;  // evaluations repeated after a capacity overflow
    size_t phi_cap = 0;     // particles ws.phi / ws.phis are sized for
    // CUDA graph of one RK4 step, valid for (n, dt, buffer epoch)
    uint64_t epoch = 0;     // bumped whenever buffers or the configuration change
    cudaGraphExec_t step_exec = nullptr;
    unsigned step_n = 0;
    double step_dt = 0;
    uint64_t step_epoch = 0;
    int64_t step_launches = 0;
    bool graph_failed = false;
    bool levels_fitted = false;  // sort_levels fitted to the tree since the last upload
    long long graph_steps = 0, direct_steps = 0, graph_captures = 0;
    std::vector<gb::PendingTimer> pending;
    std::vector<cudaEvent_t> free_events;
    gb_tuning tune{8, 8, gb::kSliceSources, 100, 0, 0, 8};
    int tune_log2n = -1;  // size bucket the tuning cache was last applied for
    long long *d_targets = nullptr;
    size_t targets_cap = 0;
    double *d_direct = nullptr;
    size_t direct_cap = 0;
};

#ifndef GB_BATCH_THREADS
#define GB_BATCH_THREADS 8
#endif

namespace {

// message of the last failed call without a context (per host thread)
thread_local std::string g_create_error;

const char *kVersion = "vipp-gb300 0.1 (sm_103a)";

#define GB_TRY(call)                                                                        \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                  \
            return GB_ERR_CUDA;                                                             \
        }                                                                                   \
    } while (0)

template <typename T>
cudaError_t dalloc(T *&p, size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc(reinterpret_cast<void **>(&p), sizeof(T) * count);
}

void dfree(void *p) {
    if (p) cudaFree(p);
}

int validate(const gb_config *c, std::string &msg) {
    if (!c) return msg = "null config", GB_ERR_INVALID;
    if (c->p < 1 || c->p > gb::kMaxP) return msg = "p must be in 1..10", GB_ERR_INVALID;
    if (c->s < 1) return msg = "s must not be 0", GB_ERR_INVALID;  // problem.hpp:182-184
    if (!(c->eps >= 0) || !std::isfinite(c->eps)) return msg = "eps must be finite and >= 0", GB_ERR_INVALID;
    if (!std::isfinite(c->G) || !std::isfinite(c->m)) return msg = "G and m must be finite", GB_ERR_INVALID;
    if (c->precision != GB_PREC_FP64 && c->precision != GB_PREC_MIXED) return msg = "unknown precision", GB_ERR_INVALID;
    if (c->mode != GB_MODE_REF && c->mode != GB_MODE_ACCURATE) return msg = "unknown mode", GB_ERR_INVALID;
    return GB_OK;
}

void apply_config(gb_ctx *ctx) {
    gb::Workspace &ws = ctx->ws;
    ws.p = ctx->cfg.p;
    ws.K = (ws.p + 1) * (ws.p + 1);
    const int s_eff = ctx->cfg.mode == GB_MODE_ACCURATE && ctx->tune.leaf_s > 0 ? ctx->tune.leaf_s : ctx->cfg.s;
    ws.T = static_cast<int>(std::floor(std::sqrt(8.0) * static_cast<double>(s_eff)));  // octree.hpp:83
    ws.eps = ctx->cfg.eps;
    ws.G = ctx->cfg.G;
    ws.m = ctx->cfg.m;
    ws.mixed = ctx->cfg.precision == GB_PREC_MIXED;
    ws.p2p_newton = (ctx->cfg.flags & GB_FLAG_P2P_NEWTON) != 0;
    ws.m2l_tensor = ws.mixed && (ctx->cfg.flags & GB_FLAG_M2L_CUDA_CORES) == 0 && gb::m2l_tc_supported(ws.p);
    ws.m2l_bf16 = (ctx->cfg.flags & GB_FLAG_M2L_BF16) != 0;
    ws.serial = (ctx->cfg.flags & GB_FLAG_SERIAL) != 0 || ctx->tune.serial != 0;
    ws.p2p_blocks = static_cast<unsigned>(ctx->tune.p2p_blocks);
    ws.p2p_blocks_conc = static_cast<unsigned>(ctx->tune.p2p_blocks_conc);
    ws.p2p_occ = ctx->tune.p2p_occupancy == 6 ? 6 : 8;
    ws.p2p_slice = static_cast<unsigned>(ctx->tune.p2p_slice);
    ws.m2l_ctas_pct = ctx->tune.m2l_ctas_pct;
    ws.accurate = ctx->cfg.mode == GB_MODE_ACCURATE;
    // Failure-detection tests make the radix sort's bounded look-back waits
    // give up early (0: at the first poll) through this variable; the sort
    // stays exact and the call reports the timeout.
    const char *polls = std::getenv("VIPP_GB_SORT_WAIT_POLLS");
    ws.sort_spin_max = polls && *polls ? static_cast<unsigned>(std::strtoul(polls, nullptr, 10)) : gb::kSortSpinMax;
}

// P2P work items: at most two partial chunks per leaf plus n/32 full ones,
// plus source slices of leaves with long near-field lists (grown on demand).
int ensure_chunks(gb_ctx *ctx, unsigned need_items = 0, unsigned need_part = 0) {
    gb::Workspace &ws = ctx->ws;
    if (!ws.c_cap) return GB_OK;
    unsigned ch = 2 * ws.c_cap + ws.n_cap / 32 + 64;
    if (need_items > ch) ch = need_items + need_items / 4;
    if (ch > ws.ch_cap || !ws.chunks) {
        ++ctx->epoch;  // reallocated: a captured step graph no longer applies
        GB_TRY(dalloc(ws.chunks, ch));
        ws.ch_cap = ch;
    }
    unsigned pc = ws.part_cap ? ws.part_cap : 4096u;
    if (need_part > pc) pc = need_part + need_part / 4;
    if (pc > ws.part_cap || !ws.part) {
        ++ctx->epoch;
        unsigned char *b = nullptr;
        GB_TRY(dalloc(b, sizeof(double) * 96 * static_cast<size_t>(pc)));
        dfree(ws.part);
        ws.part = b;
        ws.part_cap = pc;
    }
    return GB_OK;
}

// Per-particle buffers for n_cap particles.
int ensure_particles(gb_ctx *ctx, unsigned n) {
    gb::Workspace &ws = ctx->ws;
    if (n <= ws.n_cap && ws.x) return GB_OK;
    ++ctx->epoch;
    const unsigned cap = n < 1024 ? 1024 : n;
    const size_t n3 = 3 * static_cast<size_t>(cap);
    GB_TRY(dalloc(ws.x, n3));
    GB_TRY(dalloc(ws.v, n3));
    GB_TRY(dalloc(ws.x0, n3));
    GB_TRY(dalloc(ws.v0, n3));
    GB_TRY(dalloc(ws.xo, n3));
    GB_TRY(dalloc(ws.vo, n3));
    GB_TRY(dalloc(ws.acc, n3));
    GB_TRY(dalloc(ws.staging, n3));
    GB_TRY(dalloc(ws.keys0, cap));
    GB_TRY(dalloc(ws.keys1, cap));
    GB_TRY(dalloc(ws.perm0, cap));
    GB_TRY(dalloc(ws.perm1, cap));
    GB_TRY(dalloc(ws.inv, cap));
    GB_TRY(dalloc(ws.xs, n3));
    GB_TRY(dalloc(ws.ph, cap));
    GB_TRY(dalloc(ws.pl, cap));
    {
        double *a = nullptr, *b = nullptr;
        GB_TRY(dalloc(a, n3));
        GB_TRY(dalloc(b, n3));
        dfree(ws.nearf);
        dfree(ws.farf);
        ws.nearf = a, ws.farf = b;
    }
    GB_TRY(dalloc(ws.cnt, cap + 1));
    GB_TRY(dalloc(ws.off, cap + 1));
    GB_TRY(gb::sort_temp_alloc(ws.sort, cap));
    GB_TRY(gb::scan_temp_alloc(ws.scan, std::max(cap + 1, ws.c_cap + 1)));
    if (ws.accurate) {  // the softening correction computed beside the far field
        double *c = nullptr;
        GB_TRY(dalloc(c, n3));
        dfree(ws.soft_corr);
        ws.soft_corr = c;
        ws.soft_corr_cap = cap;
    }
    ws.n_cap = cap;
    return ensure_chunks(ctx);
}

// Cell-indexed buffers for s_cap split cells (c_cap = 1 + 8 s_cap cells).
int ensure_cells(gb_ctx *ctx, unsigned s_cap, unsigned r_cap) {
    gb::Workspace &ws = ctx->ws;
    const size_t esz = ws.mixed ? sizeof(float) : sizeof(double);
    if (s_cap > ws.s_cap || ws.k_cap != ws.K * static_cast<int>(esz)) {
        ++ctx->epoch;
        const unsigned c = static_cast<unsigned>(ws.forest() ? ws.nsys : 1) + 8 * s_cap;  // roots + 8 per split cell
        GB_TRY(dalloc(ws.ent0, s_cap));
        GB_TRY(dalloc(ws.ent1, s_cap));
        GB_TRY(dalloc(ws.split_cell, s_cap));
        GB_TRY(dalloc(ws.c_begin, c));
        GB_TRY(dalloc(ws.c_end, c));
        GB_TRY(dalloc(ws.c_parent, c));
        GB_TRY(dalloc(ws.c_child, c));
        GB_TRY(dalloc(ws.c_level, c));
        GB_TRY(dalloc(ws.c_path, c));
        GB_TRY(dalloc(ws.c_coord, 3 * static_cast<size_t>(c)));
        GB_TRY(dalloc(ws.c_box, 6 * static_cast<size_t>(c)));
        GB_TRY(dalloc(ws.c_ctr, 3 * static_cast<size_t>(c)));
        {
            unsigned char *a = nullptr, *b = nullptr;
            GB_TRY(dalloc(a, esz * ws.K * static_cast<size_t>(c)));
            GB_TRY(dalloc(b, esz * ws.K * static_cast<size_t>(c)));
            dfree(ws.Mexp);
            dfree(ws.Lexp);
            ws.Mexp = a, ws.Lexp = b;
        }
        GB_TRY(dalloc(ws.m2l_src, static_cast<size_t>(gb::kM2LSlots) * c));
        GB_TRY(dalloc(ws.p2p_own, static_cast<size_t>(gb::kNbrCap) * c));
        GB_TRY(dalloc(ws.p2p_cnt, c));
        GB_TRY(dalloc(ws.coll, static_cast<size_t>(gb::kNbrCap) * c));
        GB_TRY(dalloc(ws.coll_cnt, c));
        GB_TRY(dalloc(ws.flag, c + 1));
        GB_TRY(dalloc(ws.flag_off, c + 1));
        GB_TRY(dalloc(ws.leaves, c));
        GB_TRY(dalloc(ws.rng_cnt, c + 1));
        GB_TRY(dalloc(ws.rng_off, c + 1));
        GB_TRY(dalloc(ws.rng_len, c));
        GB_TRY(dalloc(ws.chunk_cnt, c + 1));
        GB_TRY(dalloc(ws.chunk_off, c + 1));
        GB_TRY(dalloc(ws.src_total, c + 1));
        GB_TRY(dalloc(ws.part_cnt, c + 1));
        GB_TRY(dalloc(ws.part_off, c + 1));
        if (ws.forest()) {  // per-cell systems and the one-system tiles (tree.cu: forest_tiles)
            GB_TRY(dalloc(ws.c_sys, c));
            GB_TRY(dalloc(ws.etile, s_cap + 1));
            GB_TRY(dalloc(ws.oct_list, c / 8 + 1));
            GB_TRY(dalloc(ws.otile, c / 8 + static_cast<size_t>(ws.nsys) + 1));
        }
        GB_TRY(gb::scan_temp_alloc(ws.scan, std::max(ws.n_cap + 1, c + 1)));
        GB_TRY(gb::sort_temp_alloc(ws.sort, std::max(ws.n_cap, s_cap)));
        ws.s_cap = s_cap;
        ws.c_cap = c;
        ws.k_cap = ws.K * static_cast<int>(esz);
    }
    if (r_cap > ws.r_cap) {
        ++ctx->epoch;
        GB_TRY(dalloc(ws.ranges, r_cap));
        ws.r_cap = r_cap;
    }
    if (ws.accurate && (ws.soft_cap != ws.c_cap || ws.soft_mixed != ws.mixed)) {
        // moment records, octant records and leaf-centre terms of the softening correction
        ++ctx->epoch;
        const size_t rec = gb::soften_cell_bytes(ws.mixed), c = ws.c_cap;
        unsigned char *a = nullptr, *b = nullptr, *t = nullptr;
        GB_TRY(dalloc(a, rec * c));
        GB_TRY(dalloc(b, 8 * rec * c));
        GB_TRY(dalloc(t, gb::soften_taylor_values() * (rec / 16) * c));
        dfree(ws.smom);
        dfree(ws.smom_oct);
        dfree(ws.staylor);
        ws.smom = a, ws.smom_oct = b, ws.staylor = t;
        ws.soft_cap = ws.c_cap, ws.soft_mixed = ws.mixed;
    }
    if (ws.accurate && (!ws.soft_corr || ws.soft_corr_cap < ws.n_cap)) {
        ++ctx->epoch;
        double *c = nullptr;
        GB_TRY(dalloc(c, 3 * static_cast<size_t>(ws.n_cap)));  // doubles: either precision fits
        dfree(ws.soft_corr);
        ws.soft_corr = c;
        ws.soft_corr_cap = ws.n_cap;
    }
    if (ws.m2l_tensor) {
        // split expansions of the tensor-core M2L and their TMA map
        const int kp = gb::m2l_tc_row_floats(ws.p);
        const unsigned rows = ws.c_cap + gb::kZeroRows;
        if (!ws.ms_tc || ws.ms_rows != rows || ws.ms_kp != kp || ws.ms_bf16 != ws.m2l_bf16) {
            ++ctx->epoch;
            GB_TRY(dalloc(ws.ms_tc, 2 * static_cast<size_t>(rows) * kp));
            ws.ms_rows = rows, ws.ms_kp = kp;
            if (const char *e = gb::m2l_tc_encode(ws)) {
                dfree(ws.ms_tc);
                ws.ms_tc = nullptr, ws.ms_rows = 0;
                ctx->err = e;
                return GB_ERR_CUDA;
            }
        }
    }
    return ensure_chunks(ctx);
}

void collect_timers(gb_ctx *ctx) {
    gb::Workspace &ws = ctx->ws;
    for (auto &pt : ctx->pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, pt.a, pt.b) == cudaSuccess) {
            ws.t_ms[pt.cls] += ms;
            ws.t_launch[pt.cls] += 1;
        }
        ctx->free_events.push_back(pt.a);
        ctx->free_events.push_back(pt.b);
    }
    ctx->pending.clear();
}

// context whose stream the timer hooks record on (set by each evaluation on
// its own host thread: a batch queues its contexts from several threads)
thread_local gb_ctx *g_timer_ctx = nullptr;

const char *const kClassNames[gb::kNumTimers] = {"tree", "operators", "p2m_m2m", "m2l",
                                                 "l2l_l2p", "p2p", "rk4", "soften"};

}  // namespace

namespace gb {

void timer_begin(Workspace &ws, int cls) {
    nvtx_push(kClassNames[cls]);
    if (!ws.timing || !g_timer_ctx) return;
    gb_ctx *ctx = g_timer_ctx;
    auto take = [&]() {
        cudaEvent_t e;
        if (!ctx->free_events.empty()) {
            e = ctx->free_events.back();
            ctx->free_events.pop_back();
        } else {
            cudaEventCreate(&e);
        }
        return e;
    };
    PendingTimer pt{cls, take(), take()};
    cudaEventRecord(pt.a, ws.st);
    ctx->pending.push_back(pt);
}

void timer_end(Workspace &ws, int cls) {
    nvtx_pop();
    if (!ws.timing || !g_timer_ctx) return;
    gb_ctx *ctx = g_timer_ctx;
    for (auto it = ctx->pending.rbegin(); it != ctx->pending.rend(); ++it)
        if (it->cls == cls) {
            cudaEventRecord(it->b, ws.st);
            return;
        }
}

}  // namespace gb

namespace {

int check_device_errors(gb_ctx *ctx, unsigned *need) {
    gb::Workspace &ws = ctx->ws;
    GB_TRY(cudaMemcpyAsync(ws.h_info, ws.info, sizeof(gb::TreeInfo), cudaMemcpyDeviceToHost, ws.st));
    unsigned counts[gb::kNumCounts];
    GB_TRY(cudaMemcpyAsync(counts, ws.d_counts, sizeof(counts), cudaMemcpyDeviceToHost, ws.st));
    GB_TRY(cudaStreamSynchronize(ws.st));
    GB_TRY(cudaGetLastError());
    collect_timers(ctx);
    const int err = ws.h_info->err;
    if (need) std::memcpy(need, counts, sizeof(counts));
    if (err & gb::kDevNonFinite) {
        ctx->err = "non-finite position";
        return GB_ERR_NONFINITE;
    }
    if (err & gb::kDevDepth) {
        ctx->err = "tree deeper than 21 levels (more than floor(sqrt(8) s) coincident particles?)";
        return GB_ERR_DEPTH;
    }
    if (err & gb::kDevForestDepth) {
        ctx->err = "a system of the forest needs more tree levels than its sort word holds beside the system index "
                   "(fewer systems per batch, or the contexts form)";
        return GB_ERR_DEPTH;
    }
    if (err & gb::kDevTimeout) {
        ctx->err = "a bounded device wait gave up (radix-sort look-back or tensor-core M2L barrier); this call's "
                   "results are discarded";
        return GB_ERR_CUDA;
    }
    if (err & gb::kDevCapacity) {
        ctx->err = "capacity";
        return GB_ERR_CAPACITY;
    }
    // After the first good evaluation of an upload, sort only the key levels
    // the tree uses plus one, rounded up to what the same number of 8-bit
    // radix passes holds (never more than now): shallow trees get fewer sort
    // passes and M2M/L2L level launches, and the margin costs no pass. A tree
    // that deepens past it later asks for more through counts[9].
    if (!ctx->levels_fitted) {
        ctx->levels_fitted = true;
        const int sb = ws.forest() ? ws.sys_bits : 0;  // a forest's sort word also holds the system
        const int passes = (3 * std::max(3, ws.h_info->depth + 1) + sb + 7) / 8;
        const int want = std::min((8 * passes - sb) / 3, ws.sort_levels_cap());
        if (want < ws.sort_levels) ws.sort_levels = want, ++ctx->epoch;
    }
    return GB_OK;
}

// One force evaluation. After the tree the near field (P2P, FP32/FP64 CUDA
// cores) and the far field (operators, P2M/M2M, M2L on the tensor cores,
// L2L/L2P) read only tree data and write separate buffers, so the near field
// runs on a second stream concurrently with the far field; finalize joins them.
// One force evaluation; with to_acc the accelerations are also written out
// in particle order (acc), which RK4 stages do not need (they read the tree-
// order parts directly).
void evaluate(gb_ctx *ctx, bool to_acc = true) {
    gb::Workspace &ws = ctx->ws;
    g_timer_ctx = ctx;
    gb::build_tree(ws);
    // Near field on the second stream, unless serial or timed: class timers
    // measure each class alone on one stream.
    const bool fork = !ws.serial && !ws.timing;
    const unsigned conc = ws.p2p_blocks_conc, full = ws.p2p_blocks;
    if (fork) {
        cudaEventRecord(ws.ev_fork, ws.st);
        cudaStreamWaitEvent(ws.st2, ws.ev_fork, 0);
        std::swap(ws.st, ws.st2);  // the stages launch on ws.st
        gb::p2p_pass(ws, conc);
        std::swap(ws.st, ws.st2);
        cudaEventRecord(ws.ev_join, ws.st2);
    }
    // accurate mode: the softening correction needs only the tree and the
    // particles, so it runs on a third stream beside the far field and is
    // folded into the far field after L2P
    const bool soft_fork = ws.accurate && fork && ws.soft_corr && ws.soft_corr_cap >= ws.n;
    if (soft_fork) {
        cudaEventRecord(ws.ev_fork3, ws.st);
        cudaStreamWaitEvent(ws.st3, ws.ev_fork3, 0);
        std::swap(ws.st, ws.st3);
        gb::soften_corr(ws);
        std::swap(ws.st, ws.st3);
        cudaEventRecord(ws.ev_join3, ws.st3);
    }
    gb::build_operators(ws);
    if (ws.forest()) gb::forest_tiles(ws, ws.m2l_tensor ? gb::kM2LTileTC : gb::kM2LTileCC);
    gb::upward_pass(ws);
    if (ws.m2l_tensor)
        gb::m2l_pass_tc(ws);
    else
        gb::m2l_pass(ws);
    gb::downward_pass(ws);
    if (soft_fork) {
        cudaStreamWaitEvent(ws.st, ws.ev_join3, 0);
        gb::soften_apply(ws);
    } else if (ws.accurate) {
        gb::soften_pass(ws);
    }
    if (!fork) {
        gb::p2p_pass(ws, full);
    } else {
        // more P2P blocks on the SMs the far field leaves, draining the same queue
        gb::p2p_pass(ws, full > conc ? full - conc : 0u);
        cudaStreamWaitEvent(ws.st, ws.ev_join, 0);
    }
    gb::p2p_finish(ws);
    if (to_acc) gb::finalize_accel(ws, ws.acc);
}

// Grow capacities after an overflow reported by the device (counts holds
// the sizes the evaluation asked for).
int grow(gb_ctx *ctx, const unsigned *counts) {
    gb::Workspace &ws = ctx->ws;
    ++ctx->epoch;
    const unsigned need_s = counts[6], need_r = counts[4], need_items = counts[7], need_part = counts[8];
    if (counts[9] > static_cast<unsigned>(ws.sort_levels))
        ws.sort_levels = std::min(gb::kMaxLevel, static_cast<int>(counts[9]));
    const unsigned s = need_s > ws.s_cap ? need_s + need_s / 2 + 64 : ws.s_cap;
    const unsigned r = need_r > ws.r_cap ? need_r + need_r / 2 + 1024 : ws.r_cap;
    const int rc = ensure_cells(ctx, s, r);
    if (rc) return rc;
    return ensure_chunks(ctx, need_items, need_part);
}

// Run f (which queues one or more evaluations) until no capacity overflow.
template <typename F>
int run_with_capacity(gb_ctx *ctx, F &&f) {
    for (int attempt = 0; attempt < 6; ++attempt) {
        f();
        unsigned counts[gb::kNumCounts];
        const int rc = check_device_errors(ctx, counts);
        if (rc != GB_ERR_CAPACITY) return rc;
        const int g = grow(ctx, counts);
        if (g != GB_OK) return g;
        ++ctx->retries;
    }
    ctx->err = "could not size the tree buffers";
    return GB_ERR_CAPACITY;
}

int initial_capacity(gb_ctx *ctx) {
    gb::Workspace &ws = ctx->ws;
    const unsigned n = ws.n;
    const unsigned guess = 2 * (n / static_cast<unsigned>(ws.T + 1)) + 64;
    if (ws.s_cap >= guess && ws.k_cap == ws.K * static_cast<int>(ws.mixed ? sizeof(float) : sizeof(double))) return GB_OK;
    return ensure_cells(ctx, std::max(guess, ws.s_cap), std::max(ws.r_cap, 32 * (1 + 8 * guess)));
}

}  // namespace

namespace {

int validate_tuning(const gb_tuning *t, std::string &msg) {
    if (!t) return msg = "null tuning", GB_ERR_INVALID;
    if (t->p2p_blocks < 1 || t->p2p_blocks > 16) return msg = "p2p_blocks must be in 1..16", GB_ERR_INVALID;
    if (t->p2p_blocks_conc < 0 || t->p2p_blocks_conc > 16) return msg = "p2p_blocks_conc must be in 0..16", GB_ERR_INVALID;
    if (t->p2p_slice < 1024 || t->p2p_slice > 65536) return msg = "p2p_slice must be in 1024..65536", GB_ERR_INVALID;
    if (t->m2l_ctas_pct < 10 || t->m2l_ctas_pct > 100) return msg = "m2l_ctas_pct must be in 10..100", GB_ERR_INVALID;
    if (t->serial != 0 && t->serial != 1) return msg = "serial must be 0 or 1", GB_ERR_INVALID;
    if (t->leaf_s < 0) return msg = "leaf_s must be >= 0", GB_ERR_INVALID;
    if (t->p2p_occupancy != 0 && t->p2p_occupancy != 6 && t->p2p_occupancy != 8)
        return msg = "p2p_occupancy must be 6 or 8 (0: 8)", GB_ERR_INVALID;
    return GB_OK;
}

int floor_log2(size_t n) {
    int k = -1;
    while (n) n >>= 1, ++k;
    return k;
}

// gb_tuning_lookup's parser: one entry per line of key=value tokens.
int tuning_from_file(const char *path, const gb_config *cfg, size_t n, gb_tuning *out, std::string &msg) {
    if (!path || !cfg || !out) return msg = "null argument", GB_ERR_INVALID;
    FILE *f = std::fopen(path, "r");
    if (!f) return msg = std::string("cannot open ") + path, GB_ERR_INVALID;
    const long want[5] = {cfg->p, cfg->precision, cfg->mode, (cfg->flags & GB_FLAG_M2L_BF16) ? 1 : 0,
                          static_cast<long>(floor_log2(n))};
    static const char *kKeys[5] = {"p", "precision", "mode", "m2l_bf16", "log2n"};
    static const char *kFields[7] = {"p2p_blocks", "p2p_blocks_conc", "p2p_slice", "m2l_ctas_pct", "serial", "leaf_s",
                                     "p2p_occupancy"};
    char line[1024];
    int rc = GB_ERR_STATE;
    int lineno = 0;
    while (std::fgets(line, sizeof line, f)) {
        ++lineno;
        if (char *h = std::strchr(line, '#')) *h = 0;
        long key[5] = {-1, -1, -1, -1, -1};
        gb_tuning t{8, 8, gb::kSliceSources, 100, 0, 0, 8};
        int *fld[7] = {&t.p2p_blocks, &t.p2p_blocks_conc, &t.p2p_slice, &t.m2l_ctas_pct, &t.serial, &t.leaf_s,
                       &t.p2p_occupancy};
        bool any = false, bad = false;
        for (char *tok = std::strtok(line, " \t\r\n"); tok; tok = std::strtok(nullptr, " \t\r\n")) {
            char *eq = std::strchr(tok, '=');
            if (!eq) {
                bad = true;
                break;
            }
            *eq = 0;
            char *end = nullptr;
            const long v = std::strtol(eq + 1, &end, 10);
            if (!end || *end || end == eq + 1) {
                bad = true;
                break;
            }
            bool known = false;
            for (int k = 0; k < 5; ++k)
                if (!std::strcmp(tok, kKeys[k])) key[k] = v, known = true;
            for (int k = 0; k < 7; ++k)
                if (!std::strcmp(tok, kFields[k])) *fld[k] = static_cast<int>(v), known = true;
            if (!known) {
                bad = true;
                break;
            }
            any = true;
        }
        if (!any) continue;
        std::string m2;
        if (bad || key[0] < 0 || key[1] < 0 || key[2] < 0 || key[3] < 0 || key[4] < 0 || validate_tuning(&t, m2) != GB_OK) {
            msg = std::string(path) + ":" + std::to_string(lineno) + ": malformed tuning entry" + (m2.empty() ? "" : " (" + m2 + ")");
            rc = GB_ERR_INVALID;
            break;
        }
        if (key[0] == want[0] && key[1] == want[1] && key[2] == want[2] && key[3] == want[3] && key[4] == want[4]) {
            *out = t;  // the last matching entry wins
            rc = GB_OK;
        }
    }
    std::fclose(f);
    if (rc == GB_ERR_STATE) msg = "no tuning entry for this configuration and size";
    return rc;
}

int apply_tuning(gb_ctx *ctx, const gb_tuning &t);

// The tuning cache named by VIPP_GB_TUNE_FILE, applied when the uploaded n
// falls into another size bucket than the last one applied. A file without an
// entry for this configuration and bucket leaves the tuning as it is.
int apply_tuning_cache(gb_ctx *ctx, size_t n) {
    const char *path = std::getenv("VIPP_GB_TUNE_FILE");
    if (!path || !*path || n == 0) return GB_OK;
    const int b = floor_log2(n);
    if (b == ctx->tune_log2n) return GB_OK;
    gb_tuning t{};
    std::string msg;
    const int rc = tuning_from_file(path, &ctx->cfg, n, &t, msg);
    if (rc == GB_ERR_INVALID) return ctx->err = msg, rc;
    ctx->tune_log2n = b;
    return rc == GB_OK ? apply_tuning(ctx, t) : GB_OK;
}

int apply_tuning(gb_ctx *ctx, const gb_tuning &t) {
    const int oldT = ctx->ws.T;
    ctx->tune = t;
    ++ctx->epoch;  // launch shapes are baked into a captured step graph
    apply_config(ctx);
    if (ctx->ws.T != oldT && ctx->have_state) {
        ctx->levels_fitted = false;
        const int r = initial_capacity(ctx);
        if (r) return r;
    }
    return GB_OK;
}

}  // namespace

extern "C" {

const char *gb_version(void) { return kVersion; }

int gb_set_tuning(gb_ctx *ctx, const gb_tuning *t) {
    if (!ctx) return GB_ERR_INVALID;
    std::string msg;
    const int rc = validate_tuning(t, msg);
    if (rc) return ctx->err = msg, rc;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    return apply_tuning(ctx, *t);
}

int gb_get_tuning(const gb_ctx *ctx, gb_tuning *out) {
    if (!ctx || !out) return GB_ERR_INVALID;
    *out = ctx->tune;
    return GB_OK;
}

int gb_tuning_lookup(const char *path, const gb_config *cfg, size_t n, gb_tuning *out) {
    std::string msg;
    const int rc = tuning_from_file(path, cfg, n, out, msg);
    if (rc != GB_OK) g_create_error = msg;
    return rc;
}

int gb_create(const gb_config *cfg, gb_ctx **out) {
    if (!out) return GB_ERR_INVALID;
    *out = nullptr;
    std::string msg;
    int rc = validate(cfg, msg);
    if (rc) {
        g_create_error = msg;
        return rc;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_create_error = "no CUDA device";
        return GB_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) {
        g_create_error = "device ordinal out of range";
        return GB_ERR_INVALID;
    }
    auto *ctx = new gb_ctx;
    ctx->cfg = *cfg;
    apply_config(ctx);
    gb::Workspace &ws = ctx->ws;
    // gb_destroy frees whatever was created before the failure (the
    // workspace's handles and buffers start out null)
    auto fail = [&](const char *what, cudaError_t e) {
        g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
        gb_destroy(ctx);
        return GB_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) return fail("cudaSetDevice", e);
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, cfg->device);
    if (e != cudaSuccess) return fail("cudaGetDeviceProperties", e);
    if (prop.major < 10) {
        g_create_error = "this build targets sm_103a (Blackwell Ultra); device is sm_" + std::to_string(prop.major) +
                         std::to_string(prop.minor);
        gb_destroy(ctx);
        return GB_ERR_NO_DEVICE;
    }
    ws.num_sms = prop.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&ws.st, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", e);
    if ((e = cudaStreamCreateWithFlags(&ws.st2, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", e);
    if ((e = cudaEventCreateWithFlags(&ws.ev_fork, cudaEventDisableTiming)) != cudaSuccess) return fail("event", e);
    if ((e = cudaEventCreateWithFlags(&ws.ev_join, cudaEventDisableTiming)) != cudaSuccess) return fail("event", e);
    if ((e = cudaStreamCreateWithFlags(&ws.st3, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", e);
    if ((e = cudaEventCreateWithFlags(&ws.ev_fork3, cudaEventDisableTiming)) != cudaSuccess) return fail("event", e);
    if ((e = cudaEventCreateWithFlags(&ws.ev_join3, cudaEventDisableTiming)) != cudaSuccess) return fail("event", e);
    if ((e = gb::upload_tables()) != cudaSuccess) return fail("tables", e);
    if ((e = cudaMalloc(&ws.info, sizeof(gb::TreeInfo))) != cudaSuccess) return fail("info", e);
    if ((e = cudaMalloc(&ws.d_counts, gb::kNumCounts * sizeof(unsigned))) != cudaSuccess) return fail("counts", e);
    if ((e = cudaMalloc(&ws.queue, sizeof(unsigned))) != cudaSuccess) return fail("queue", e);
    if ((e = cudaMalloc(&ws.bbox_part, sizeof(double) * 6 * 2 * ws.num_sms)) != cudaSuccess) return fail("bbox", e);
    if ((e = cudaMallocHost(&ws.h_info, sizeof(gb::TreeInfo))) != cudaSuccess) return fail("pinned info", e);
    std::memset(ws.h_info, 0, sizeof(gb::TreeInfo));
    const size_t kk = static_cast<size_t>(ws.K) * ws.K * gb::kNumOps;
    if ((e = cudaMalloc(&ws.ops_d, sizeof(double) * kk)) != cudaSuccess) return fail("ops", e);
    if ((e = cudaMalloc(&ws.ops_f, sizeof(float) * kk)) != cudaSuccess) return fail("ops", e);
    if ((e = cudaMalloc(&ws.zf, sizeof(float) * gb::zf_table_floats(ws.p))) != cudaSuccess) return fail("ops", e);
    if ((e = cudaMalloc(&ws.bimg, sizeof(float) * gb::m2l_tc_image_floats(ws.p))) != cudaSuccess) return fail("ops", e);
    // image rows past K are never written (k_build_bimg): zero once
    if ((e = cudaMemset(ws.bimg, 0, sizeof(float) * gb::m2l_tc_image_floats(ws.p))) != cudaSuccess) return fail("ops", e);
    if ((e = cudaMalloc(&ws.m2l_tab, gb::m2l_table_bytes(ws.p))) != cudaSuccess) return fail("ops", e);
    gb::build_m2l_table(ws);
    if ((e = cudaStreamSynchronize(ws.st)) != cudaSuccess) return fail("ops table", e);
    *out = ctx;
    return GB_OK;
}

void gb_destroy(gb_ctx *ctx) {
    if (!ctx) return;
    gb::Workspace &ws = ctx->ws;
    cudaSetDevice(ctx->cfg.device);
    if (ws.st) cudaStreamSynchronize(ws.st);
    collect_timers(ctx);
    for (auto e : ctx->free_events) cudaEventDestroy(e);
    void *bufs[] = {ws.x, ws.v, ws.x0, ws.v0, ws.xo, ws.vo, ws.acc, ws.phi, ws.staging, ws.bbox_part, ws.keys0, ws.keys1,
                    ws.perm0, ws.perm1, ws.inv, ws.xs, ws.ph, ws.pl, ws.nearf, ws.farf, ws.phis, ws.cnt, ws.off, ws.ent0, ws.ent1,
                    ws.split_cell, ws.c_begin, ws.c_end, ws.c_parent, ws.c_child, ws.c_level, ws.c_path, ws.c_coord,
                    ws.c_box, ws.c_ctr, ws.Mexp, ws.Lexp, ws.m2l_src, ws.p2p_own, ws.p2p_cnt, ws.coll, ws.coll_cnt,
                    ws.flag, ws.flag_off, ws.leaves, ws.rng_cnt, ws.rng_off, ws.rng_len, ws.ranges, ws.chunk_cnt,
                    ws.chunk_off, ws.chunks, ws.src_total, ws.part_cnt, ws.part_off, ws.part, ws.queue, ws.ops_d, ws.bimg, ws.m2l_tab, ws.ms_tc, ws.diag, ws.ops_f, ws.zf, ws.info, ws.d_counts, ctx->d_targets, ws.smom, ws.smom_oct, ws.staylor,
                    ctx->d_direct, ws.seg, ws.psys, ws.c_sys, ws.sys_par, ws.mkeys, ws.etile, ws.oct_list, ws.otile,
                    ws.ocnt, ws.soft_corr};
    for (void *b : bufs) dfree(b);
    gb::sort_temp_free(ws.sort);
    gb::scan_temp_free(ws.scan);
    if (ws.h_info) cudaFreeHost(ws.h_info);
    if (ctx->step_exec) cudaGraphExecDestroy(ctx->step_exec);
    if (ws.ev_fork) cudaEventDestroy(ws.ev_fork);
    if (ws.ev_join) cudaEventDestroy(ws.ev_join);
    if (ws.ev_fork3) cudaEventDestroy(ws.ev_fork3);
    if (ws.ev_join3) cudaEventDestroy(ws.ev_join3);
    if (ws.st3) cudaStreamDestroy(ws.st3);
    if (ws.st2) cudaStreamDestroy(ws.st2);
    if (ws.st) cudaStreamDestroy(ws.st);
    if (g_timer_ctx == ctx) g_timer_ctx = nullptr;
    delete ctx;
}

const char *gb_last_error(const gb_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int gb_set_config(gb_ctx *ctx, const gb_config *cfg) {
    if (ctx) ctx->levels_fitted = false;
    if (!ctx) return GB_ERR_INVALID;
    ++ctx->epoch;  // buffers, sizes or configuration may change: the step graph is rebuilt
    std::string msg;
    int rc = validate(cfg, msg);
    if (rc) return ctx->err = msg, rc;
    if (cfg->device != ctx->cfg.device) return ctx->err = "device cannot change", GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    const int oldK = ctx->ws.K;
    const int oldT = ctx->ws.T;
    ctx->cfg = *cfg;
    apply_config(ctx);
    if (ctx->ws.K != oldK) {
        const size_t kk = static_cast<size_t>(ctx->ws.K) * ctx->ws.K * gb::kNumOps;
        GB_TRY(dalloc(ctx->ws.ops_d, kk));
        GB_TRY(dalloc(ctx->ws.ops_f, kk));
        GB_TRY(dalloc(ctx->ws.zf, gb::zf_table_floats(ctx->ws.p)));
        GB_TRY(dalloc(ctx->ws.bimg, gb::m2l_tc_image_floats(ctx->ws.p)));
        GB_TRY(cudaMemset(ctx->ws.bimg, 0, sizeof(float) * gb::m2l_tc_image_floats(ctx->ws.p)));
        unsigned char *t = nullptr;
        GB_TRY(dalloc(t, gb::m2l_table_bytes(ctx->ws.p)));
        dfree(ctx->ws.m2l_tab);
        ctx->ws.m2l_tab = t;
        gb::build_m2l_table(ctx->ws);
    }
    if (ctx->ws.T != oldT && ctx->have_state) {
        const int r = initial_capacity(ctx);
        if (r) return r;
    }
    if (ctx->have_state) {
        const int r = ensure_cells(ctx, ctx->ws.s_cap, ctx->ws.r_cap);
        if (r) return r;
    }
    return GB_OK;
}

int gb_upload(gb_ctx *ctx, const double *x_aos, const double *v_aos, size_t n) {
    gb::NvtxRange nvtx_("gb_upload");
    if (ctx) ctx->levels_fitted = false;
    if (!ctx) return GB_ERR_INVALID;
    if (n > 0x7fffffffu) return ctx->err = "too many particles", GB_ERR_INVALID;
    if (n && (!x_aos || !v_aos)) return ctx->err = "null input", GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    const unsigned nn = static_cast<unsigned>(n);
    int rc = apply_tuning_cache(ctx, n);
    if (rc) return rc;
    rc = ensure_particles(ctx, nn);
    if (rc) return rc;
    ws.n = nn;
    if (nn) {
        GB_TRY(cudaMemcpyAsync(ws.staging, x_aos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ws.st));
        gb::aos_to_soa(ws, ws.staging, ws.x, nn);
        GB_TRY(cudaMemcpyAsync(ws.staging, v_aos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ws.st));
        gb::aos_to_soa(ws, ws.staging, ws.v, nn);
        rc = initial_capacity(ctx);
        if (rc) return rc;
    }
    GB_TRY(cudaStreamSynchronize(ws.st));
    ctx->have_state = true;
    ctx->state_steps = 0;
    return GB_OK;
}

int gb_init_plummer(gb_ctx *ctx, size_t n, uint64_t seed, double r_max) {
    gb::NvtxRange nvtx_("gb_init_plummer");
    if (ctx) ctx->levels_fitted = false;
    if (!ctx) return GB_ERR_INVALID;
    if (n > 0x7fffffffu) return ctx->err = "too many particles", GB_ERR_INVALID;
    if (!(r_max >= 0) || !std::isfinite(r_max)) return ctx->err = "r_max must be finite and >= 0", GB_ERR_INVALID;
    if (r_max == 0 && !(ctx->cfg.eps > 0 && ctx->cfg.eps < 1))
        return ctx->err = "the reference's radius cap needs 0 < eps < 1 (or give r_max)", GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    const unsigned nn = static_cast<unsigned>(n);
    int rc = apply_tuning_cache(ctx, n);
    if (rc) return rc;
    rc = ensure_particles(ctx, nn);
    if (rc) return rc;
    ws.n = nn;
    if (nn) {
        gb::generate_plummer(ws, nn, seed, 1.0 - ctx->cfg.eps, r_max);
        GB_TRY(cudaGetLastError());
        int err = 0;
        GB_TRY(cudaMemcpyAsync(&err, &ws.info->err, sizeof(int), cudaMemcpyDeviceToHost, ws.st));
        GB_TRY(cudaStreamSynchronize(ws.st));
        if (err) return ctx->err = "initial-condition sampling did not converge", GB_ERR_CUDA;
        rc = initial_capacity(ctx);
        if (rc) return rc;
    }
    GB_TRY(cudaStreamSynchronize(ws.st));
    ctx->have_state = true;
    ctx->state_steps = 0;
    return GB_OK;
}

int gb_init_clustered(gb_ctx *ctx, size_t n, uint64_t seed, int clusters, double background, double r_max,
                      double *params) {
    gb::NvtxRange nvtx_("gb_init_clustered");
    if (ctx) ctx->levels_fitted = false;
    if (!ctx) return GB_ERR_INVALID;
    if (n > 0x7fffffffu) return ctx->err = "too many particles", GB_ERR_INVALID;
    if (clusters < 1 || clusters > 8) return ctx->err = "clusters must be in 1..8", GB_ERR_INVALID;
    if (!(background >= 0 && background < 1)) return ctx->err = "background must be in [0, 1)", GB_ERR_INVALID;
    if (!(r_max > 0) || !std::isfinite(r_max)) return ctx->err = "r_max must be finite and > 0", GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    const unsigned nn = static_cast<unsigned>(n);
    int rc = apply_tuning_cache(ctx, n);
    if (rc) return rc;
    rc = ensure_particles(ctx, nn);
    if (rc) return rc;
    ws.n = nn;
    if (nn) {
        if (gb::generate_clustered(ws, nn, seed, clusters, background, r_max, params) != 0)
            return ctx->err = "bad cluster parameters", GB_ERR_INVALID;
        GB_TRY(cudaGetLastError());
        int err = 0;
        GB_TRY(cudaMemcpyAsync(&err, &ws.info->err, sizeof(int), cudaMemcpyDeviceToHost, ws.st));
        GB_TRY(cudaStreamSynchronize(ws.st));
        if (err) return ctx->err = "initial-condition sampling did not converge", GB_ERR_CUDA;
        rc = initial_capacity(ctx);
        if (rc) return rc;
    }
    GB_TRY(cudaStreamSynchronize(ws.st));
    ctx->have_state = true;
    ctx->state_steps = 0;
    return GB_OK;
}

int gb_download(gb_ctx *ctx, double *x_aos, double *v_aos) {
    gb::NvtxRange nvtx_("gb_download");
    if (!ctx) return GB_ERR_INVALID;
    if (!ctx->have_state) return ctx->err = "no state uploaded", GB_ERR_STATE;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    if (ws.n == 0) return GB_OK;
    if (x_aos) {
        gb::soa_to_aos(ws, ws.x, ws.staging, ws.n);
        GB_TRY(cudaMemcpyAsync(x_aos, ws.staging, sizeof(double) * 3 * ws.n, cudaMemcpyDeviceToHost, ws.st));
        GB_TRY(cudaStreamSynchronize(ws.st));
    }
    if (v_aos) {
        gb::soa_to_aos(ws, ws.v, ws.staging, ws.n);
        GB_TRY(cudaMemcpyAsync(v_aos, ws.staging, sizeof(double) * 3 * ws.n, cudaMemcpyDeviceToHost, ws.st));
        GB_TRY(cudaStreamSynchronize(ws.st));
    }
    GB_TRY(cudaGetLastError());
    return GB_OK;
}

// Captures one RK4 step (restore, 4 x evaluate + stage) into a CUDA graph.
// Kernel sizes come from the device, so the graph holds while n, dt and the
// buffers stay the same. On any capture failure the context stops using
// graphs and launches the kernels directly.
static void capture_step(gb_ctx *ctx, double dt, const std::function<void()> &body) {
    gb::Workspace &ws = ctx->ws;
    if (ctx->step_exec) cudaGraphExecDestroy(ctx->step_exec);
    ctx->step_exec = nullptr;
    const int64_t l0 = ws.launches;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(ws.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        ctx->graph_failed = true;
        return;
    }
    body();
    cudaError_t e = cudaStreamEndCapture(ws.st, &g);
    ctx->step_launches = ws.launches - l0;
    ws.launches = l0;  // counted when the graph runs
    if (e == cudaSuccess && g) e = cudaGraphInstantiate(&ctx->step_exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess || !ctx->step_exec) {
        cudaGetLastError();
        ctx->step_exec = nullptr;
        ctx->graph_failed = true;
        return;
    }
    ctx->step_n = ws.n, ctx->step_dt = dt, ctx->step_epoch = ctx->epoch;
    ++ctx->graph_captures;
}

// Queue one RK4 step from the saved step start (rk4_begin): the captured
// graph when graphs are on, else every kernel. Asynchronous.
static void step_enqueue(gb_ctx *ctx, double dt) {
    gb::Workspace &ws = ctx->ws;
    const std::function<void()> body = [ctx, dt]() {
        gb::Workspace &w = ctx->ws;
        gb::rk4_restore(w);
        for (int stage = 0; stage < 4; ++stage) {
            evaluate(ctx, false);
            gb::rk4_stage(w, stage, dt);
        }
    };
    const bool graphs = !ws.timing && (ctx->cfg.flags & GB_FLAG_NO_GRAPH) == 0 && !ctx->graph_failed;
    if (graphs) {
        if (!ctx->step_exec || ctx->step_n != ws.n || ctx->step_dt != dt || ctx->step_epoch != ctx->epoch)
            capture_step(ctx, dt, body);
        if (ctx->step_exec && cudaGraphLaunch(ctx->step_exec, ws.st) == cudaSuccess) {
            ws.launches += ctx->step_launches;
            ++ctx->graph_steps;
            return;
        }
        cudaGetLastError();
    }
    body();
    ++ctx->direct_steps;
}

int gb_rk4_step(gb_ctx *ctx, double dt) {
    gb::NvtxRange nvtx_("gb_rk4_step");
    if (!ctx) return GB_ERR_INVALID;
    if (!ctx->have_state) return ctx->err = "no state uploaded", GB_ERR_STATE;
    if (!std::isfinite(dt)) return ctx->err = "dt must be finite", GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    if (ws.n == 0) return ++ctx->state_steps, GB_OK;
    gb::rk4_begin(ws);
    const int rc = run_with_capacity(ctx, [&]() { step_enqueue(ctx, dt); });
    if (rc != GB_OK) {
        // leave the state as it was before the step
        gb::rk4_restore(ws);
        cudaStreamSynchronize(ws.st);
    } else {
        ++ctx->state_steps;
    }
    return rc;
}

// ------------------------------------------------------------------- batches
// Many independent systems of uneven size (the batching form of the
// benchmark: systems concatenated with segment offsets), in one of two forms.
//  * Forest (default): one context holds every system. Each kernel class runs
//    as one launch over all systems (the tree kernels over all particles and
//    cells; the far-field kernels over tiles that each hold one system's
//    cells, with that system's operators), so a batch step is one step graph
//    of the same ~60 launches per force evaluation as a single system's.
//    Every system keeps its own root box, tree, operators, particle mass and
//    G m, and gets the results a context of its own computes (the same
//    operations in the same order per particle and per cell).
//  * Contexts (GB_FLAG_BATCH_CONTEXTS, and the accurate mode): every system
//    has its own context, tree, operators and step graph on its own stream;
//    a batch step queues all systems' steps before waiting for any. A system
//    whose buffers overflow is grown and stepped again on its own.
}  // extern "C"

struct gb_batch {
    std::vector<gb_ctx *> ctx;  // contexts form: one per system
    gb_ctx *forest = nullptr;   // forest form: one context over every system
    std::vector<uint64_t> off;  // nsys + 1 particle offsets
    std::vector<double> m;      // particle mass of each system
    long long steps = 0;        // batch steps since the state was set
    std::string err;
    size_t nsys() const { return off.size() - 1; }
};

namespace {

// Per-system data of a forest context: systems, their TreeInfo entries and
// operators, the system of every particle position, masses and G m.
int forest_setup(gb_ctx *ctx, size_t nsys, const uint64_t *off, const std::vector<double> &m) {
    gb::Workspace &ws = ctx->ws;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    const size_t n = off[nsys];
    ws.nsys = static_cast<int>(nsys);
    ws.sys_bits = 0;
    while ((1ull << ws.sys_bits) < nsys) ++ws.sys_bits;
    GB_TRY(dalloc(ws.info, nsys));
    GB_TRY(cudaMemset(ws.info, 0, sizeof(gb::TreeInfo) * nsys));
    const size_t kk = static_cast<size_t>(ws.K) * ws.K * gb::kNumOps * nsys;
    GB_TRY(dalloc(ws.ops_d, kk));
    GB_TRY(dalloc(ws.ops_f, kk));
    GB_TRY(dalloc(ws.zf, gb::zf_table_floats(ws.p) * nsys));
    GB_TRY(dalloc(ws.bimg, gb::m2l_tc_image_floats(ws.p) * nsys));
    GB_TRY(cudaMemset(ws.bimg, 0, sizeof(float) * gb::m2l_tc_image_floats(ws.p) * nsys));
    std::vector<unsigned> seg(nsys + 1);
    std::vector<int> ps(n);
    std::vector<double2> par(nsys);
    for (size_t k = 0; k <= nsys; ++k) seg[k] = static_cast<unsigned>(off[k]);
    for (size_t k = 0; k < nsys; ++k) {
        for (uint64_t i = off[k]; i < off[k + 1]; ++i) ps[i] = static_cast<int>(k);
        par[k] = make_double2(m[k], ws.G * m[k]);
    }
    GB_TRY(dalloc(ws.seg, nsys + 1));
    GB_TRY(cudaMemcpy(ws.seg, seg.data(), sizeof(unsigned) * (nsys + 1), cudaMemcpyHostToDevice));
    GB_TRY(dalloc(ws.psys, n));
    if (n) GB_TRY(cudaMemcpy(ws.psys, ps.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GB_TRY(dalloc(ws.sys_par, nsys));
    GB_TRY(cudaMemcpy(ws.sys_par, par.data(), sizeof(double2) * nsys, cudaMemcpyHostToDevice));
    GB_TRY(dalloc(ws.mkeys, n));
    GB_TRY(dalloc(ws.ocnt, 3 * nsys + 1));
    ws.sort_levels = std::min(ws.sort_levels, ws.sort_levels_cap());
    return GB_OK;
}

int forest_fail(gb_batch *b, int rc) {
    b->err = b->forest->err;
    return rc;
}

}  // namespace

extern "C" {

int gb_batch_create(const gb_config *cfg, size_t nsys, const uint64_t *seg_offsets, const double *m_per_system,
                    gb_batch **out) {
    if (!out) return GB_ERR_INVALID;
    *out = nullptr;
    if (!cfg || !seg_offsets || nsys == 0) {
        g_create_error = "batch needs a config, segment offsets and at least one system";
        return GB_ERR_INVALID;
    }
    for (size_t k = 0; k < nsys; ++k)
        if (seg_offsets[k + 1] < seg_offsets[k]) {
            g_create_error = "segment offsets must not decrease";
            return GB_ERR_INVALID;
        }
    if (seg_offsets[0] != 0) {
        g_create_error = "segment offsets must start at 0";
        return GB_ERR_INVALID;
    }
    auto *b = new gb_batch;
    b->off.assign(seg_offsets, seg_offsets + nsys + 1);
    b->m.resize(nsys);
    for (size_t k = 0; k < nsys; ++k) b->m[k] = m_per_system ? m_per_system[k] : cfg->m;
    const bool contexts = (cfg->flags & GB_FLAG_BATCH_CONTEXTS) != 0 || cfg->mode == GB_MODE_ACCURATE;
    if (!contexts) {
        if (seg_offsets[nsys] > 0x7fffffffu || nsys > 0x7fffffffu) {
            g_create_error = "too many particles or systems for one forest";
            delete b;
            return GB_ERR_INVALID;
        }
        for (size_t k = 0; k < nsys; ++k)
            if (!std::isfinite(b->m[k])) {
                g_create_error = "masses must be finite";
                delete b;
                return GB_ERR_INVALID;
            }
        gb_ctx *h = nullptr;
        int rc = gb_create(cfg, &h);
        if (rc == GB_OK) {
            rc = forest_setup(h, nsys, seg_offsets, b->m);
            if (rc != GB_OK) g_create_error = h->err;
        }
        if (rc != GB_OK) {
            gb_destroy(h);
            delete b;
            return rc;
        }
        b->forest = h;
        *out = b;
        return GB_OK;
    }
    for (size_t k = 0; k < nsys; ++k) {
        gb_config c = *cfg;
        c.m = b->m[k];
        gb_ctx *h = nullptr;
        const int rc = gb_create(&c, &h);
        if (rc != GB_OK) {
            for (gb_ctx *x : b->ctx) gb_destroy(x);
            delete b;
            return rc;
        }
        b->ctx.push_back(h);
    }
    *out = b;
    return GB_OK;
}

void gb_batch_destroy(gb_batch *b) {
    if (!b) return;
    for (gb_ctx *x : b->ctx) gb_destroy(x);
    gb_destroy(b->forest);
    delete b;
}

const char *gb_batch_last_error(const gb_batch *b) { return b ? b->err.c_str() : g_create_error.c_str(); }

int gb_batch_is_forest(const gb_batch *b) { return b && b->forest ? 1 : 0; }

gb_ctx *gb_batch_forest(gb_batch *b) { return b ? b->forest : nullptr; }

static int batch_fail(gb_batch *b, size_t k, int rc) {
    b->err = "system " + std::to_string(k) + ": " + b->ctx[k]->err;
    return rc;
}

int gb_batch_upload(gb_batch *b, const double *x_aos, const double *v_aos) {
    gb::NvtxRange nvtx_("gb_batch_upload");
    if (!b || !x_aos || !v_aos) return GB_ERR_INVALID;
    b->steps = 0;
    if (b->forest) {
        const int rc = gb_upload(b->forest, x_aos, v_aos, b->off.back());
        return rc == GB_OK ? rc : forest_fail(b, rc);
    }
    for (size_t k = 0; k < b->ctx.size(); ++k) {
        const uint64_t o = b->off[k], n = b->off[k + 1] - o;
        const int rc = gb_upload(b->ctx[k], x_aos + 3 * o, v_aos + 3 * o, n);
        if (rc != GB_OK) return batch_fail(b, k, rc);
    }
    return GB_OK;
}

int gb_batch_init_plummer(gb_batch *b, uint64_t seed, double r_lo, double r_hi, double r_max, double *radii) {
    return gb_batch_init_plummer_at(b, seed, 0, r_lo, r_hi, r_max, radii);
}

int gb_batch_init_plummer_at(gb_batch *b, uint64_t seed, uint64_t first, double r_lo, double r_hi, double r_max,
                             double *radii) {
    gb::NvtxRange nvtx_("gb_batch_init_plummer_at");
    if (!b) return GB_ERR_INVALID;
    if (!(r_lo > 0) || !(r_hi >= r_lo) || !std::isfinite(r_hi)) return b->err = "need 0 < r_lo <= r_hi", GB_ERR_INVALID;
    if (!(r_max > 0) || !std::isfinite(r_max)) return b->err = "r_max must be finite and > 0", GB_ERR_INVALID;
    auto mix = [](uint64_t z) {  // SplitMix64 output function, as the device streams (ic.cu)
        z += 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    };
    // system k: radius R_k from the batch seed, particle stream family mix(seed + k)
    const size_t ns = b->nsys();
    std::vector<uint64_t> seeds(ns);
    std::vector<double2> scales(ns);
    for (size_t k = 0; k < ns; ++k) {
        const uint64_t id = first + k;  // the system's index in the seeded family
        const double u = static_cast<double>(mix(mix(seed ^ 0x2545f4914f6cdd1dull) + id) >> 11) * 0x1.0p-53;
        const double R = r_lo + (r_hi - r_lo) * u;
        if (radii) radii[k] = R;
        seeds[k] = mix(seed + id);
        scales[k] = make_double2(R, 1.0 / std::sqrt(R));  // total mass 1, scale radius R (G = 1)
    }
    if (b->forest) {
        gb_ctx *ctx = b->forest;
        gb::Workspace &ws = ctx->ws;
        ctx->levels_fitted = false;
        if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return b->err = "cudaSetDevice failed", GB_ERR_CUDA;
        const size_t n = b->off.back();
        int rc = apply_tuning_cache(ctx, n);
        if (rc == GB_OK) rc = ensure_particles(ctx, static_cast<unsigned>(n));
        if (rc != GB_OK) return forest_fail(b, rc);
        ws.n = static_cast<unsigned>(n);
        uint64_t *d_seeds = nullptr;
        double2 *d_scales = nullptr;
        int err = 0;
        bool ok = dalloc(d_seeds, ns) == cudaSuccess && dalloc(d_scales, ns) == cudaSuccess &&
                  cudaMemcpy(d_seeds, seeds.data(), sizeof(uint64_t) * ns, cudaMemcpyHostToDevice) == cudaSuccess &&
                  cudaMemcpy(d_scales, scales.data(), sizeof(double2) * ns, cudaMemcpyHostToDevice) == cudaSuccess;
        if (ok && n) {
            gb::generate_plummer_forest(ws, d_seeds, d_scales, 1.0, r_max);
            ok = cudaMemcpyAsync(&err, &ws.info->err, sizeof(int), cudaMemcpyDeviceToHost, ws.st) == cudaSuccess &&
                 cudaStreamSynchronize(ws.st) == cudaSuccess;
        }
        dfree(d_seeds);
        dfree(d_scales);
        if (!ok) return b->err = "initial-condition generation failed", GB_ERR_CUDA;
        if (err) return b->err = "initial-condition sampling did not converge", GB_ERR_CUDA;
        if (n) {
            rc = initial_capacity(ctx);
            if (rc != GB_OK) return forest_fail(b, rc);
        }
        ctx->have_state = true;
        ctx->state_steps = 0;
        b->steps = 0;
        return GB_OK;
    }
    for (size_t k = 0; k < ns; ++k) {
        gb_ctx *ctx = b->ctx[k];
        const uint64_t n = b->off[k + 1] - b->off[k];
        ctx->levels_fitted = false;
        if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return batch_fail(b, k, GB_ERR_CUDA);
        gb::Workspace &ws = ctx->ws;
        int rc = apply_tuning_cache(ctx, n);
        if (rc == GB_OK) rc = ensure_particles(ctx, static_cast<unsigned>(n));
        if (rc != GB_OK) return batch_fail(b, k, rc);
        ws.n = static_cast<unsigned>(n);
        if (n) {
            gb::generate_plummer(ws, ws.n, seeds[k], 1.0, r_max, scales[k].x, scales[k].y);
            rc = initial_capacity(ctx);
            if (rc != GB_OK) return batch_fail(b, k, rc);
        }
        ctx->have_state = true;
        ctx->state_steps = 0;
    }
    for (size_t k = 0; k < ns; ++k) {
        gb::Workspace &ws = b->ctx[k]->ws;
        int err = 0;
        if (cudaMemcpyAsync(&err, &ws.info->err, sizeof(int), cudaMemcpyDeviceToHost, ws.st) != cudaSuccess ||
            cudaStreamSynchronize(ws.st) != cudaSuccess)
            return batch_fail(b, k, GB_ERR_CUDA);
        if (err) {
            b->ctx[k]->err = "initial-condition sampling did not converge";
            return batch_fail(b, k, GB_ERR_CUDA);
        }
    }
    b->steps = 0;
    return GB_OK;
}

int gb_batch_download(gb_batch *b, double *x_aos, double *v_aos) {
    gb::NvtxRange nvtx_("gb_batch_download");
    if (!b || !x_aos || !v_aos) return GB_ERR_INVALID;
    if (b->forest) {
        const int rc = gb_download(b->forest, x_aos, v_aos);
        return rc == GB_OK ? rc : forest_fail(b, rc);
    }
    for (size_t k = 0; k < b->ctx.size(); ++k) {
        const uint64_t o = b->off[k];
        const int rc = gb_download(b->ctx[k], x_aos + 3 * o, v_aos + 3 * o);
        if (rc != GB_OK) return batch_fail(b, k, rc);
    }
    return GB_OK;
}

int gb_batch_rk4_step(gb_batch *b, double dt) {
    gb::NvtxRange nvtx_("gb_batch_rk4_step");
    if (!b) return GB_ERR_INVALID;
    if (!std::isfinite(dt)) return b->err = "dt must be finite", GB_ERR_INVALID;
    if (b->forest) {
        if (!b->forest->have_state) return b->err = "no state uploaded", GB_ERR_STATE;
        const int rc = gb_rk4_step(b->forest, dt);
        if (rc == GB_OK) ++b->steps;
        return rc == GB_OK ? rc : forest_fail(b, rc);
    }
    const size_t ns = b->ctx.size();
    std::vector<char> live(ns, 0);
    for (size_t k = 0; k < ns; ++k) {
        if (!b->ctx[k]->have_state) return b->err = "system " + std::to_string(k) + ": no state uploaded", GB_ERR_STATE;
        live[k] = b->ctx[k]->ws.n > 0;
    }
    // queue every system's step; the host cost of a graph launch grows with its
    // node count, so several host threads queue disjoint sets of systems
    auto enqueue = [&](size_t k0, size_t k1) {
        for (size_t k = k0; k < k1; ++k) {
            if (!live[k]) continue;
            gb_ctx *c = b->ctx[k];
            cudaSetDevice(c->cfg.device);
            gb::rk4_begin(c->ws);
            step_enqueue(c, dt);
        }
    };
    const size_t nt = std::min<size_t>(GB_BATCH_THREADS, ns);
    if (nt <= 1) {
        enqueue(0, ns);
    } else {
        std::vector<std::thread> th;
        for (size_t t = 0; t < nt; ++t) th.emplace_back(enqueue, ns * t / nt, ns * (t + 1) / nt);
        for (auto &x : th) x.join();
    }
    int first_rc = GB_OK;
    for (size_t k = 0; k < ns; ++k) {  // then check them
        if (!live[k]) continue;
        gb_ctx *c = b->ctx[k];
        cudaSetDevice(c->cfg.device);
        unsigned counts[gb::kNumCounts];
        int rc = check_device_errors(c, counts);
        if (rc == GB_ERR_CAPACITY) {
            rc = grow(c, counts);
            if (rc == GB_OK) {
                ++c->retries;
                rc = run_with_capacity(c, [&]() { step_enqueue(c, dt); });
            }
        }
        if (rc != GB_OK) {
            gb::rk4_restore(c->ws);
            cudaStreamSynchronize(c->ws.st);
            if (first_rc == GB_OK) first_rc = batch_fail(b, k, rc);
        } else {
            ++c->state_steps;
        }
    }
    for (size_t k = 0; k < ns; ++k)
        if (!live[k]) ++b->ctx[k]->state_steps;
    if (first_rc == GB_OK) ++b->steps;
    return first_rc;
}

int gb_batch_size(const gb_batch *b, size_t *nsys, uint64_t *n_total) {
    if (!b) return GB_ERR_INVALID;
    if (nsys) *nsys = b->nsys();
    if (n_total) *n_total = b->off.back();
    return GB_OK;
}

gb_ctx *gb_batch_system(gb_batch *b, size_t k) { return b && k < b->ctx.size() ? b->ctx[k] : nullptr; }

// Potential buffers (allocated on the first request): ws.phi [N] in the
// caller's order, ws.phis [2][N] near and far parts in tree order, ws.diag.
int ensure_potential(gb_ctx *ctx) {
    gb::Workspace &ws = ctx->ws;
    if (ws.n <= ctx->phi_cap && ws.phi) return GB_OK;
    GB_TRY(dalloc(ws.phi, ws.n));
    GB_TRY(dalloc(ws.phis, 2 * static_cast<size_t>(ws.n)));
    if (!ws.diag) GB_TRY(dalloc(ws.diag, gb::diag_scratch_doubles()));
    ctx->phi_cap = ws.n;
    return GB_OK;
}

int gb_accel(gb_ctx *ctx, double *a_aos, double *phi) {
    gb::NvtxRange nvtx_("gb_accel");
    if (!ctx) return GB_ERR_INVALID;
    if (!ctx->have_state) return ctx->err = "no state uploaded", GB_ERR_STATE;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    if (ws.n == 0) return GB_OK;
    if (phi) {
        const int r = ensure_potential(ctx);
        if (r) return r;
    }
    const int rc = run_with_capacity(ctx, [&]() { evaluate(ctx); });
    if (rc) return rc;
    if (a_aos)  // acc is [N][3] already
        GB_TRY(cudaMemcpyAsync(a_aos, ws.acc, sizeof(double) * 3 * ws.n, cudaMemcpyDeviceToHost, ws.st));
    if (phi) {
        gb::potential_orig(ws, ws.phi);
        GB_TRY(cudaMemcpyAsync(phi, ws.phi, sizeof(double) * ws.n, cudaMemcpyDeviceToHost, ws.st));
    }
    GB_TRY(cudaStreamSynchronize(ws.st));
    return GB_OK;
}

int gb_get_conserved(gb_ctx *ctx, gb_conserved *out) {
    gb::NvtxRange nvtx_("gb_get_conserved");
    if (!ctx || !out) return GB_ERR_INVALID;
    if (!ctx->have_state) return ctx->err = "no state uploaded", GB_ERR_STATE;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    std::memset(out, 0, sizeof(*out));
    if (ws.n == 0) return GB_OK;
    int rc = ensure_potential(ctx);
    if (rc) return rc;
    rc = run_with_capacity(ctx, [&]() { evaluate(ctx); });
    if (rc) return rc;
    gb::potential_orig(ws, ws.phi);
    double *sums = ws.diag + gb::diag_scratch_doubles() - 8;
    gb::conserved_sums(ws, ws.phi, sums);
    double h[8];
    GB_TRY(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, ws.st));
    GB_TRY(cudaStreamSynchronize(ws.st));
    const double m = ws.m;
    out->kinetic = 0.5 * m * h[0];
    out->potential = 0.5 * m * h[1];
    out->total = out->kinetic + out->potential;
    for (int a = 0; a < 3; ++a) out->momentum[a] = m * h[2 + a], out->angular_momentum[a] = m * h[5 + a];
    return GB_OK;
}

int gb_direct_accel(gb_ctx *ctx, const int64_t *targets, size_t ntargets, double *a_aos) {
    gb::NvtxRange nvtx_("gb_direct_accel");
    if (!ctx) return GB_ERR_INVALID;
    if (!ctx->have_state) return ctx->err = "no state uploaded", GB_ERR_STATE;
    if (!a_aos) return ctx->err = "null output", GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    const size_t nt = targets ? ntargets : ws.n;
    if (nt > 0x7fffffffu) return ctx->err = "too many targets", GB_ERR_INVALID;
    if (nt == 0 || ws.n == 0) return GB_OK;
    if (targets) {
        for (size_t k = 0; k < nt; ++k)
            if (targets[k] < 0 || static_cast<uint64_t>(targets[k]) >= ws.n) return ctx->err = "target out of range", GB_ERR_INVALID;
        if (nt > ctx->targets_cap) {
            GB_TRY(dalloc(ctx->d_targets, nt));
            ctx->targets_cap = nt;
        }
        GB_TRY(cudaMemcpyAsync(ctx->d_targets, targets, sizeof(long long) * nt, cudaMemcpyHostToDevice, ws.st));
    }
    const unsigned nsplit = gb::direct_nsplit(ws.n, static_cast<unsigned>(nt), ws.num_sms);
    const size_t need = 3 * nt * (1 + static_cast<size_t>(nsplit));  // result planes + per-slice partial sums
    if (need > ctx->direct_cap) {
        GB_TRY(dalloc(ctx->d_direct, need));
        ctx->direct_cap = need;
    }
    gb::direct_sum(ws, ws.x, targets ? ctx->d_targets : nullptr, static_cast<unsigned>(nt), ctx->d_direct,
                   ctx->d_direct + 3 * nt, nsplit);
    std::vector<double> soa(3 * nt);
    GB_TRY(cudaMemcpyAsync(soa.data(), ctx->d_direct, sizeof(double) * 3 * nt, cudaMemcpyDeviceToHost, ws.st));
    GB_TRY(cudaStreamSynchronize(ws.st));
    GB_TRY(cudaGetLastError());
    for (size_t k = 0; k < nt; ++k)
        for (int a = 0; a < 3; ++a) a_aos[3 * k + a] = soa[a * nt + k];
    return GB_OK;
}

int gb_sync(gb_ctx *ctx) {
    gb::NvtxRange nvtx_("gb_sync");
    if (!ctx) return GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    GB_TRY(cudaStreamSynchronize(ctx->ws.st));
    GB_TRY(cudaGetLastError());
    return GB_OK;
}

int gb_get_stats(gb_ctx *ctx, gb_stats *out) {
    if (!ctx || !out) return GB_ERR_INVALID;
    const gb::TreeInfo &h = *ctx->ws.h_info;
    out->n = ctx->ws.n;
    out->ncells = h.ncells;
    out->nleaves = h.nleaves;
    out->depth = h.depth;
    out->m2l_pairs = h.m2l_pairs;
    out->p2p_pairs = h.p2p_pairs;
    out->p2p_ranges = h.p2p_ranges;
    out->retries = ctx->retries;
    out->graph_steps = ctx->graph_steps;
    out->graph_captures = ctx->graph_captures;
    out->direct_steps = ctx->direct_steps;
    out->steps = ctx->state_steps;
    return GB_OK;
}

// Batch accessors: the contexts form asks each system's context; the forest
// form evaluates the whole forest once and splits the results by system.
int gb_batch_accel(gb_batch *b, double *a_aos, double *phi) {
    gb::NvtxRange nvtx_("gb_batch_accel");
    if (!b) return GB_ERR_INVALID;
    if (b->forest) {
        const int rc = gb_accel(b->forest, a_aos, phi);
        return rc == GB_OK ? rc : forest_fail(b, rc);
    }
    for (size_t k = 0; k < b->ctx.size(); ++k) {
        const uint64_t o = b->off[k];
        if (b->off[k + 1] == o) continue;
        const int rc = gb_accel(b->ctx[k], a_aos ? a_aos + 3 * o : nullptr, phi ? phi + o : nullptr);
        if (rc != GB_OK) return batch_fail(b, k, rc);
    }
    return GB_OK;
}

int gb_batch_conserved(gb_batch *b, gb_conserved *out) {
    gb::NvtxRange nvtx_("gb_batch_conserved");
    if (!b || !out) return GB_ERR_INVALID;
    const size_t ns = b->nsys();
    if (!b->forest) {
        for (size_t k = 0; k < ns; ++k) {
            const int rc = gb_get_conserved(b->ctx[k], out + k);
            if (rc != GB_OK) return batch_fail(b, k, rc);
        }
        return GB_OK;
    }
    // forest: the potentials of one evaluation, then the sums per system in FP64 on the host
    const size_t n = b->off.back();
    std::vector<double> x(3 * n), v(3 * n), phi(n);
    int rc = n ? gb_batch_accel(b, nullptr, phi.data()) : GB_OK;
    if (rc == GB_OK && n) rc = gb_batch_download(b, x.data(), v.data());
    if (rc != GB_OK) return rc;
    for (size_t k = 0; k < ns; ++k) {
        double h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (uint64_t i = b->off[k]; i < b->off[k + 1]; ++i) {
            const double *xi = &x[3 * i], *vi = &v[3 * i];
            h[0] += vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2];
            h[1] += phi[i];
            for (int a = 0; a < 3; ++a) h[2 + a] += vi[a];
            h[5] += xi[1] * vi[2] - xi[2] * vi[1];
            h[6] += xi[2] * vi[0] - xi[0] * vi[2];
            h[7] += xi[0] * vi[1] - xi[1] * vi[0];
        }
        const double m = b->m[k];
        gb_conserved &o = out[k];
        o.kinetic = 0.5 * m * h[0];
        o.potential = 0.5 * m * h[1];
        o.total = o.kinetic + o.potential;
        for (int a = 0; a < 3; ++a) o.momentum[a] = m * h[2 + a], o.angular_momentum[a] = m * h[5 + a];
    }
    return GB_OK;
}

int gb_batch_stats(gb_batch *b, gb_stats *out) {
    if (!b || !out) return GB_ERR_INVALID;
    if (b->forest) {
        gb_get_stats(b->forest, out);
        out->steps = b->steps;
        return GB_OK;
    }
    std::memset(out, 0, sizeof(*out));
    for (gb_ctx *c : b->ctx) {
        gb_stats t;
        gb_get_stats(c, &t);
        out->n += t.n, out->ncells += t.ncells, out->nleaves += t.nleaves, out->depth = std::max(out->depth, t.depth);
        out->m2l_pairs += t.m2l_pairs, out->p2p_pairs += t.p2p_pairs, out->p2p_ranges += t.p2p_ranges;
        out->retries += t.retries, out->graph_steps += t.graph_steps, out->direct_steps += t.direct_steps;
        out->graph_captures += t.graph_captures;
    }
    out->steps = b->steps;
    return GB_OK;
}

int64_t gb_batch_launch_count(const gb_batch *b) {
    if (!b) return 0;
    if (b->forest) return b->forest->ws.launches;
    int64_t t = 0;
    for (const gb_ctx *c : b->ctx) t += c->ws.launches;
    return t;
}

}  // extern "C"

namespace {

// Leaf parameter a context builds its trees with.
int leaf_param(const gb_ctx *ctx) {
    return ctx->cfg.mode == GB_MODE_ACCURATE && ctx->tune.leaf_s > 0 ? ctx->tune.leaf_s : ctx->cfg.s;
}

// The leaf parameter an upload of n particles would give the context (the
// tuning cache's entry for n's bucket, when the upload would apply one),
// without applying anything.
int leaf_param_for(const gb_ctx *ctx, size_t n) {
    gb_tuning t = ctx->tune;
    const char *path = std::getenv("VIPP_GB_TUNE_FILE");
    if (path && *path && n && floor_log2(n) != ctx->tune_log2n) {
        gb_tuning ft{};
        std::string msg;
        if (tuning_from_file(path, &ctx->cfg, n, &ft, msg) == GB_OK) t = ft;
    }
    return ctx->cfg.mode == GB_MODE_ACCURATE && t.leaf_s > 0 ? t.leaf_s : ctx->cfg.s;
}

gb_checkpoint_info info_of(const gb_ctx *ctx, uint64_t n, uint64_t nsys, long long steps, double t) {
    gb_checkpoint_info in{};
    in.n = n;
    in.nsys = nsys;
    in.steps = steps;
    in.t = t;
    in.cfg = ctx->cfg;
    in.cfg.device = 0;
    in.leaf_s = leaf_param(ctx);
    return in;
}

// Empty when a checkpoint written with f's configuration continues in ctx
// with the same results; else what differs. Batches compare their masses
// per system instead of m, and leave out the leaf parameter (their contexts
// take it from the tuning cache per system size, the same on a reload).
std::string config_mismatch(const gb_checkpoint_info &f, const gb_ctx *ctx, bool one_system, int leaf_now) {
    const gb_config &c = ctx->cfg;
    constexpr int kResultFlags = GB_FLAG_P2P_NEWTON | GB_FLAG_M2L_CUDA_CORES | GB_FLAG_M2L_BF16;
    auto num = [](double v) {
        char buf[40];
        std::snprintf(buf, sizeof buf, "%.17g", v);
        return std::string(buf);
    };
    auto differs = [](const char *what, const std::string &a, const std::string &b) {
        return std::string(what) + " " + a + " (context " + b + ")";
    };
    if (f.cfg.p != c.p) return differs("p", std::to_string(f.cfg.p), std::to_string(c.p));
    if (f.cfg.s != c.s) return differs("s", std::to_string(f.cfg.s), std::to_string(c.s));
    if (f.cfg.precision != c.precision)
        return differs("precision", std::to_string(f.cfg.precision), std::to_string(c.precision));
    if (f.cfg.mode != c.mode) return differs("mode", std::to_string(f.cfg.mode), std::to_string(c.mode));
    if ((f.cfg.flags ^ c.flags) & kResultFlags)
        return differs("flags", std::to_string(f.cfg.flags & kResultFlags), std::to_string(c.flags & kResultFlags));
    if (f.cfg.eps != c.eps) return differs("eps", num(f.cfg.eps), num(c.eps));
    if (f.cfg.G != c.G) return differs("G", num(f.cfg.G), num(c.G));
    if (one_system && f.cfg.m != c.m) return differs("m", num(f.cfg.m), num(c.m));
    if (one_system && f.leaf_s != leaf_now) return differs("leaf_s", std::to_string(f.leaf_s), std::to_string(leaf_now));
    return std::string();
}

}  // namespace

extern "C" {

int gb_checkpoint_write(const char *path, const gb_checkpoint_info *info, const uint64_t *seg_offsets,
                        const double *m_per_system, const double *x_aos, const double *v_aos) {
    std::string err;
    const int rc = gb::checkpoint_write(path, info, seg_offsets, m_per_system, x_aos, v_aos, err);
    if (rc != GB_OK) g_create_error = err;
    return rc;
}

int gb_checkpoint_read(const char *path, gb_checkpoint_info *info, uint64_t *seg_offsets, double *m_per_system,
                       size_t nsys_cap, double *x_aos, double *v_aos, size_t n_cap) {
    std::string err;
    const int rc = gb::checkpoint_read(path, info, seg_offsets, m_per_system, nsys_cap, x_aos, v_aos, n_cap, err);
    if (rc != GB_OK) g_create_error = err;
    return rc;
}

int gb_checkpoint_save(gb_ctx *ctx, const char *path, double t) {
    gb::NvtxRange nvtx_("gb_checkpoint_save");
    if (!ctx) return GB_ERR_INVALID;
    if (ctx->ws.forest()) return ctx->err = "a forest context is saved through its batch", GB_ERR_INVALID;
    if (!ctx->have_state) return ctx->err = "no state uploaded", GB_ERR_STATE;
    const uint64_t n = ctx->ws.n;
    std::vector<double> x(3 * n + 1), v(3 * n + 1);
    int rc = gb_download(ctx, x.data(), v.data());
    if (rc != GB_OK) return rc;
    const gb_checkpoint_info info = info_of(ctx, n, 1, ctx->state_steps, t);
    std::string err;
    rc = gb::checkpoint_write(path, &info, nullptr, nullptr, x.data(), v.data(), err);
    if (rc != GB_OK) ctx->err = err;
    return rc;
}

int gb_checkpoint_load(gb_ctx *ctx, const char *path, int flags, double *t) {
    gb::NvtxRange nvtx_("gb_checkpoint_load");
    if (!ctx) return GB_ERR_INVALID;
    if (ctx->ws.forest()) return ctx->err = "a forest context is loaded through its batch", GB_ERR_INVALID;
    gb_checkpoint_info info;
    std::string err;
    int rc = gb::checkpoint_read(path, &info, nullptr, nullptr, 0, nullptr, nullptr, 0, err);
    if (rc != GB_OK) return ctx->err = err, rc;
    if (info.nsys != 1)
        return ctx->err = "the checkpoint holds " + std::to_string(info.nsys) + " systems; load it into a batch",
               GB_ERR_INVALID;
    if (info.n > 0x7fffffffu) return ctx->err = "too many particles", GB_ERR_INVALID;
    if (!(flags & GB_CHECKPOINT_ANY_CONFIG)) {
        const std::string d = config_mismatch(info, ctx, true, leaf_param_for(ctx, info.n));
        if (!d.empty()) return ctx->err = "checkpoint configuration differs: " + d, GB_ERR_INVALID;
    }
    std::vector<double> x(3 * info.n + 1), v(3 * info.n + 1);
    double m = 0;
    rc = gb::checkpoint_read(path, &info, nullptr, &m, 1, x.data(), v.data(), info.n, err);
    if (rc != GB_OK) return ctx->err = err, rc;
    rc = gb_upload(ctx, x.data(), v.data(), info.n);
    if (rc != GB_OK) return rc;
    ctx->state_steps = info.steps;
    if (t) *t = info.t;
    return GB_OK;
}

int gb_batch_checkpoint_save(gb_batch *b, const char *path, double t) {
    gb::NvtxRange nvtx_("gb_batch_checkpoint_save");
    if (!b) return GB_ERR_INVALID;
    const uint64_t n = b->off.back();
    std::vector<double> x(3 * n + 1), v(3 * n + 1);
    int rc = gb_batch_download(b, x.data(), v.data());
    if (rc != GB_OK) return rc;
    const gb_ctx *rep = b->forest ? b->forest : b->ctx[0];
    const gb_checkpoint_info info = info_of(rep, n, b->nsys(), b->steps, t);
    std::string err;
    rc = gb::checkpoint_write(path, &info, b->off.data(), b->m.data(), x.data(), v.data(), err);
    if (rc != GB_OK) b->err = err;
    return rc;
}

int gb_batch_checkpoint_load(gb_batch *b, const char *path, int flags, double *t) {
    gb::NvtxRange nvtx_("gb_batch_checkpoint_load");
    if (!b) return GB_ERR_INVALID;
    gb_checkpoint_info info;
    std::string err;
    int rc = gb::checkpoint_read(path, &info, nullptr, nullptr, 0, nullptr, nullptr, 0, err);
    if (rc != GB_OK) return b->err = err, rc;
    const size_t ns = b->nsys();
    const uint64_t n = b->off.back();
    if (info.nsys != ns || info.n != n)
        return b->err = "the checkpoint holds " + std::to_string(info.nsys) + " systems and " + std::to_string(info.n) +
                        " particles; the batch " + std::to_string(ns) + " and " + std::to_string(n),
               GB_ERR_INVALID;
    std::vector<uint64_t> seg(ns + 1);
    std::vector<double> m(ns), x(3 * n + 1), v(3 * n + 1);
    rc = gb::checkpoint_read(path, &info, seg.data(), m.data(), ns, x.data(), v.data(), n, err);
    if (rc != GB_OK) return b->err = err, rc;
    if (seg != b->off) return b->err = "checkpoint segment offsets differ from the batch's", GB_ERR_INVALID;
    if (!(flags & GB_CHECKPOINT_ANY_CONFIG)) {
        for (size_t k = 0; k < ns; ++k)
            if (m[k] != b->m[k]) return b->err = "checkpoint mass of system " + std::to_string(k) + " differs", GB_ERR_INVALID;
        const std::string d = config_mismatch(info, b->forest ? b->forest : b->ctx[0], false, 0);
        if (!d.empty()) return b->err = "checkpoint configuration differs: " + d, GB_ERR_INVALID;
    }
    rc = gb_batch_upload(b, x.data(), v.data());
    if (rc != GB_OK) return rc;
    b->steps = info.steps;
    if (b->forest) b->forest->state_steps = info.steps;
    for (gb_ctx *c : b->ctx) c->state_steps = info.steps;
    if (t) *t = info.t;
    return GB_OK;
}

int gb_tree_dump(gb_ctx *ctx, int64_t *ncells, int64_t *list_sizes, int32_t *level, int64_t *parent, int64_t *first_child,
                 uint64_t *path, double *box_min, double *box_max, int64_t *pt_begin, int64_t *pt_end, int64_t *order,
                 int64_t *m2l_off, int64_t *m2l, int64_t *p2p_off, int64_t *p2p_own, int64_t *coll_off, int64_t *coll) {
    if (!ctx || !ncells || !list_sizes) return GB_ERR_INVALID;
    if (level && !(parent && first_child && path && box_min && box_max && pt_begin && pt_end && order && m2l_off && m2l &&
                   p2p_off && p2p_own && coll_off && coll))
        return ctx->err = "tree dump: give every output array or none", GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    gb::Workspace &ws = ctx->ws;
    GB_TRY(cudaStreamSynchronize(ws.st));
    const int C = ctx->ws.h_info->ncells;
    if (ws.n == 0 || C <= 0) {
        *ncells = 0;
        list_sizes[0] = list_sizes[1] = list_sizes[2] = 0;
        return GB_OK;
    }
    std::vector<int> lv(C), par(C), ch(C), b(C), e(C), m2ls(static_cast<size_t>(C) * gb::kM2LSlots),
        pown(static_cast<size_t>(C) * gb::kNbrCap), pcnt(C), col(static_cast<size_t>(C) * gb::kNbrCap), ccnt(C);
    std::vector<uint64_t> pth(C);
    std::vector<double> box(6 * static_cast<size_t>(C));
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ws.st);
    };
    GB_TRY(cp(lv.data(), ws.c_level, sizeof(int) * C));
    GB_TRY(cp(par.data(), ws.c_parent, sizeof(int) * C));
    GB_TRY(cp(ch.data(), ws.c_child, sizeof(int) * C));
    GB_TRY(cp(b.data(), ws.c_begin, sizeof(int) * C));
    GB_TRY(cp(e.data(), ws.c_end, sizeof(int) * C));
    GB_TRY(cp(pth.data(), ws.c_path, sizeof(uint64_t) * C));
    GB_TRY(cp(box.data(), ws.c_box, sizeof(double) * 6 * C));
    GB_TRY(cp(m2ls.data(), ws.m2l_src, sizeof(int) * m2ls.size()));
    GB_TRY(cp(pown.data(), ws.p2p_own, sizeof(int) * pown.size()));
    GB_TRY(cp(pcnt.data(), ws.p2p_cnt, sizeof(int) * C));
    GB_TRY(cp(col.data(), ws.coll, sizeof(int) * col.size()));
    GB_TRY(cp(ccnt.data(), ws.coll_cnt, sizeof(int) * C));
    std::vector<unsigned> perm(ws.n);
    GB_TRY(cp(perm.data(), ws.perm, sizeof(unsigned) * ws.n));
    GB_TRY(cudaStreamSynchronize(ws.st));
    // M2L lists in the reference's order: slots sorted by source cell number
    std::vector<std::vector<int>> ml(C);
    size_t nm = 0, np = 0, nc = 0;
    for (int c = 0; c < C; ++c) {
        if (lv[c] >= 2) {
            for (int s = 0; s < gb::kM2LSlots; ++s) {
                const int u = m2ls[static_cast<size_t>(c) * gb::kM2LSlots + s];
                if (u >= 0) ml[c].push_back(u);
            }
            std::sort(ml[c].begin(), ml[c].end());
        }
        nm += ml[c].size();
        np += static_cast<size_t>(pcnt[c]);
        nc += static_cast<size_t>(ccnt[c]);
    }
    *ncells = C;
    list_sizes[0] = static_cast<int64_t>(nm);
    list_sizes[1] = static_cast<int64_t>(np);
    list_sizes[2] = static_cast<int64_t>(nc);
    if (!level) return GB_OK;
    size_t a = 0, bb = 0, cc = 0;
    for (int c = 0; c < C; ++c) {
        level[c] = lv[c];
        parent[c] = par[c];
        first_child[c] = ch[c];
        path[c] = pth[c];
        for (int k = 0; k < 3; ++k) box_min[3 * c + k] = box[6 * static_cast<size_t>(c) + k], box_max[3 * c + k] = box[6 * static_cast<size_t>(c) + 3 + k];
        pt_begin[c] = b[c];
        pt_end[c] = e[c];
        m2l_off[c] = static_cast<int64_t>(a);
        for (int u : ml[c]) m2l[a++] = u;
        p2p_off[c] = static_cast<int64_t>(bb);
        for (int k = 0; k < pcnt[c]; ++k) p2p_own[bb++] = pown[static_cast<size_t>(c) * gb::kNbrCap + k];
        coll_off[c] = static_cast<int64_t>(cc);
        for (int k = 0; k < ccnt[c]; ++k) coll[cc++] = col[static_cast<size_t>(c) * gb::kNbrCap + k];
    }
    m2l_off[C] = static_cast<int64_t>(a);
    p2p_off[C] = static_cast<int64_t>(bb);
    coll_off[C] = static_cast<int64_t>(cc);
    for (unsigned j = 0; j < ws.n; ++j) order[j] = perm[j];
    return GB_OK;
}

int gb_enable_timing(gb_ctx *ctx, int on) {
    if (!ctx) return GB_ERR_INVALID;
    ctx->ws.timing = on != 0;
    return GB_OK;
}

int gb_kernel_times(gb_ctx *ctx, double *ms, int64_t *launches, int n) {
    if (!ctx) return GB_ERR_INVALID;
    GB_TRY(cudaSetDevice(ctx->cfg.device));
    GB_TRY(cudaStreamSynchronize(ctx->ws.st));
    collect_timers(ctx);
    for (int k = 0; k < n && k < gb::kNumTimers; ++k) {
        if (ms) ms[k] = ctx->ws.t_ms[k];
        if (launches) launches[k] = ctx->ws.t_launch[k];
        ctx->ws.t_ms[k] = 0;
        ctx->ws.t_launch[k] = 0;
    }
    return GB_OK;
}

int64_t gb_launch_count(const gb_ctx *ctx) { return ctx ? ctx->ws.launches : 0; }

void *gb_stream(gb_ctx *ctx) { return ctx ? static_cast<void *>(ctx->ws.st) : nullptr; }

}  // extern "C"
