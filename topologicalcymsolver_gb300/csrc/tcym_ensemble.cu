// Ensembles: many independent lattices (mixed groups, sizes, precisions and
// dynamics) advanced together.  The reference runs such trajectories as
// independent MPI ranks that only share a seed (SU2Solver.cpp:161-164); here
// they share launches on one GPU.
//
// Per step and per storage format present, one persistent batched kernel
// (k_step_batch) covers every member of that format; the formats run as
// independent chains on their own streams.  A chunk of K steps is captured
// once as a CUDA graph and replayed; the member table (ping-pong parity and
// noise counters) is refreshed in device memory before each replay, so the
// graph is rebuilt only when membership or K changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <tuple>
#include <vector>

#include "../../include/tcym.h"
#include "tcym_batch.cuh"
#include "tcym_internal.h"

// TCYM_BATCH_PERSISTENT (tcym_batch.cuh) 0, the default: one block per work
// item, scheduled by the hardware, so the formats' launches interleave on the
// SMs and tails fill; 1: one wave of resident blocks walking the work items
// (measured 6% slower on a 256-member mixed ensemble).

using namespace tcym;

namespace {

struct EnsMember {
    tcym_lattice lat;
    int mode;
    double dt, gamma, T;
    uint64_t seed, next_step;
};

struct FmtGroup {
    std::vector<int> idx;        // members of this format, in ensemble order
    void *d_members = nullptr;   // device Member<T> table
    size_t d_bytes = 0;
    std::vector<char> h_members; // host copy of the table
    int total_blocks = 0, red_total = 0, grid = 0, red_grid = 0, red_offset = 0;
    bool general = false;        // some member is unpaired or tiled: the general batch kernel
    // runs of members (idx is ordered by coefficients) that share the mode, force, staple
    // and link factors: each steps in one launch with them as kernel parameters
    struct Class {
        StepCoef<double> coef;
        int m0, m1, item0, item1;
        // persistent launches: groups of members (class-relative first blocks) and the
        // offsets of the class's schedule and control words in the format's arrays
        std::vector<int> group_first_block;
        int sched_off = 0, ctl_off = 0;
    };
    std::vector<Class> classes;
    std::vector<int> member_block;             // first block of each member (idx order)
    int *d_sched = nullptr, *d_ctl = nullptr;  // persistent schedules and control words
    size_t sched_cap = 0, ctl_cap = 0, ctl_used = 0;
    std::vector<int> h_sched;
};

int fail(tcym_ctx ctx, cudaError_t e, const char *w) {
    tcym_set_error(ctx, "%s: %s", w, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TCYM_ERR_OOM : TCYM_ERR_CUDA;
}

}  // namespace

struct tcym_ensemble_s {
    tcym_ctx ctx = nullptr;
    std::vector<EnsMember> members;
    FmtGroup groups[4];
    cudaStream_t st[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[4] = {nullptr, nullptr, nullptr, nullptr};
    double *partial = nullptr;
    size_t partial_records = 0;
    MemberReduce *d_reduce = nullptr;
    double *d_out = nullptr, *h_out = nullptr;
    size_t reduce_cap = 0;
    cudaGraphExec_t exec = nullptr;
    int graph_steps = -1;
    bool layout_dirty = true;
    // K-step persistent launches per coefficient class (k_step_persistent) instead of
    // one launch per step; group_blocks: blocks per member group (0: one group)
    bool persistent = false;
    int group_blocks = 0;
    std::vector<int> h_ctl;
};

#define CKE(call)                                                 \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return fail(ens->ctx, e_, #call);  \
    } while (0)

template <int FMT> static void fill_group(tcym_ensemble ens, FmtGroup &G, int sm_count) {
    using T = typename Fmt<FMT>::T;
    constexpr int TPB = threads_for<FMT>();
    std::vector<Member<T>> tab(G.idx.size());
    int blk = 0, red = 0;
    G.general = false;
    G.classes.clear();
    G.member_block.assign(G.idx.size(), 0);
    for (size_t i = 0; i < G.idx.size(); ++i) {
        const EnsMember &em = ens->members[G.idx[i]];
        const tcym_lattice L = em.lat;
        Member<T> &m = tab[i];
        m.g = L->g;
        m.U[0] = L->U[0];
        m.U[1] = L->U[1];
        m.E = L->E;
        m.result = L->result;
        const StepCoef<double> cd = tcym_coef(L->a, em.mode, em.dt, em.gamma, em.T, em.seed, em.next_step);
        m.c = coef_cast<T>(cd);
        const FmtGroup::Class *last = G.classes.empty() ? nullptr : &G.classes.back();
        if (!last || cd.mode != last->coef.mode || std::memcmp(cd.fc, last->coef.fc, sizeof cd.fc) ||
            std::memcmp(cd.cnu, last->coef.cnu, sizeof cd.cnu) || std::memcmp(cd.uc, last->coef.uc, sizeof cd.uc))
            G.classes.push_back(FmtGroup::Class{cd, (int)i, (int)i, blk, blk});
        m.cur = L->cur;
        m.block_begin = blk;
        G.member_block[i] = blk;
        m.paired = Fmt<FMT>::PAIRED && L->g.nz % 2 == 0;
        m.tile = m.paired ? tcym_lattice_tile_of(L) : Tile{0, 0, 0, 0, 0, 0};
        if (!m.paired || m.tile.tx != 0) G.general = true;
        blk += m.paired ? (int)tile_blocks(L->g, m.tile) : grid_for(L->g.V, TPB);
        G.classes.back().m1 = (int)i + 1;
        G.classes.back().item1 = blk;
        m.red_begin = red;
        m.red_blocks = grid_for(L->g.V, kRedThreads);
        red += m.red_blocks;
        m.ncs_dt = 0.0;
    }
    G.total_blocks = blk;
    G.red_total = red;
#if TCYM_BATCH_PERSISTENT
    G.grid = std::max(1, std::min(blk, sm_count * LaunchBatch<FMT>::resident_blocks()));
#else
    G.grid = std::max(1, blk);
#endif
    G.red_grid = std::max(1, std::min(red, sm_count * 8));
    G.h_members.resize(sizeof(Member<T>) * tab.size());
    if (!tab.empty()) std::memcpy(G.h_members.data(), tab.data(), G.h_members.size());
}

static void fill_all(tcym_ensemble ens) {
    for (int f = 0; f < 4; ++f) ens->groups[f].idx.clear();
    for (size_t i = 0; i < ens->members.size(); ++i) ens->groups[ens->members[i].lat->fmt].idx.push_back((int)i);
    // members with the same step coefficients next to each other (mode, dt, spacings decide them)
    for (auto &G : ens->groups)
        std::stable_sort(G.idx.begin(), G.idx.end(), [&](int x, int y) {
            const EnsMember &a = ens->members[x], &b = ens->members[y];
            return std::make_tuple(a.mode, a.dt, a.lat->a[0], a.lat->a[1], a.lat->a[2]) <
                   std::make_tuple(b.mode, b.dt, b.lat->a[0], b.lat->a[1], b.lat->a[2]);
        });
    const int sm = ens->ctx->sm_count;
    fill_group<FMT_SU2_F32>(ens, ens->groups[FMT_SU2_F32], sm);
    fill_group<FMT_SU2_F64>(ens, ens->groups[FMT_SU2_F64], sm);
    fill_group<FMT_SU3_F32>(ens, ens->groups[FMT_SU3_F32], sm);
    fill_group<FMT_SU3_F64>(ens, ens->groups[FMT_SU3_F64], sm);
    int off = 0;
    for (int f = 0; f < 4; ++f) {
        ens->groups[f].red_offset = off;
        off += ens->groups[f].red_total;
    }
}

// Members of each class cut into groups of at least ens->group_blocks blocks (one
// group when 0); a member is never split.
static void plan_groups(tcym_ensemble ens, FmtGroup &G) {
    G.ctl_used = 0;
    for (FmtGroup::Class &c : G.classes) {
        c.group_first_block.assign(1, 0);
        int start = c.item0;
        for (int i = c.m0; i + 1 < c.m1; ++i) {
            const int next = G.member_block[i + 1];
            if (ens->group_blocks > 0 && next - start >= ens->group_blocks) {
                c.group_first_block.push_back(next - c.item0);
                start = next;
            }
        }
        c.group_first_block.push_back(c.item1 - c.item0);
        c.ctl_off = (int)G.ctl_used;
        G.ctl_used += 2 + (size_t)(c.m1 - c.m0);
    }
}

// Sizes the device tables and scratch for the current members and uploads the tables.
static int upload_tables(tcym_ensemble ens) {
    fill_all(ens);
    size_t records = 0;
    for (int f = 0; f < 4; ++f) {
        FmtGroup &G = ens->groups[f];
        records += (size_t)G.red_total;
        // device tables grow by doubling: cudaFree synchronises the device, so
        // members that come and go (the request loop) rarely reallocate
        if (G.h_members.size() > G.d_bytes) {
            cudaFree(G.d_members);
            G.d_members = nullptr;
            const size_t cap = std::max(G.h_members.size(), 2 * G.d_bytes);
            G.d_bytes = 0;
            CKE(cudaMalloc(&G.d_members, cap));
            G.d_bytes = cap;
            ens->layout_dirty = true;
        }
        if (!G.h_members.empty())
            CKE(cudaMemcpyAsync(G.d_members, G.h_members.data(), G.h_members.size(), cudaMemcpyHostToDevice,
                                ens->st[0]));
    }
    if (records > ens->partial_records) {
        cudaFree(ens->partial);
        ens->partial = nullptr;
        const size_t cap = std::max(records, 2 * ens->partial_records);
        ens->partial_records = 0;
        CKE(cudaMalloc(&ens->partial, sizeof(double) * P_WIDTH * cap));
        ens->partial_records = cap;
        ens->layout_dirty = true;
    }
    const size_t n0 = ens->members.size();
    if (n0 > ens->reduce_cap) {
        const size_t n = std::max(n0, 2 * ens->reduce_cap);
        cudaFree(ens->d_reduce);
        cudaFree(ens->d_out);
        cudaFreeHost(ens->h_out);
        ens->d_reduce = nullptr;
        ens->d_out = ens->h_out = nullptr;
        ens->reduce_cap = 0;
        CKE(cudaMalloc(&ens->d_reduce, sizeof(MemberReduce) * n));
        CKE(cudaMalloc(&ens->d_out, sizeof(double) * 2 * n));
        CKE(cudaMallocHost(&ens->h_out, sizeof(double) * 2 * n));
        ens->reduce_cap = n;
    }
    return TCYM_OK;
}

template <int FMT> static cudaError_t launch_group_step(tcym_ensemble ens, int f, int k, cudaStream_t s) {
    using T = typename Fmt<FMT>::T;
    const FmtGroup &G = ens->groups[f];
    const Member<T> *table = static_cast<const Member<T> *>(G.d_members);
    if constexpr (Fmt<FMT>::PAIRED) {
        if (!G.general) {
            for (const FmtGroup::Class &c : G.classes) {
                const cudaError_t e =
                    LaunchBatch<FMT>::step_uniform(table, c.m0, c.m1 - c.m0, c.item0, c.item1, k, c.coef, s);
                if (e != cudaSuccess) return e;
            }
            return cudaSuccess;
        }
    }
    return LaunchBatch<FMT>::step(table, (int)G.idx.size(), G.total_blocks, k, G.grid, G.general, s);
}

// Does format f step by persistent K-step launches?
static bool persistent_format(tcym_ensemble ens, int f) {
    const FmtGroup &G = ens->groups[f];
    return ens->persistent && (f == FMT_SU2_F32 || f == FMT_SU3_F32) && !G.general && !G.idx.empty();
}

// Schedules and control words of the persistent launches for chunks of nsteps
// (uploaded before the capture, which only refers to them).
static int prepare_persistent(tcym_ensemble ens, int nsteps) {
    for (int f = 0; f < 4; ++f) {
        if (!persistent_format(ens, f)) continue;
        FmtGroup &G = ens->groups[f];
        plan_groups(ens, G);
        G.h_sched.clear();
        for (FmtGroup::Class &c : G.classes) {
            c.sched_off = (int)G.h_sched.size();
            for (int b : c.group_first_block) G.h_sched.push_back(nsteps * b);
            for (int b : c.group_first_block) G.h_sched.push_back(b);
        }
        if (G.h_sched.size() > G.sched_cap) {
            cudaFree(G.d_sched);
            G.d_sched = nullptr;
            const size_t cap = std::max(G.h_sched.size(), 2 * G.sched_cap);
            G.sched_cap = 0;
            CKE(cudaMalloc(&G.d_sched, sizeof(int) * cap));
            G.sched_cap = cap;
        }
        CKE(cudaMemcpy(G.d_sched, G.h_sched.data(), sizeof(int) * G.h_sched.size(), cudaMemcpyHostToDevice));
        if (G.ctl_used > G.ctl_cap) {
            cudaFree(G.d_ctl);
            G.d_ctl = nullptr;
            const size_t cap = std::max(G.ctl_used, 2 * G.ctl_cap);
            G.ctl_cap = 0;
            CKE(cudaMalloc(&G.d_ctl, sizeof(int) * cap));
            G.ctl_cap = cap;
        }
    }
    return TCYM_OK;
}

// The K steps of format f as one persistent launch per coefficient class (captured).
template <int FMT> static cudaError_t launch_group_persistent(tcym_ensemble ens, int f, int nsteps, cudaStream_t s) {
    using T = typename Fmt<FMT>::T;
    const FmtGroup &G = ens->groups[f];
    const Member<T> *table = static_cast<const Member<T> *>(G.d_members);
    cudaError_t e = cudaMemsetAsync(G.d_ctl, 0, sizeof(int) * G.ctl_used, s);
    const int resident = ens->ctx->sm_count * LaunchBatch<FMT>::persistent_resident_blocks();
    for (const FmtGroup::Class &c : G.classes) {
        if (e != cudaSuccess) break;
        const int ng = (int)c.group_first_block.size() - 1;
        // each wait gives up after ~1 s at the GB300's 2 GHz clock
        const PersistentPlan plan{G.d_sched + c.sched_off, ng, nsteps, c.item0, c.item1, 2000000000LL};
        const int items = nsteps * (c.item1 - c.item0);
        e = LaunchBatch<FMT>::step_persistent(table, c.m0, c.m1 - c.m0, plan, c.coef, G.d_ctl + c.ctl_off,
                                              std::max(1, std::min(resident, items)), s);
    }
    return e;
}
static cudaError_t group_persistent(tcym_ensemble ens, int f, int nsteps, cudaStream_t s) {
    if (f == FMT_SU2_F32) return launch_group_persistent<FMT_SU2_F32>(ens, f, nsteps, s);
    return launch_group_persistent<FMT_SU3_F32>(ens, f, nsteps, s);
}

static cudaError_t group_step(tcym_ensemble ens, int f, int k, cudaStream_t s) {
    switch (f) {
        case FMT_SU2_F32: return launch_group_step<FMT_SU2_F32>(ens, f, k, s);
        case FMT_SU2_F64: return launch_group_step<FMT_SU2_F64>(ens, f, k, s);
        case FMT_SU3_F32: return launch_group_step<FMT_SU3_F32>(ens, f, k, s);
        default: return launch_group_step<FMT_SU3_F64>(ens, f, k, s);
    }
}

// Captures nsteps steps of every format chain into one graph.
static int capture(tcym_ensemble ens, int nsteps) {
    if (ens->exec) {
        cudaGraphExecDestroy(ens->exec);
        ens->exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    int r = prepare_persistent(ens, nsteps);
    if (r) return r;
    CKE(cudaStreamBeginCapture(ens->st[0], cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaEventRecord(ens->fork, ens->st[0]);
    for (int f = 0; f < 4 && err == cudaSuccess; ++f) {
        if (ens->groups[f].idx.empty()) continue;
        cudaStream_t s = ens->st[f];
        if (f != 0) err = cudaStreamWaitEvent(s, ens->fork, 0);
        if (persistent_format(ens, f)) {
            if (err == cudaSuccess) err = group_persistent(ens, f, nsteps, s);
        } else {
            for (int k = 0; k < nsteps && err == cudaSuccess; ++k) err = group_step(ens, f, k, s);
        }
        if (f != 0 && err == cudaSuccess) {
            err = cudaEventRecord(ens->join[f], s);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(ens->st[0], ens->join[f], 0);
        }
    }
    cudaError_t e2 = cudaStreamEndCapture(ens->st[0], &graph);
    if (err != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(ens->ctx, err, "ensemble capture");
    }
    if (e2 != cudaSuccess) return fail(ens->ctx, e2, "cudaStreamEndCapture");
    err = cudaGraphInstantiate(&ens->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (err != cudaSuccess) return fail(ens->ctx, err, "cudaGraphInstantiate");
    ens->graph_steps = nsteps;
    ens->layout_dirty = false;
    return TCYM_OK;
}

extern "C" int tcym_ensemble_create(tcym_ctx ctx, tcym_ensemble *out) {
    if (!ctx || !out) return TCYM_ERR_ARG;
    *out = nullptr;
    tcym_ensemble ens = new (std::nothrow) tcym_ensemble_s();
    if (!ens) return TCYM_ERR_OOM;
    ens->ctx = ctx;
    cudaSetDevice(ctx->device);
    // the ensemble's streams take the device's highest priority: work queued beside
    // them (a request being prepared in the request loop) fills the SMs they leave
    int lo = 0, hi = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i)
        e = cudaStreamCreateWithPriority(&ens->st[i], cudaStreamNonBlocking, hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ens->fork, cudaEventDisableTiming);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&ens->join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        int r = fail(ctx, e, "tcym_ensemble_create");
        tcym_ensemble_destroy(ens);
        return r;
    }
    *out = ens;
    return TCYM_OK;
}

extern "C" int tcym_ensemble_destroy(tcym_ensemble ens) {
    if (!ens) return TCYM_ERR_ARG;
    cudaSetDevice(ens->ctx->device);
    for (int i = 0; i < 4; ++i)
        if (ens->st[i]) cudaStreamSynchronize(ens->st[i]);
    if (ens->exec) cudaGraphExecDestroy(ens->exec);
    for (int f = 0; f < 4; ++f) {
        cudaFree(ens->groups[f].d_members);
        cudaFree(ens->groups[f].d_sched);
        cudaFree(ens->groups[f].d_ctl);
    }
    cudaFree(ens->partial);
    cudaFree(ens->d_reduce);
    cudaFree(ens->d_out);
    if (ens->h_out) cudaFreeHost(ens->h_out);
    for (int i = 0; i < 4; ++i) {
        if (ens->join[i]) cudaEventDestroy(ens->join[i]);
        if (ens->st[i]) cudaStreamDestroy(ens->st[i]);
    }
    if (ens->fork) cudaEventDestroy(ens->fork);
    delete ens;
    return TCYM_OK;
}

extern "C" int tcym_ensemble_add(tcym_ensemble ens, tcym_lattice lat, int dynamics, double dt, double gamma, double T,
                                 uint64_t seed, uint64_t step0) {
    if (!ens || !lat || lat->ctx != ens->ctx || (dynamics != TCYM_DYN_LEAPFROG && dynamics != TCYM_DYN_LANGEVIN) ||
        dt < 0 || gamma < 0 || T < 0)
        return TCYM_ERR_ARG;
    for (const EnsMember &m : ens->members)
        if (m.lat == lat) {
            tcym_set_error(ens->ctx, "tcym_ensemble_add: the lattice is already a member");
            return TCYM_ERR_STATE;
        }
    cudaSetDevice(ens->ctx->device);
    CKE(cudaStreamSynchronize(lat->stream));  // the ensemble orders its own work from here on
    ens->members.push_back(EnsMember{lat, dynamics == TCYM_DYN_LANGEVIN ? MODE_LANGEVIN : MODE_LEAPFROG, dt, gamma, T,
                                     seed, step0});
    ens->layout_dirty = true;
    return TCYM_OK;
}

extern "C" int tcym_ensemble_set_persistent(tcym_ensemble ens, int group_blocks) {
    if (!ens) return TCYM_ERR_ARG;
    ens->persistent = group_blocks >= 0;
    ens->group_blocks = group_blocks > 0 ? group_blocks : 0;
    ens->layout_dirty = true;
    return TCYM_OK;
}

extern "C" int tcym_ensemble_remove(tcym_ensemble ens, tcym_lattice lat) {
    if (!ens || !lat) return TCYM_ERR_ARG;
    auto it = std::find_if(ens->members.begin(), ens->members.end(), [&](const EnsMember &m) { return m.lat == lat; });
    if (it == ens->members.end()) return TCYM_ERR_ARG;
    ens->members.erase(it);
    ens->layout_dirty = true;
    return TCYM_OK;
}

extern "C" int tcym_ensemble_size(tcym_ensemble ens, int *n) {
    if (!ens || !n) return TCYM_ERR_ARG;
    *n = (int)ens->members.size();
    return TCYM_OK;
}

extern "C" int tcym_ensemble_step(tcym_ensemble ens, int nsteps) {
    TCYM_RANGE("tcym_ensemble_step");
    if (!ens || nsteps < 0) return TCYM_ERR_ARG;
    if (nsteps == 0 || ens->members.empty()) return TCYM_OK;
    cudaSetDevice(ens->ctx->device);
    int r = upload_tables(ens);
    if (r) return r;
    if (ens->layout_dirty || !ens->exec || ens->graph_steps != nsteps)
        if ((r = capture(ens, nsteps))) return r;
    CKE(cudaGraphLaunch(ens->exec, ens->st[0]));
    // a persistent launch that gave up waiting raised its error word
    for (int f = 0; f < 4; ++f) {
        if (!persistent_format(ens, f)) continue;
        FmtGroup &G = ens->groups[f];
        ens->h_ctl.resize(G.ctl_used);
        CKE(cudaMemcpyAsync(ens->h_ctl.data(), G.d_ctl, sizeof(int) * G.ctl_used, cudaMemcpyDeviceToHost,
                            ens->st[0]));
        CKE(cudaStreamSynchronize(ens->st[0]));
        for (const FmtGroup::Class &c : G.classes)
            if (ens->h_ctl[c.ctl_off + 1]) {
                tcym_set_error(ens->ctx, "tcym_ensemble_step: a persistent launch timed out waiting for a member's "
                                         "previous step");
                return TCYM_ERR_TIMEOUT;
            }
    }
    // bookkeeping of every member; periodic FP64 reunitarisation of FP32 links
    for (EnsMember &m : ens->members) {
        tcym_lattice L = m.lat;
        L->cur ^= (nsteps & 1);
        L->steps_done += nsteps;
        m.next_step += (uint64_t)nsteps;
        L->steps_since_reunit += nsteps;
        if (L->reunit_period > 0 && L->steps_since_reunit >= L->reunit_period) {
            int rr = 0;
            switch (L->fmt) {
                case FMT_SU2_F32: rr = Launch<FMT_SU2_F32>::reunitarize(L->g, L->U[L->cur], ens->st[0]); break;
                case FMT_SU2_F64: rr = Launch<FMT_SU2_F64>::reunitarize(L->g, L->U[L->cur], ens->st[0]); break;
                case FMT_SU3_F32: rr = Launch<FMT_SU3_F32>::reunitarize(L->g, L->U[L->cur], ens->st[0]); break;
                default: rr = Launch<FMT_SU3_F64>::reunitarize(L->g, L->U[L->cur], ens->st[0]); break;
            }
            if (rr != cudaSuccess) return fail(ens->ctx, (cudaError_t)rr, "ensemble reunitarize");
            L->steps_since_reunit = 0;
        }
    }
    CKE(cudaStreamSynchronize(ens->st[0]));
    return TCYM_OK;
}

template <int FMT> static cudaError_t launch_group_obs(tcym_ensemble ens, int f, int mask) {
    using T = typename Fmt<FMT>::T;
    const FmtGroup &G = ens->groups[f];
    if (G.idx.empty()) return cudaSuccess;
    return LaunchBatch<FMT>::observables(static_cast<const Member<T> *>(G.d_members), (int)G.idx.size(), G.red_total,
                                         mask, ens->partial + (size_t)G.red_offset * P_WIDTH, G.red_grid, ens->st[0]);
}

extern "C" int tcym_ensemble_measure(tcym_ensemble ens, int ncs_stride, double *edotb, double *ncs) {
    if (!ens || ncs_stride < 0) return TCYM_ERR_ARG;
    const size_t n = ens->members.size();
    if (n == 0) return TCYM_OK;
    cudaSetDevice(ens->ctx->device);
    int r = upload_tables(ens);
    if (r) return r;
    cudaError_t e = launch_group_obs<FMT_SU2_F32>(ens, FMT_SU2_F32, OBS_EDOTB);
    if (e == cudaSuccess) e = launch_group_obs<FMT_SU2_F64>(ens, FMT_SU2_F64, OBS_EDOTB);
    if (e == cudaSuccess) e = launch_group_obs<FMT_SU3_F32>(ens, FMT_SU3_F32, OBS_EDOTB);
    if (e == cudaSuccess) e = launch_group_obs<FMT_SU3_F64>(ens, FMT_SU3_F64, OBS_EDOTB);
    if (e != cudaSuccess) return fail(ens->ctx, e, "ensemble observables");
    // per-member finalisers, in ensemble order
    std::vector<MemberReduce> items(n);
    for (int f = 0; f < 4; ++f) {
        const FmtGroup &G = ens->groups[f];
        int red = 0;
        for (size_t i = 0; i < G.idx.size(); ++i) {
            const EnsMember &m = ens->members[G.idx[i]];
            const int rb = grid_for(m.lat->g.V, kRedThreads);
            items[G.idx[i]] = MemberReduce{ens->partial + (size_t)G.red_offset * P_WIDTH, red, rb,
                                           m.lat->nc == 2 ? 3 : 8, m.lat->g.V,
                                           ncs_stride > 0 ? m.dt * ncs_stride : 0.0, m.lat->result};
            red += rb;
        }
    }
    CKE(cudaMemcpyAsync(ens->d_reduce, items.data(), sizeof(MemberReduce) * n, cudaMemcpyHostToDevice, ens->st[0]));
    if ((e = finalize_members(ens->d_reduce, (int)n, ens->d_out, ens->st[0])) != cudaSuccess)
        return fail(ens->ctx, e, "ensemble finalize");
    CKE(cudaMemcpyAsync(ens->h_out, ens->d_out, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, ens->st[0]));
    CKE(cudaStreamSynchronize(ens->st[0]));
    for (size_t i = 0; i < n; ++i) {
        if (edotb) edotb[i] = ens->h_out[2 * i];
        if (ncs) ncs[i] = ens->h_out[2 * i + 1];
    }
    return TCYM_OK;
}
