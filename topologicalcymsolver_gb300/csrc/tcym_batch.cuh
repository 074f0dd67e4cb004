// Batched kernels: many independent lattices of one storage format advance in
// one launch.  The grid walks a flattened list of (member, block) work items;
// each work item is exactly the block the single-lattice kernel would run
// (site pairs for FP32 members with even nz, single sites otherwise), calling
// the same per-site function with the member's own geometry, buffers and
// coefficients, so a member's arithmetic does not depend on which other
// lattices share the launch.
#pragma once

#include "tcym_kernels.cuh"

namespace tcym {

// One ensemble member as the device sees it.
template <class T> struct Member {
    Geom g;
    void *U[2];
    void *E;
    double *result;      // the lattice's device result block (Kahan N_CS lives there)
    StepCoef<T> c;       // c.step is the member's noise counter at the start of the chunk
    int cur;             // link buffer holding the state at the start of the chunk
    int block_begin;     // first step work item of this member
    int red_begin;       // first reduction work item of this member
    int red_blocks;      // reduction work items of this member
    int paired;          // step work items cover site pairs (FP32 format, even nz)
    Tile tile;           // their block tiling
    double ncs_dt;       // Kahan increment factor for measurements (0: no N_CS update)
};

// 1: the batched kernels walk their work items with a grid of the resident
// blocks; 0: one block per work item
#ifndef TCYM_BATCH_PERSISTENT
#define TCYM_BATCH_PERSISTENT 0
#endif
// the batched step reading its coefficients from the member table holds more
// than the single-lattice step: SU(2) at 7 blocks per SM (72 registers) spills
// there, so it keeps its own target (the uniform-coefficient kernel takes the
// single-lattice one)
#ifndef TCYM_SU2_BATCH_MINBLOCKS
#define TCYM_SU2_BATCH_MINBLOCKS 6
#endif
// SU(3) likewise: at 4 blocks (128 registers) the table-reading step spills
#ifndef TCYM_SU3_BATCH_MINBLOCKS
#define TCYM_SU3_BATCH_MINBLOCKS 3
#endif
template <int FMT> constexpr int batch_min_blocks_for() {
    if constexpr (Fmt<FMT>::PAIRED && Fmt<FMT>::NA == 3) return TCYM_SU2_BATCH_MINBLOCKS;
    if constexpr (Fmt<FMT>::PAIRED && Fmt<FMT>::NA == 8) return TCYM_SU3_BATCH_MINBLOCKS;
    return Fmt<FMT>::PAIRED ? pair_min_blocks_for<FMT>() : min_blocks_for<FMT>();
}

// index of the member owning work item `item` (begins sorted ascending)
template <class T>
__device__ __forceinline__ int find_member(const Member<T> *m, int n, int item, bool reduction) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int b = reduction ? m[mid].red_begin : m[mid].block_begin;
        if (b <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Step k of a chunk for every member: reads U[cur ^ (k&1)], writes U[cur ^ (k&1) ^ 1].
// GENERAL = false is the lean kernel for the common case of a paired format whose
// members all take pairs with the linear mapping; true handles every member kind.
template <int FMT, bool GENERAL>
__global__ void __launch_bounds__(threads_for<FMT>(), batch_min_blocks_for<FMT>())
    k_step_batch(const Member<typename Fmt<FMT>::T> *__restrict__ members, int nmembers, int total_blocks, int k) {
    static_assert(!Fmt<FMT>::PAIRED || threads_for<FMT>() == kThreadsPair, "one block shape for both paths");
    using T = typename Fmt<FMT>::T;
    // each thread's plaquette slots (its own only: no thread reads another's); the
    // per-site path of an FP32 member uses the same array as floats
    using S = typename std::conditional<Fmt<FMT>::PAIRED, f2, T>::type;
    __shared__ S sm_pair[plaq_slots<FMT>() * threads_for<FMT>()];
    T *const sm_site = reinterpret_cast<T *>(sm_pair);
    for (int item = blockIdx.x; item < total_blocks; item += gridDim.x) {
        const int mi = find_member(members, nmembers, item, false);
        // the table is read-only and never aliases the fields (__restrict__), so
        // the coefficients are read where used, block-uniform, from L1, rather
        // than held in registers for the whole step
        const Member<typename Fmt<FMT>::T> &m = members[mi];
        const Geom g = m.g;
        if constexpr (Fmt<FMT>::PAIRED && !GENERAL) {
            const int64_t p0 = (int64_t)(item - m.block_begin) * kThreadsPair, p = p0 + threadIdx.x;
            if (p < (g.V >> 1)) {
                const int in = m.cur ^ (k & 1);
                if (pairs_touch_seam(g, p0, kThreadsPair))
                    site_step_pair<Fmt<FMT>, true>(g, m.U[in], m.U[in ^ 1], m.E, m.c, p, (uint64_t)k,
                                                   sm_pair + threadIdx.x, kThreadsPair);
                else
                    site_step_pair<Fmt<FMT>, false>(g, m.U[in], m.U[in ^ 1], m.E, m.c, p, (uint64_t)k,
                                                    sm_pair + threadIdx.x, kThreadsPair);
            }
            continue;
        }
        if constexpr (Fmt<FMT>::PAIRED) {
            if (m.paired) {  // block-uniform
                int64_t p;
                bool seam;
                if (tile_pair(g, m.tile, item - m.block_begin, threadIdx.x, p, seam)) {
                    const int in = m.cur ^ (k & 1);
                    if (seam)
                        site_step_pair<Fmt<FMT>, true>(g, m.U[in], m.U[in ^ 1], m.E, m.c, p, (uint64_t)k,
                                                       sm_pair + threadIdx.x, kThreadsPair);
                    else
                        site_step_pair<Fmt<FMT>, false>(g, m.U[in], m.U[in ^ 1], m.E, m.c, p, (uint64_t)k,
                                                        sm_pair + threadIdx.x, kThreadsPair);
                }
                continue;
            }
        }
        const int64_t s = (int64_t)(item - m.block_begin) * blockDim.x + threadIdx.x;
        if (s < g.V) {
            const int in = m.cur ^ (k & 1);
            site_step<Fmt<FMT>, true, true>(g, m.U[in], m.U[in ^ 1], m.E, m.c, s, (uint64_t)k,
                                            sm_site + threadIdx.x, (int)blockDim.x);
        }
    }
}

// The lean path when every member takes the same step coefficients (the same
// mode, dt and spacings): they come from the kernel's parameters, as in the
// single-lattice step, instead of from the member table in memory at each use
// (the single-lattice kernel was 11% (SU(3)) and 29% (SU(2)) faster than the
// table-reading one on the same 128^3 lattice).  Langevin noise coefficients
// (seed, step, damping and kick, per member) still come from the table.
// The members are a slice of a format's table (one coefficient class), whose
// work items run from item0 to total_blocks.
template <int FMT>
__global__ void __launch_bounds__(kThreadsPair, pair_min_blocks_for<FMT>())
    k_step_batch_uniform(const Member<float> *__restrict__ members, int nmembers, int item0, int total_blocks, int k,
                         StepCoef<float> c) {
    static_assert(Fmt<FMT>::PAIRED, "paired formats only");
    __shared__ f2 sm[plaq_slots<FMT>() * kThreadsPair];
#if TCYM_BATCH_PERSISTENT
    for (int item = item0 + blockIdx.x; item < total_blocks; item += gridDim.x) {
#else
    {  // one work item per block
        const int item = item0 + blockIdx.x;
        if (item >= total_blocks) return;
#endif
        const int mi = find_member(members, nmembers, item, false);
        const Member<float> &m = members[mi];
        const Geom g = m.g;
        const int64_t p0 = (int64_t)(item - m.block_begin) * kThreadsPair, p = p0 + threadIdx.x;
        if (p < (g.V >> 1)) {
            const int in = m.cur ^ (k & 1);
            if (pairs_touch_seam(g, p0, kThreadsPair))
                site_step_pair<Fmt<FMT>, true>(g, m.U[in], m.U[in ^ 1], m.E, c, m.c, p, (uint64_t)k,
                                               sm + threadIdx.x, kThreadsPair);
            else
                site_step_pair<Fmt<FMT>, false>(g, m.U[in], m.U[in ^ 1], m.E, c, m.c, p, (uint64_t)k,
                                                sm + threadIdx.x, kThreadsPair);
        }
    }
}

// ---------------------------------------------------------------- persistent
// K steps of one coefficient class in a single launch.  The class's work items
// (one block of 128 site pairs of one member at one step) are handed out by an
// atomic counter in a fixed order: the members are cut into groups, and a group
// runs all K steps before the next group starts, step by step within the group.
// A group small enough keeps its links and fields in the 129 MB L2 across its
// steps, where one launch per step streams every member through DRAM each step.
//
// The item of step k of member m waits until all of m's step k-1 items are done
// (a per-member counter, raised by each finished item with release semantics;
// the waiter reads it, fences and releases its block with a barrier, the
// pattern of a grid-wide barrier).  The wait cannot deadlock and needs no
// co-resident grid: items are taken in increasing order and only ever wait for
// items taken earlier, so the oldest unfinished item can always run.  Each wait
// gives up after `spin_limit` clock cycles: it raises the error flag, every
// block then stops taking items, and the host reports a timeout.
//
// ctl: [0] next item, [1] error flag, [2 + i] items done of member i.  A member's
// arithmetic is that of the other step kernels.
struct PersistentPlan {
    const int *sched;  // [0, ngroups]: first item of group g; [ngroups + 1, 2 ngroups + 1]: its first block
    int ngroups;
    int K;
    int item0, item1;  // the class's blocks in the format's block numbering
    long long spin_limit;
};

__device__ __forceinline__ int find_group(const int *first_item, int ngroups, int item) {
    int lo = 0, hi = ngroups - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first_item[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <int FMT>
__global__ void __launch_bounds__(kThreadsPair, batch_min_blocks_for<FMT>())
    k_step_persistent(const Member<float> *__restrict__ members, int nmembers, PersistentPlan plan,
                      StepCoef<float> c, int *ctl) {
    static_assert(Fmt<FMT>::PAIRED, "paired formats only");
    __shared__ f2 sm[plaq_slots<FMT>() * kThreadsPair];
    __shared__ int s_item, s_stop;
    const int *first_item = plan.sched, *first_block = plan.sched + plan.ngroups + 1;
    const int total = first_item[plan.ngroups];
    for (;;) {
        if (threadIdx.x == 0) {
            const int it = atomicAdd(&ctl[0], 1);
            s_item = *(volatile int *)&ctl[1] ? total : it;
        }
        __syncthreads();
        const int item = s_item;
        if (item >= total) return;
        const int g = find_group(first_item, plan.ngroups, item);
        const int nbg = first_block[g + 1] - first_block[g];
        const int rel = item - first_item[g];
        const int k = rel / nbg;
        const int blk = plan.item0 + first_block[g] + (rel - k * nbg);
        const int mi = find_member(members, nmembers, blk, false);
        const Member<float> &m = members[mi];
        if (k > 0) {
            if (threadIdx.x == 0) {
                const int nblk = (mi + 1 < nmembers ? members[mi + 1].block_begin : plan.item1) - m.block_begin;
                const int need = k * nblk;
                const long long t0 = clock64();
                int stop = 0;
                while (*(volatile int *)&ctl[2 + mi] < need) {
                    if (*(volatile int *)&ctl[1] || clock64() - t0 > plan.spin_limit) {
                        atomicExch(&ctl[1], 1);
                        stop = 1;
                        break;
                    }
                }
                __threadfence();
                s_stop = stop;
            }
            __syncthreads();
            if (s_stop) return;
        }
        const Geom g0 = m.g;
        const int64_t p0 = (int64_t)(blk - m.block_begin) * kThreadsPair, p = p0 + threadIdx.x;
        if (p < (g0.V >> 1)) {
            const int in = m.cur ^ (k & 1);
            if (pairs_touch_seam(g0, p0, kThreadsPair))
                site_step_pair<Fmt<FMT>, true>(g0, m.U[in], m.U[in ^ 1], m.E, c, m.c, p, (uint64_t)k,
                                               sm + threadIdx.x, kThreadsPair);
            else
                site_step_pair<Fmt<FMT>, false>(g0, m.U[in], m.U[in ^ 1], m.E, c, m.c, p, (uint64_t)k,
                                                sm + threadIdx.x, kThreadsPair);
        }
        __syncthreads();  // every thread's stores are issued (and s_item may be reused)
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&ctl[2 + mi], 1);
        }
    }
}

// Observables of every member: one partial record per reduction work item.
// The N_CS sample (mask OBS_EDOTB) of every member: members in FP32 pair storage
// (even nz) one thread per site pair, the others per site as k_observables_batch.
// A member keeps its grid_for(V, kRedThreads) records (the finaliser's layout);
// paired, its first grid_for(V/2, kRedThreads) hold the pairs and the rest zeros.
template <int FMT>
__global__ void __launch_bounds__(kRedThreads)
    k_edotb_obs_batch(const Member<typename Fmt<FMT>::T> *members, int nmembers, int total_blocks, double *partial) {
    using F = Fmt<FMT>;
    for (int item = blockIdx.x; item < total_blocks; item += gridDim.x) {
        const int mi = find_member(members, nmembers, item, true);
        const Geom g = members[mi].g;
        const void *u = members[mi].U[members[mi].cur], *e = members[mi].E;
        double v[P_WIDTH];
#pragma unroll
        for (int q = 0; q < P_WIDTH; ++q) v[q] = 0.0;
        const int64_t i = (int64_t)(item - members[mi].red_begin) * blockDim.x + threadIdx.x;
        if constexpr (F::PAIRED) {
            if (members[mi].paired) {
                const int64_t Vh = g.V >> 1, plane = (int64_t)g.nx * g.ny;
                if (i < Vh) {
                    const bool seam = i < plane || i >= Vh - plane;
#pragma unroll 1
                    for (int mu = 0; mu < 3; ++mu) {
                        f2 esq, bsq;
                        const f2 edb = seam ? pair_edotb_obs<F, true>(g, u, e, i, mu, esq, bsq)
                                            : pair_edotb_obs<F, false>(g, u, e, i, mu, esq, bsq);
                        const double es = (double)esq.v.x + (double)esq.v.y, bs = (double)bsq.v.x + (double)bsq.v.y;
                        if (mu == 0) { v[P_ESQ0] += es; v[P_BSQ0] += bs; }
                        else if (mu == 1) { v[P_ESQ0 + 1] += es; v[P_BSQ0 + 1] += bs; }
                        else { v[P_ESQ0 + 2] += es; v[P_BSQ0 + 2] += bs; }
                        v[P_EDB] += (double)edb.v.x + (double)edb.v.y;
                    }
                }
            }
        }
        if (!(F::PAIRED && members[mi].paired) && i < g.V) {
            SiteObs<F> o;
            site_observables<F>(g, u, e, OBS_EDOTB, i, o);
            for (int q = 0; q < 3; ++q) { v[P_ESQ0 + q] = o.esq[q]; v[P_BSQ0 + q] = o.bsq[q]; }
            v[P_EDB] = o.edotb;
        }
        __shared__ double sh[32][P_WIDTH];
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int q = 0; q < P_WIDTH; ++q) v[q] = q < P_GMAX ? warp_sum(v[q]) : warp_max(v[q]);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < P_WIDTH; ++q) sh[w][q] = v[q];
        __syncthreads();
        if (threadIdx.x < P_WIDTH) {
            const int q = threadIdx.x;
            double r = sh[0][q];
            for (int k = 1; k < nw; ++k) r = q < P_GMAX ? r + sh[k][q] : fmax(r, sh[k][q]);
            partial[(int64_t)item * P_WIDTH + q] = r;
        }
        __syncthreads();
    }
}

template <int FMT>
__global__ void __launch_bounds__(kRedThreads)
    k_observables_batch(const Member<typename Fmt<FMT>::T> *members, int nmembers, int total_blocks, int mask,
                        double *partial) {
    using F = Fmt<FMT>;
    using T = typename F::T;
    for (int item = blockIdx.x; item < total_blocks; item += gridDim.x) {
        const int mi = find_member(members, nmembers, item, true);
        const Geom g = members[mi].g;
        const void *u = members[mi].U[members[mi].cur], *e = members[mi].E;
        double v[P_WIDTH];
#pragma unroll
        for (int q = 0; q < P_WIDTH; ++q) v[q] = 0.0;
        const int64_t s = (int64_t)(item - members[mi].red_begin) * blockDim.x + threadIdx.x;
        if (s < g.V) {
            SiteObs<F> o;
            site_observables<F>(g, u, e, mask, s, o);
            for (int q = 0; q < 3; ++q) { v[P_ESQ0 + q] = o.esq[q]; v[P_BSQ0 + q] = o.bsq[q]; }
            for (int a = 0; a < F::NA; ++a) {
                v[P_GSQ] += o.g[a] * o.g[a];
                v[P_GMAX] = fmax(v[P_GMAX], o.g[a]);
                v[P_GABS] = fmax(v[P_GABS], fabs(o.g[a]));
            }
            for (int q = 0; q < 3; ++q) { v[P_USQ] += o.un[q] * o.un[q]; v[P_UMAX] = fmax(v[P_UMAX], o.un[q]); }
            v[P_EDB] = o.edotb;
        }
        // block_partial writes at blockIdx.x: give it the work item's slot instead
        __shared__ double sh[32][P_WIDTH];
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int q = 0; q < P_WIDTH; ++q) v[q] = q < P_GMAX ? warp_sum(v[q]) : warp_max(v[q]);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < P_WIDTH; ++q) sh[w][q] = v[q];
        __syncthreads();
        if (threadIdx.x < P_WIDTH) {
            const int q = threadIdx.x;
            double r = sh[0][q];
            for (int i = 1; i < nw; ++i) r = q < P_GMAX ? r + sh[i][q] : fmax(r, sh[i][q]);
            partial[(int64_t)item * P_WIDTH + q] = r;
        }
        __syncthreads();
    }
}

// Launchers for one format.
template <int FMT> struct LaunchBatch {
    using T = typename Fmt<FMT>::T;
    static constexpr int TPB = threads_for<FMT>();
    static int resident_blocks() {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_step_batch<FMT, true>, TPB, 0);
        return b > 0 ? b : 1;
    }
    // general: some member is unpaired or tiled (see k_step_batch)
    static cudaError_t step(const Member<T> *members, int n, int total_blocks, int k, int grid, bool general,
                            cudaStream_t st) {
        if (general || !Fmt<FMT>::PAIRED) k_step_batch<FMT, true><<<grid, TPB, 0, st>>>(members, n, total_blocks, k);
        else k_step_batch<FMT, false><<<grid, TPB, 0, st>>>(members, n, total_blocks, k);
        return cudaGetLastError();
    }
    // the members [m0, m0 + n) of one coefficient class, work items [item0, item1),
    // stepped with their shared coefficients cu (k_step_batch_uniform)
    static cudaError_t step_uniform(const Member<T> *members, int m0, int n, int item0, int item1, int k,
                                    const StepCoef<double> &cu, cudaStream_t st) {
        if constexpr (Fmt<FMT>::PAIRED) {
            k_step_batch_uniform<FMT><<<item1 - item0, TPB, 0, st>>>(members + m0, n, item0, item1, k,
                                                                    coef_cast<float>(cu));
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;
    }
    // the persistent K-step launch of one coefficient class (k_step_persistent)
    static int persistent_resident_blocks() {
        int b = 0;
        if constexpr (Fmt<FMT>::PAIRED)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_step_persistent<FMT>, kThreadsPair, 0);
        return b > 0 ? b : 1;
    }
    static cudaError_t step_persistent(const Member<T> *members, int m0, int n, const PersistentPlan &plan,
                                       const StepCoef<double> &cu, int *ctl, int grid, cudaStream_t st) {
        if constexpr (Fmt<FMT>::PAIRED) {
            k_step_persistent<FMT><<<grid, kThreadsPair, 0, st>>>(members + m0, n, plan, coef_cast<float>(cu), ctl);
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;
    }
    static cudaError_t observables(const Member<T> *members, int n, int total_blocks, int mask, double *partial,
                                   int grid, cudaStream_t st) {
        if constexpr (Fmt<FMT>::PAIRED) {
            if (mask == OBS_EDOTB) {  // the N_CS sample: paired members in packed FP32
                k_edotb_obs_batch<FMT><<<grid, kRedThreads, 0, st>>>(members, n, total_blocks, partial);
                return cudaGetLastError();
            }
        }
        k_observables_batch<FMT><<<grid, kRedThreads, 0, st>>>(members, n, total_blocks, mask, partial);
        return cudaGetLastError();
    }
};

// Per-member fixed-order sum of its reduction records into its result block
// (one block per member); advances its Kahan N_CS by ncs_dt * E.B / (8 pi^2).
struct MemberReduce {
    const double *partial;
    int red_begin, red_blocks, na;
    int64_t V;
    double ncs_dt;
    double *result;
};
cudaError_t finalize_members(const MemberReduce *items, int n, double *out, cudaStream_t st);

}  // namespace tcym

// The kernels are instantiated once, in the tcym_kern_su{2,3}_f{32,64}*.cu units
// (which define TCYM_KERNEL_TU); every other unit only refers to them.
#ifndef TCYM_KERNEL_TU
namespace tcym {
extern template struct Launch<FMT_SU2_F32>;
extern template struct Launch<FMT_SU2_F64>;
extern template struct Launch<FMT_SU3_F32>;
extern template struct Launch<FMT_SU3_F64>;
extern template struct LaunchBatch<FMT_SU2_F32>;
extern template struct LaunchBatch<FMT_SU2_F64>;
extern template struct LaunchBatch<FMT_SU3_F32>;
extern template struct LaunchBatch<FMT_SU3_F64>;
}  // namespace tcym
#endif
