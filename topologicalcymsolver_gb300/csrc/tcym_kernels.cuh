// CUDA kernels and their launchers, one instantiation per storage format
// (tcym_kern_su{2,3}_f{32,64}*.cu).
//
// Every kernel is one thread per site (or per link for the checkerboard
// flow), grid-strided over the lattice.  Reductions are deterministic: each
// block writes one partial record (FP64) and a single-block finaliser sums the
// partials in block order, so a result never depends on scheduling.
#pragma once

#include <cuda_runtime.h>

#include "tcym_site.cuh"

namespace tcym {

// partial record of one block: 9 sums and 3 maxima
enum : int {
    P_ESQ0 = 0, P_BSQ0 = 3, P_GSQ = 6, P_USQ = 7, P_EDB = 8, P_GMAX = 9, P_GABS = 10, P_UMAX = 11, P_WIDTH = 12
};
// device result block (doubles), written by finalize_obs
enum : int {
    R_ESQ0 = 0, R_BSQ0 = 3, R_GMAX = 6, R_GRMS = 7, R_GABS = 8, R_UMAX = 9, R_URMS = 10, R_EDB = 11,
    R_NCS = 12, R_NCS_COMP = 13, R_NONFINITE = 14, R_WIDTH = 16
};

#ifndef TCYM_SU2_THREADS
#define TCYM_SU2_THREADS 128
#endif
constexpr int kThreadsSU2 = TCYM_SU2_THREADS;
constexpr int kThreadsSU3 = 128;
constexpr int kRedThreads = 256;
// Resident blocks per SM requested for the step kernels (register cap = 65536 / (blocks * threads)).
#ifndef TCYM_SU3_STEP_MINBLOCKS
#define TCYM_SU3_STEP_MINBLOCKS 4
#endif
#ifndef TCYM_SU2_STEP_MINBLOCKS
#define TCYM_SU2_STEP_MINBLOCKS 8
#endif
template <int FMT> constexpr int min_blocks_for() {
    return Fmt<FMT>::NA == 8 ? TCYM_SU3_STEP_MINBLOCKS : (FMT == FMT_SU2_F32 ? TCYM_SU2_STEP_MINBLOCKS : 1);
}

template <int FMT> constexpr int threads_for() { return Fmt<FMT>::NA == 3 ? kThreadsSU2 : kThreadsSU3; }

// The paired step (FP32 formats, even nz): one thread per site pair, 128 per
// block; resident blocks per SM requested (register cap 65536 / (blocks * 128)).
constexpr int kThreadsPair = 128;
// 1: blocks away from the seam run a copy of the step without the lane-swap
// tests; 0: one copy, the swaps decided per load
#ifndef TCYM_PAIR_SEAM_SPLIT
#define TCYM_PAIR_SEAM_SPLIT 1
#endif
// SU(3): 4 blocks (128 registers, no spills) measured 0.331 ms per 128^3 step
// against 0.342 ms at 3 (166 registers)
#ifndef TCYM_SU3_PAIR_MINBLOCKS
#define TCYM_SU3_PAIR_MINBLOCKS 4
#endif
// SU(2): 7 blocks (72 registers, a 4-byte spill) measured 0.090 ms per 128^3
// step against 0.094 ms at 6 (80 registers) and 0.107 ms at 5 (96, no spill)
#ifndef TCYM_SU2_PAIR_MINBLOCKS
#define TCYM_SU2_PAIR_MINBLOCKS 7
#endif
template <int FMT> constexpr int pair_min_blocks_for() {
    return Fmt<FMT>::NA == 8 ? TCYM_SU3_PAIR_MINBLOCKS : TCYM_SU2_PAIR_MINBLOCKS;
}
// L2 prefetch at the start of a block of the linear paired step: bit 0 the
// block's own field lines, bit 1 the lines of U_0, U_1 one pair-plane up in z
#ifndef TCYM_PAIR_PREFETCH
#define TCYM_PAIR_PREFETCH 0
#endif

// The lines a block of the linear paired step (pairs [p0, p0 + kThreadsPair))
// reads first from DRAM: its own fields, loaded only when each direction's
// update needs them, and the links U_0, U_1 of the pairs one step up in z,
// which its plaquettes read before the block owning them runs.  Each thread
// issues a few L2 prefetches (hints: no registers held, nothing waits on them),
// all inside the field and link arrays.  Planes: SU(3) FP32 links 6 x 16 B per
// pair and direction, fields 4 x 16 B; SU(2) FP32 links 2 x 16 B, fields 3 x 8 B.
template <int FMT>
__device__ __forceinline__ void prefetch_pair_block(const Geom &g, const void *Uin, const void *E, int64_t p0, int what) {
    constexpr bool su3 = Fmt<FMT>::NA == 8;
    constexpr int LP = su3 ? 6 : 2, LB = 16;   // link planes per direction, bytes per pair
    constexpr int EP = su3 ? 4 : 3, EB = su3 ? 16 : 8;
    constexpr int e_lines = 3 * EP * (kThreadsPair * EB / 128);
    constexpr int z_lines = 2 * LP * (kThreadsPair * LB / 128);
    const int64_t Vh = g.V >> 1;
    const int64_t sz = (int64_t)g.nx * g.ny;
    int64_t pz = p0 + sz;  // one pair-plane up; from the last plane, the seam's partner plane 0
    if (pz >= Vh) pz -= Vh;
    for (int i = threadIdx.x; i < e_lines + z_lines; i += kThreadsPair) {
        const char *addr = nullptr;
        if (i < e_lines) {
            if (!(what & 1)) continue;
            constexpr int per = kThreadsPair * EB / 128;
            const int plane = i / per;
            const int64_t q = p0 + (int64_t)(i % per) * (128 / EB);
            if (q < Vh) addr = static_cast<const char *>(E) + ((int64_t)plane * Vh + q) * EB;
        } else {
            if (!(what & 2)) continue;
            constexpr int per = kThreadsPair * LB / 128;
            const int j = i - e_lines;
            const int plane = j / per;  // direction plane / LP, component plane % LP
            const int64_t q = pz + (int64_t)(j % per) * (128 / LB);
            if (q < Vh) addr = static_cast<const char *>(Uin) + ((int64_t)plane * Vh + q) * LB;
        }
        if (addr) asm volatile("prefetch.global.L2 [%0];" ::"l"(addr));
    }
}

inline int grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (int)(b < 1 ? 1 : b);
}

template <class T> StepCoef<T> coef_cast(const StepCoef<double> &c) {
    StepCoef<T> r;
    r.mode = c.mode;
    r.seed = c.seed;
    r.step = c.step;
    for (int i = 0; i < 3; ++i) {
        r.fc[i] = (T)c.fc[i]; r.cnu[i] = (T)c.cnu[i]; r.uc[i] = (T)c.uc[i];
        r.damp[i] = (T)c.damp[i]; r.kick[i] = (T)c.kick[i];
    }
    return r;
}

// ------------------------------------------------------------------ kernels
// sites [s0, s1)
// shared-memory slots of the plaquette projections (site_step, site_step_pair)
template <int FMT> constexpr int plaq_slots() { return 3 * Fmt<FMT>::NA; }

template <int FMT, bool DO_E, bool DO_U>
__global__ void __launch_bounds__(threads_for<FMT>(), min_blocks_for<FMT>()) k_step(Geom g, const void *Uin, void *Uout, void *E,
                                                             StepCoef<typename Fmt<FMT>::T> c, int64_t s0, int64_t s1) {
    using T = typename Fmt<FMT>::T;
    __shared__ T sm[DO_E ? plaq_slots<FMT>() * threads_for<FMT>() : 1];
    const int64_t s = s0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= s1) return;
    site_step<Fmt<FMT>, DO_E, DO_U>(g, Uin, Uout, E, c, s, 0, sm + threadIdx.x, threads_for<FMT>());
}

// one thread per site pair (FP32 formats, even nz); blocks touching the seam
// take the lane-swapping loads
// TILED = false: the linear mapping, compiled apart so its index arithmetic
// stays as light as the kernel's register budget wants
template <int FMT, bool TILED>
__global__ void __launch_bounds__(kThreadsPair, pair_min_blocks_for<FMT>())
    k_step_pair(Geom g, const void *Uin, void *Uout, void *E, StepCoef<float> c, Tile t) {
    __shared__ f2 sm[plaq_slots<FMT>() * kThreadsPair];
    int64_t p;
    bool seam;
    if constexpr (TILED) {
        if (!tile_pair(g, t, blockIdx.x, threadIdx.x, p, seam)) return;
    } else {
        const int64_t p0 = ((int64_t)blockIdx.x + t.b0) * kThreadsPair;
        if (TCYM_PAIR_PREFETCH) prefetch_pair_block<FMT>(g, Uin, E, p0, TCYM_PAIR_PREFETCH);
        p = p0 + threadIdx.x;
        if (p >= (g.V >> 1)) return;
        seam = pairs_touch_seam(g, p0, kThreadsPair);
    }
#if TCYM_PAIR_SEAM_SPLIT
    if (seam) site_step_pair<Fmt<FMT>, true>(g, Uin, Uout, E, c, p, 0, sm + threadIdx.x, kThreadsPair);
    else site_step_pair<Fmt<FMT>, false>(g, Uin, Uout, E, c, p, 0, sm + threadIdx.x, kThreadsPair);
#else
    site_step_pair<Fmt<FMT>, true>(g, Uin, Uout, E, c, p, 0, sm + threadIdx.x, kThreadsPair);
#endif
}

// sites of parity p, for even extents: t -> (x, row) with x of the right parity
template <int FMT>
__global__ void __launch_bounds__(threads_for<FMT>(), min_blocks_for<FMT>()) k_flow_cb(Geom g, void *U, int parity, int mu,
                                                                typename Fmt<FMT>::T fc0, typename Fmt<FMT>::T fc1,
                                                                typename Fmt<FMT>::T fc2, typename Fmt<FMT>::T cn0,
                                                                typename Fmt<FMT>::T cn1, typename Fmt<FMT>::T cn2,
                                                                typename Fmt<FMT>::T uc0, typename Fmt<FMT>::T uc1,
                                                                typename Fmt<FMT>::T uc2) {
    using T = typename Fmt<FMT>::T;
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.V / 2) return;
    const int hx = g.nx / 2;
    int64_t row = t / hx;
    int xh = (int)(t - row * hx);
    int y = (int)(row % g.ny), z = (int)(row / g.ny);
    int x = 2 * xh + ((y + z + parity) & 1);
    int64_t s = x + (int64_t)g.nx * row;
    const T fc[3] = {fc0, fc1, fc2}, cn[3] = {cn0, cn1, cn2}, uc[3] = {uc0, uc1, uc2};
    link_flow<Fmt<FMT>>(g, U, mu, fc, cn, uc, s);
}

// block reduction helpers (FP64)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Reduce vals[0..P_WIDTH) over the block into partial[blockIdx.x * P_WIDTH ..].
__device__ __forceinline__ void block_partial(double *vals, double *partial) {
    __shared__ double sh[32][P_WIDTH];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < P_WIDTH; ++k) vals[k] = k < P_GMAX ? warp_sum(vals[k]) : warp_max(vals[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < P_WIDTH; ++k) sh[w][k] = vals[k];
    __syncthreads();
    if (threadIdx.x < P_WIDTH) {
        const int k = threadIdx.x;
        double r = sh[0][k];
        for (int i = 1; i < nw; ++i) r = k < P_GMAX ? r + sh[i][k] : fmax(r, sh[i][k]);
        partial[(int64_t)blockIdx.x * P_WIDTH + k] = r;
    }
}

template <int FMT>
__global__ void __launch_bounds__(kRedThreads) k_observables(Geom g, const void *U, const void *E, int mask,
                                                             double *partial) {
    using F = Fmt<FMT>;
    double v[P_WIDTH];
#pragma unroll
    for (int k = 0; k < P_WIDTH; ++k) v[k] = 0.0;
    v[P_GMAX] = 0.0;  // signed maximum starts at 0 (GaussLawViolation.cpp:17,44)
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.V; s += (int64_t)gridDim.x * blockDim.x) {
        SiteObs<F> o;
        site_observables<F>(g, U, E, mask, s, o);
        for (int m = 0; m < 3; ++m) { v[P_ESQ0 + m] += o.esq[m]; v[P_BSQ0 + m] += o.bsq[m]; }
        for (int a = 0; a < F::NA; ++a) {
            v[P_GSQ] += o.g[a] * o.g[a];
            v[P_GMAX] = fmax(v[P_GMAX], o.g[a]);
            v[P_GABS] = fmax(v[P_GABS], fabs(o.g[a]));
        }
        for (int m = 0; m < 3; ++m) { v[P_USQ] += o.un[m] * o.un[m]; v[P_UMAX] = fmax(v[P_UMAX], o.un[m]); }
        v[P_EDB] += o.edotb;
    }
    block_partial(v, partial);
}

// The N_CS sample (mask OBS_EDOTB) of FP32 pair storage with even nz: one thread
// per site pair, the same block partials as k_observables with that mask (the
// Gauss and unitarity slots stay 0).
template <int FMT>
__global__ void __launch_bounds__(kRedThreads) k_edotb_obs_pair(Geom g, const void *U, const void *E,
                                                                double *partial) {
    using F = Fmt<FMT>;
    double v[P_WIDTH];
#pragma unroll
    for (int k = 0; k < P_WIDTH; ++k) v[k] = 0.0;
    const int64_t Vh = g.V >> 1, plane = (int64_t)g.nx * g.ny;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < Vh; p += (int64_t)gridDim.x * blockDim.x) {
        const bool seam = p < plane || p >= Vh - plane;
#pragma unroll 1
        for (int mu = 0; mu < 3; ++mu) {
            f2 esq, bsq;
            const f2 edb = seam ? pair_edotb_obs<F, true>(g, U, E, p, mu, esq, bsq)
                                : pair_edotb_obs<F, false>(g, U, E, p, mu, esq, bsq);
            const double es = (double)esq.v.x + (double)esq.v.y, bs = (double)bsq.v.x + (double)bsq.v.y;
            // fixed slots (a run-time index would put v in local memory)
            if (mu == 0) { v[P_ESQ0] += es; v[P_BSQ0] += bs; }
            else if (mu == 1) { v[P_ESQ0 + 1] += es; v[P_BSQ0 + 1] += bs; }
            else { v[P_ESQ0 + 2] += es; v[P_BSQ0 + 2] += bs; }
            v[P_EDB] += (double)edb.v.x + (double)edb.v.y;
        }
    }
    block_partial(v, partial);
}

// Gauss violation into the FP64 scratch G[a*V + s]; partial maxima as for observables.
template <int FMT>
__device__ __forceinline__ void gauss_compute_block(const Geom &g, const void *U, const void *E, double *G,
                                                    double *partial) {
    using F = Fmt<FMT>;
    double v[P_WIDTH];
#pragma unroll
    for (int k = 0; k < P_WIDTH; ++k) v[k] = 0.0;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.V; s += (int64_t)gridDim.x * blockDim.x) {
        double gv[F::NA];
        site_gauss<F>(g, U, E, s, gv);
        for (int a = 0; a < F::NA; ++a) {
            G[a * g.V + s] = gv[a];
            v[P_GSQ] += gv[a] * gv[a];
            v[P_GMAX] = fmax(v[P_GMAX], gv[a]);
            v[P_GABS] = fmax(v[P_GABS], fabs(gv[a]));
        }
    }
    block_partial(v, partial);
}
template <int FMT>
__global__ void __launch_bounds__(kRedThreads) k_gauss_compute(Geom g, const void *U, const void *E, double *G,
                                                               double *partial) {
    gauss_compute_block<FMT>(g, U, E, G, partial);
}

template <int FMT>
__global__ void __launch_bounds__(threads_for<FMT>()) k_gauss_update(Geom g, const void *U, void *E, const double *G,
                                                                     double gam) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.V) return;
    site_gauss_update<Fmt<FMT>>(g, U, E, G, gam, s);
}

// The same two kernels for iteration `it` of a restore whose control block
// holds, in ctl[0], the first iteration that is not to run (the finaliser of the
// deciding reduction lowers it): a kernel of a later iteration returns at once,
// so the host can queue many iterations between its checks.
template <int FMT>
__global__ void __launch_bounds__(kRedThreads) k_gauss_compute_it(Geom g, const void *U, const void *E, double *G,
                                                                  double *partial, const double *ctl, int it) {
    if ((double)it >= ctl[0]) return;  // the same value for every thread of the grid
    gauss_compute_block<FMT>(g, U, E, G, partial);
}
template <int FMT>
__global__ void __launch_bounds__(threads_for<FMT>()) k_gauss_update_it(Geom g, const void *U, void *E, const double *G,
                                                                        double gam, const double *ctl, int it) {
    if ((double)it >= ctl[0]) return;
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.V) return;
    site_gauss_update<Fmt<FMT>>(g, U, E, G, gam, s);
}

// The restore iteration for the FP32 formats with even nz: one thread per site
// pair in packed FP32, G(x) kept as FP32 pair planes G2[a * Vh + p] (the
// storage's precision; the scratch holds na * V doubles, twice what they need).
// The per-site sums run in FP32 per thread and the block partials in FP64,
// with the same signed maximum (fmax drops NaN; the sums keep it).
// 0: the FP32 formats restore through the per-site kernels too
#ifndef TCYM_RESTORE_PAIRED
#define TCYM_RESTORE_PAIRED 1
#endif

template <int FMT>
__global__ void __launch_bounds__(kRedThreads) k_gauss_compute_pair_it(Geom g, const void *U, const void *E, f2 *G2,
                                                                       double *partial, const double *ctl, int it) {
    if ((double)it >= ctl[0]) return;
    using F = Fmt<FMT>;
    using GG = typename F::G2;
    constexpr int NA = F::NA;
    const int64_t Vh = g.V >> 1;
    float gsq = 0.f, gmax = 0.f, gabs = 0.f;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < Vh; p += (int64_t)gridDim.x * blockDim.x) {
        const PairNbhd nb(g, p);
        f2 gv[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) gv[a] = f2(0.0);
#pragma unroll 1
        for (int mu = 0; mu < 3; ++mu) {
            const int64_t pm = nb.at(mu, -1);
            const bool sw = nb.swapped(mu, -1);
            f2 e[NA], em[NA], t[NA];
            F::load_e2(E, Vh, mu, pm, em);
            if (sw) {
#pragma unroll
                for (int a = 0; a < NA; ++a) em[a] = swap_f2(em[a]);
            }
            GG::inverse_adjoint(F::load2(U, Vh, mu, pm, sw), em, t);
            F::load_e2(E, Vh, mu, p, e);
#pragma unroll
            for (int a = 0; a < NA; ++a) gv[a] += e[a] - t[a];
        }
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            G2[a * Vh + p] = gv[a];
            const float x = gv[a].v.x, y = gv[a].v.y;
            gsq = fmaf(x, x, fmaf(y, y, gsq));
            gmax = fmaxf(gmax, fmaxf(x, y));
            gabs = fmaxf(gabs, fmaxf(fabsf(x), fabsf(y)));
        }
    }
    double v[P_WIDTH];
#pragma unroll
    for (int k = 0; k < P_WIDTH; ++k) v[k] = 0.0;
    v[P_GSQ] = gsq;
    v[P_GMAX] = gmax;
    v[P_GABS] = gabs;
    block_partial(v, partial);
}

// E_mu(x) -= gam (G(x) - U_mu(x) G(x+mu) U_mu^dag(x)) for both sites of a pair, in FP32
template <int FMT>
__global__ void __launch_bounds__(kThreadsPair) k_gauss_update_pair_it(Geom g, const void *U, void *E, const f2 *G2,
                                                                      float gam, const double *ctl, int it) {
    if ((double)it >= ctl[0]) return;
    using F = Fmt<FMT>;
    using GG = typename F::G2;
    constexpr int NA = F::NA;
    const int64_t Vh = g.V >> 1;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= Vh) return;
    const PairNbhd nb(g, p);
    const f2 mg(-(double)gam);
    f2 gx[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) gx[a] = G2[a * Vh + p];
#pragma unroll 1
    for (int mu = 0; mu < 3; ++mu) {
        const int64_t pp = nb.at(mu, 1);
        const bool sw = nb.swapped(mu, 1);
        f2 gp[NA], t[NA], e[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) gp[a] = sw ? swap_f2(G2[a * Vh + pp]) : G2[a * Vh + pp];
        GG::adjoint(F::load2(U, Vh, mu, p, false), gp, t);
        F::load_e2(E, Vh, mu, p, e);
#pragma unroll
        for (int a = 0; a < NA; ++a) e[a] = fma(mg, gx[a] - t[a], e[a]);
        F::store_e2(E, Vh, mu, p, e);
    }
}

template <int FMT> __global__ void k_set_zero(Geom g, void *U, void *E) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < g.V) site_set_zero<Fmt<FMT>>(g, U, E, s);
}
template <int FMT> __global__ void k_gaussian_efield(Geom g, void *E, double sigma, uint64_t seed, uint64_t step) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < g.V) site_gaussian_efield<Fmt<FMT>>(g, E, sigma, seed, s, step);
}
template <int FMT> __global__ void k_random_links(Geom g, void *U, double sigma, uint64_t seed) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < g.V) site_random_links<Fmt<FMT>>(g, U, sigma, seed, s);
}
template <int FMT> __global__ void k_block(Geom gs, Geom gd, const void *Us, void *Ud) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < gd.V) site_block<Fmt<FMT>>(gs, gd, Us, Ud, s);
}
template <int FMT> __global__ void k_reunitarize(Geom g, void *U) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < g.V) site_reunitarize<Fmt<FMT>>(g, U, s);
}
template <int FMT>
__global__ void k_geodesic(Geom g, const void *Uold, const void *Unew, double c, void *Umid, void *Emid) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < g.V) site_geodesic<Fmt<FMT>>(g, Uold, Unew, c, Umid, Emid, s);
}
// Sites [s0, s0 + n) between the reference's AoS FP64 arrays and the device
// layout.  A block takes kAosSites sites: their AoS records (SU(3): 432 + 192 B a
// site) pass through shared memory, so that the AoS side is read or written by
// consecutive threads at consecutive addresses; each thread then converts one link.
constexpr int kAosSites = 64, kAosThreads = 192;
template <int FMT> constexpr int aos_link_doubles() { return Fmt<FMT>::NA == 3 ? 4 : 18; }
template <int FMT> constexpr size_t aos_smem() {
    return sizeof(double) * kAosSites * 3 * (aos_link_doubles<FMT>() + Fmt<FMT>::NA);
}
template <int FMT>
__global__ void __launch_bounds__(kAosThreads)
    k_from_aos(Geom g, void *U, void *E, const double *Ua, const double *Ea, int64_t s0, int64_t n) {
    using F = Fmt<FMT>;
    constexpr int NMD = aos_link_doubles<FMT>(), NA = F::NA;
    extern __shared__ double aos_sh[];
    double *su = aos_sh, *se = aos_sh + kAosSites * 3 * NMD;
    const int64_t b0 = s0 + (int64_t)blockIdx.x * kAosSites;
    const int ns = (int)(n - (b0 - s0) < kAosSites ? n - (b0 - s0) : kAosSites);
    if (Ua)
        for (int i = threadIdx.x; i < ns * 3 * NMD; i += blockDim.x) su[i] = Ua[b0 * 3 * NMD + i];
    if (Ea)
        for (int i = threadIdx.x; i < ns * 3 * NA; i += blockDim.x) se[i] = Ea[b0 * 3 * NA + i];
    __syncthreads();
    const int l = threadIdx.x, site = l / 3, mu = l - 3 * site;
    if (site >= ns) return;
    site_link_from_aos<F>(g, U, E, Ua ? su : nullptr, Ea ? se : nullptr, site, b0 + site, mu);
}
template <int FMT>
__global__ void __launch_bounds__(kAosThreads)
    k_to_aos(Geom g, const void *U, const void *E, double *Ua, double *Ea, int64_t s0, int64_t n) {
    using F = Fmt<FMT>;
    constexpr int NMD = aos_link_doubles<FMT>(), NA = F::NA;
    extern __shared__ double aos_sh[];
    double *su = aos_sh, *se = aos_sh + kAosSites * 3 * NMD;
    const int64_t b0 = s0 + (int64_t)blockIdx.x * kAosSites;
    const int ns = (int)(n - (b0 - s0) < kAosSites ? n - (b0 - s0) : kAosSites);
    const int l = threadIdx.x, site = l / 3, mu = l - 3 * site;
    if (site < ns) site_link_to_aos<F>(g, U, E, Ua ? su : nullptr, Ea ? se : nullptr, site, b0 + site, mu);
    __syncthreads();
    if (Ua)
        for (int i = threadIdx.x; i < ns * 3 * NMD; i += blockDim.x) Ua[b0 * 3 * NMD + i] = su[i];
    if (Ea)
        for (int i = threadIdx.x; i < ns * 3 * NA; i += blockDim.x) Ea[b0 * 3 * NA + i] = se[i];
}

// ------------------------------------------------------------------ launchers
template <int FMT> struct Launch {
    using F = Fmt<FMT>;
    using T = typename F::T;
    static constexpr int FMT_ID = FMT;
    static constexpr int TPB = threads_for<FMT>();

    // t: the block tiling of the paired step (FP32 formats with even nz)
    static cudaError_t step(const Geom &g, const void *Uin, void *Uout, void *E, const StepCoef<double> &cd, bool doE,
                            bool doU, cudaStream_t st, const Tile &t = Tile{0, 0, 0, 0, 0, 0}) {
        StepCoef<T> c = coef_cast<T>(cd);
        if constexpr (F::PAIRED) {
            if (doE && doU && g.nz % 2 == 0) {
                const unsigned blocks = (unsigned)tile_blocks(g, t);
                if (t.tx) k_step_pair<FMT, true><<<blocks, kThreadsPair, 0, st>>>(g, Uin, Uout, E, c, t);
                else k_step_pair<FMT, false><<<blocks, kThreadsPair, 0, st>>>(g, Uin, Uout, E, c, t);
                return cudaGetLastError();
            }
        }
        int grid = grid_for(g.V, TPB);
        if (doE && doU) k_step<FMT, true, true><<<grid, TPB, 0, st>>>(g, Uin, Uout, E, c, 0, g.V);
        else if (doE) k_step<FMT, true, false><<<grid, TPB, 0, st>>>(g, Uin, Uout, E, c, 0, g.V);
        else k_step<FMT, false, true><<<grid, TPB, 0, st>>>(g, Uin, Uout, E, c, 0, g.V);
        return cudaGetLastError();
    }
    // Does step() take the paired kernel (one thread per site pair)?
    static bool paired_step(const Geom &g) { return F::PAIRED && g.nz % 2 == 0; }
    // One fused step (E and links) of the storage indices [i0, i1) only: site
    // pairs when paired_step(g), else sites; i0 a multiple of 128 for pairs.
    // The linear block mapping.
    static cudaError_t step_range(const Geom &g, const void *Uin, void *Uout, void *E, const StepCoef<double> &cd,
                                  int64_t i0, int64_t i1, cudaStream_t st) {
        StepCoef<T> c = coef_cast<T>(cd);
        if (i1 <= i0) return cudaSuccess;
        if constexpr (F::PAIRED) {
            if (paired_step(g)) {
                Tile t{0, 0, 0, 0, 0, (int)(i0 / kThreadsPair)};
                const unsigned blocks = (unsigned)((i1 - i0 + kThreadsPair - 1) / kThreadsPair);
                k_step_pair<FMT, false><<<blocks, kThreadsPair, 0, st>>>(g, Uin, Uout, E, c, t);
                return cudaGetLastError();
            }
        }
        k_step<FMT, true, true><<<grid_for(i1 - i0, TPB), TPB, 0, st>>>(g, Uin, Uout, E, c, i0, i1);
        return cudaGetLastError();
    }
    static cudaError_t flow_cb(const Geom &g, void *U, int parity, int mu, const double *fc, const double *cn,
                               const double *uc, cudaStream_t st) {
        int grid = grid_for(g.V / 2, TPB);
        k_flow_cb<FMT><<<grid, TPB, 0, st>>>(g, U, parity, mu, (T)fc[0], (T)fc[1], (T)fc[2], (T)cn[0], (T)cn[1],
                                             (T)cn[2], (T)uc[0], (T)uc[1], (T)uc[2]);
        return cudaGetLastError();
    }
    static int reduce_grid(const Geom &g, int max_blocks) {
        int b = grid_for(g.V, kRedThreads);
        return b < max_blocks ? b : max_blocks;
    }
    static cudaError_t observables(const Geom &g, const void *U, const void *E, int mask, double *partial, int blocks,
                                   cudaStream_t st) {
        if constexpr (Fmt<FMT>::PAIRED) {
            if (mask == OBS_EDOTB && g.nz % 2 == 0) {  // the N_CS sample: paired FP32
                k_edotb_obs_pair<FMT><<<blocks, kRedThreads, 0, st>>>(g, U, E, partial);
                return cudaGetLastError();
            }
        }
        k_observables<FMT><<<blocks, kRedThreads, 0, st>>>(g, U, E, mask, partial);
        return cudaGetLastError();
    }
    static cudaError_t gauss_compute(const Geom &g, const void *U, const void *E, double *G, double *partial,
                                     int blocks, cudaStream_t st) {
        k_gauss_compute<FMT><<<blocks, kRedThreads, 0, st>>>(g, U, E, G, partial);
        return cudaGetLastError();
    }
    static cudaError_t gauss_update(const Geom &g, const void *U, void *E, const double *G, double gam,
                                    cudaStream_t st) {
        k_gauss_update<FMT><<<grid_for(g.V, TPB), TPB, 0, st>>>(g, U, E, G, gam);
        return cudaGetLastError();
    }
    // the restore iteration: paired FP32 kernels where the storage is paired
    static constexpr bool restore_paired(const Geom &g) { return TCYM_RESTORE_PAIRED && Fmt<FMT>::PAIRED && g.nz % 2 == 0; }
    static cudaError_t gauss_compute_it(const Geom &g, const void *U, const void *E, double *G, double *partial,
                                        int blocks, const double *ctl, int it, cudaStream_t st) {
        if constexpr (Fmt<FMT>::PAIRED) {
            if (restore_paired(g)) {
                k_gauss_compute_pair_it<FMT><<<blocks, kRedThreads, 0, st>>>(g, U, E, reinterpret_cast<f2 *>(G),
                                                                             partial, ctl, it);
                return cudaGetLastError();
            }
        }
        k_gauss_compute_it<FMT><<<blocks, kRedThreads, 0, st>>>(g, U, E, G, partial, ctl, it);
        return cudaGetLastError();
    }
    static cudaError_t gauss_update_it(const Geom &g, const void *U, void *E, const double *G, double gam,
                                       const double *ctl, int it, cudaStream_t st) {
        if constexpr (Fmt<FMT>::PAIRED) {
            if (restore_paired(g)) {
                k_gauss_update_pair_it<FMT><<<grid_for(g.V >> 1, kThreadsPair), kThreadsPair, 0, st>>>(
                    g, U, E, reinterpret_cast<const f2 *>(G), (float)gam, ctl, it);
                return cudaGetLastError();
            }
        }
        k_gauss_update_it<FMT><<<grid_for(g.V, TPB), TPB, 0, st>>>(g, U, E, G, gam, ctl, it);
        return cudaGetLastError();
    }
    static cudaError_t set_zero(const Geom &g, void *U, void *E, cudaStream_t st) {
        k_set_zero<FMT><<<grid_for(g.V, 256), 256, 0, st>>>(g, U, E);
        return cudaGetLastError();
    }
    static cudaError_t gaussian_efield(const Geom &g, void *E, double sigma, uint64_t seed, uint64_t step,
                                       cudaStream_t st) {
        k_gaussian_efield<FMT><<<grid_for(g.V, 128), 128, 0, st>>>(g, E, sigma, seed, step);
        return cudaGetLastError();
    }
    static cudaError_t random_links(const Geom &g, void *U, double sigma, uint64_t seed, cudaStream_t st) {
        k_random_links<FMT><<<grid_for(g.V, 128), 128, 0, st>>>(g, U, sigma, seed);
        return cudaGetLastError();
    }
    static cudaError_t geodesic(const Geom &g, const void *Uold, const void *Unew, double c, void *Umid, void *Emid,
                                cudaStream_t st) {
        k_geodesic<FMT><<<grid_for(g.V, 128), 128, 0, st>>>(g, Uold, Unew, c, Umid, Emid);
        return cudaGetLastError();
    }
    // the blocked links of gs on gd (half the even extents)
    static cudaError_t block(const Geom &gs, const Geom &gd, const void *Us, void *Ud, cudaStream_t st) {
        k_block<FMT><<<grid_for(gd.V, 128), 128, 0, st>>>(gs, gd, Us, Ud);
        return cudaGetLastError();
    }
    static cudaError_t reunitarize(const Geom &g, void *U, cudaStream_t st) {
        k_reunitarize<FMT><<<grid_for(g.V, 128), 128, 0, st>>>(g, U);
        return cudaGetLastError();
    }
    // sites [s0, s0 + n) (n < 0: all)
    static cudaError_t from_aos(const Geom &g, void *U, void *E, const double *Ua, const double *Ea, cudaStream_t st,
                                int64_t s0 = 0, int64_t n = -1) {
        if (n < 0) n = g.V - s0;
        k_from_aos<FMT><<<grid_for(n, kAosSites), kAosThreads, aos_smem<FMT>(), st>>>(g, U, E, Ua, Ea, s0, n);
        return cudaGetLastError();
    }
    static cudaError_t to_aos(const Geom &g, const void *U, const void *E, double *Ua, double *Ea, cudaStream_t st,
                              int64_t s0 = 0, int64_t n = -1) {
        if (n < 0) n = g.V - s0;
        k_to_aos<FMT><<<grid_for(n, kAosSites), kAosThreads, aos_smem<FMT>(), st>>>(g, U, E, Ua, Ea, s0, n);
        return cudaGetLastError();
    }
};

// Sum the block partials in block order and write the result block; optionally
// advance the Kahan-compensated N_CS by ncs_dt * E.B / (8 pi^2).
cudaError_t finalize_obs(const double *partial, int blocks, int na, int64_t V, double ncs_dt, double *result,
                         cudaStream_t st);
// loads k_finalize's code now (with lazy module loading it would load at its first launch)
cudaError_t preload_finalize();
// The finaliser of a Gauss restore's reduction in iteration `it` (-1: the initial
// deviation), skipped when it >= ctl[0].  A non-finite reduction sets ctl[1] and
// stops the restore after this iteration; with `check` (the deviation the
// reference tests, GaussRestore.cpp:150), a signed maximum <= tol stops it too.
cudaError_t finalize_restore(const double *partial, int blocks, int na, int64_t V, double *result, double *ctl,
                             double tol, int it, bool check, cudaStream_t st);

}  // namespace tcym
