// Gauss-law restoration on caller-owned device buffers that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc.  One kind has its device
// memory wholly reserved by its own allocator (a framework's caching allocator
// that has claimed the GPU), so a fresh allocation fails or fragments the
// pool.  Another kind runs a steady-state loop that must never stall: cudaFree
// synchronises the whole device, and cudaMalloc can fail at an arbitrary point
// under memory pressure.  Such a caller already keeps U and E in the
// reference's AoS FP64 layout in its own device memory and cannot create a
// tcym lattice, which owns separate buffers.
//
// tcym_gauss_restore_noalloc runs the same Gauss-restore kernels as
// tcym_gauss_restore directly on those buffers.  Its scratch (the FP64
// violation array, the per-block reduction records and the result block)
// lives in one file-scope static __device__ array of kNoAllocScratchDoubles
// doubles (8 MiB).  Every GPU that loads libtcym.so holds this array until the
// process exits.  Lattices whose violation array does not fit are rejected.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/tcym.h"
#include "tcym_kernels.cuh"

namespace tcym {

// storage formats of the reference's AoS FP64 arrays (LATTICE/GaugeLinks.cpp:27-47,
// LATTICE/ElectricFields.cpp:36-46), used only by this entry point
enum : int { FMT_SU2_AOS64 = 10, FMT_SU3_AOS64 = 11 };

template <> struct Fmt<FMT_SU2_AOS64> {
    using T = double;
    using G = SU2<double>;
    using Mat = G::Mat;
    static constexpr int NA = 3;
    static TCYM_HD Mat load(const void *U, int64_t, int mu, int64_t s) {
        const double *a = static_cast<const double *>(U) + 4 * (mu + 3 * s);
        return Mat{{a[0], a[1], a[2], a[3]}};
    }
    static TCYM_HD void load_e(const void *E, int64_t, int mu, int64_t s, T *e) {
        const double *p = static_cast<const double *>(E) + 3 * (mu + 3 * s);
        e[0] = p[0]; e[1] = p[1]; e[2] = p[2];
    }
    static TCYM_HD void store_e(void *E, int64_t, int mu, int64_t s, const T *e) {
        double *p = static_cast<double *>(E) + 3 * (mu + 3 * s);
        p[0] = e[0]; p[1] = e[1]; p[2] = e[2];
    }
};

template <> struct Fmt<FMT_SU3_AOS64> {
    using T = double;
    using G = SU3<double>;
    using Mat = G::Mat;
    static constexpr int NA = 8;
    static TCYM_HD Mat load(const void *U, int64_t, int mu, int64_t s) {
        const double *a = static_cast<const double *>(U) + 18 * (mu + 3 * s);
        Mat m;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) m.m[i][j] = cx<double>{a[2 * (i + 3 * j)], a[2 * (i + 3 * j) + 1]};
        return m;
    }
    static TCYM_HD void load_e(const void *E, int64_t, int mu, int64_t s, T *e) {
        const double *p = static_cast<const double *>(E) + 8 * (mu + 3 * s);
        for (int a = 0; a < 8; ++a) e[a] = p[a];
    }
    static TCYM_HD void store_e(void *E, int64_t, int mu, int64_t s, const T *e) {
        double *p = static_cast<double *>(E) + 8 * (mu + 3 * s);
        for (int a = 0; a < 8; ++a) p[a] = e[a];
    }
};

// Scratch layout (doubles): result block | reduction records | violation array
constexpr int kNoAllocMaxBlocks = 1024;
constexpr size_t kNoAllocScratchDoubles = size_t(1) << 20;
constexpr size_t kNoAllocViolationCapacity =
    kNoAllocScratchDoubles - R_WIDTH - (size_t)P_WIDTH * kNoAllocMaxBlocks;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Device address of g_noalloc_scratch on the current device, looked up on every
// call with that device current (host code may not use the symbol itself).  The
// lookup allocates nothing once the module is loaded, and it stays right when
// the primary context is torn down and created again (the module then reloads
// and the array may move).  The same call makes sure every kernel the entry
// point runs is loaded, for both groups: with lazy module loading the runtime
// would otherwise place a kernel's code in device memory at its first launch.
static cudaError_t scratch_address(double **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, k_gauss_compute<FMT_SU2_AOS64>)) != cudaSuccess ||
        (e = cudaFuncGetAttributes(&fa, k_gauss_compute<FMT_SU3_AOS64>)) != cudaSuccess ||
        (e = cudaFuncGetAttributes(&fa, k_gauss_update<FMT_SU2_AOS64>)) != cudaSuccess ||
        (e = cudaFuncGetAttributes(&fa, k_gauss_update<FMT_SU3_AOS64>)) != cudaSuccess ||
        (e = preload_finalize()) != cudaSuccess)
        return e;
    *out = static_cast<double *>(p);
    return cudaSuccess;
}

template <int FMT>
static cudaError_t restore_aos(const Geom &g, const double *U, double *E, double tol, int maxit, double *scratch,
                               cudaStream_t st, int *iters, double *final_max, bool *nonfinite) {
    constexpr int NA = Fmt<FMT>::NA;
    constexpr int TPB = threads_for<FMT>();
    double *result = scratch;
    double *partial = scratch + R_WIDTH;
    double *G = partial + (size_t)P_WIDTH * kNoAllocMaxBlocks;
    int blocks = grid_for(g.V, kRedThreads);
    if (blocks > kNoAllocMaxBlocks) blocks = kNoAllocMaxBlocks;
    // the array keeps the previous call's contents: clear the result block
    cudaError_t e = cudaMemsetAsync(result, 0, sizeof(double) * R_WIDTH, st);
    if (e != cudaSuccess) return e;
    // the result block's signed maximum and its non-finite flag (set when a
    // reduction saw NaN or Inf; the maxima alone would drop a NaN)
    double host[R_WIDTH];
    auto fetch = [&](double *gmax, bool *bad) -> cudaError_t {
        cudaError_t r = cudaMemcpyAsync(host, result, sizeof(host), cudaMemcpyDeviceToHost, st);
        if (r != cudaSuccess) return r;
        if ((r = cudaStreamSynchronize(st)) != cudaSuccess) return r;
        *gmax = host[R_GMAX];
        *bad = host[R_NONFINITE] != 0.0 || !(host[R_GMAX] == host[R_GMAX]);
        return cudaSuccess;
    };
    auto deviation = [&]() -> cudaError_t {
        k_gauss_compute<FMT><<<blocks, kRedThreads, 0, st>>>(g, U, E, G, partial);
        cudaError_t r = cudaGetLastError();
        if (r != cudaSuccess) return r;
        return finalize_obs(partial, blocks, NA, g.V, 0.0, result, st);
    };
    const double gam[3] = {7.0 / 24.0, 7.0 / 48.0, 7.0 / 72.0};
    double gmax = 0.0;
    bool bad = false;
    if ((e = deviation()) != cudaSuccess || (e = fetch(&gmax, &bad)) != cudaSuccess) return e;
    int it = 0;
    while (!bad && it < maxit && gmax > tol) {
        for (int k = 0; k < 3; ++k) {
            if ((e = deviation()) != cudaSuccess) return e;
            k_gauss_update<FMT><<<grid_for(g.V, TPB), TPB, 0, st>>>(g, U, E, G, gam[k]);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        // maximum of the last deviation, as the reference tests it (GaussRestore.cpp:150)
        if ((e = fetch(&gmax, &bad)) != cudaSuccess) return e;
        ++it;
    }
    *iters = it;
    *final_max = gmax;
    *nonfinite = bad || gmax > 1e300;
    return cudaSuccess;
}

}  // namespace tcym

using namespace tcym;

static int noalloc_fail(char *errbuf, size_t errlen, int code, const char *msg) {
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", msg);
    return code;
}

extern "C" int tcym_gauss_restore_noalloc(int nc, int nx, int ny, int nz, const double *U_aos, double *E_aos,
                                          double tol, int maxit, void *stream, int *iters, double *final_max,
                                          char *errbuf, size_t errlen) {
    if (errbuf && errlen) errbuf[0] = '\0';
    if ((nc != 2 && nc != 3) || nx < 2 || ny < 2 || nz < 2 || !U_aos || !E_aos || maxit < 0)
        return noalloc_fail(errbuf, errlen, TCYM_ERR_ARG,
                            "tcym_gauss_restore_noalloc: nc must be 2 or 3, extents >= 2, buffers non-null");
    const int64_t V = (int64_t)nx * ny * nz;
    const int64_t need = (int64_t)(nc == 2 ? 3 : 8) * V;
    if (need > (int64_t)kNoAllocViolationCapacity) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "tcym_gauss_restore_noalloc: lattice too large for the fixed scratch: the violation array "
                      "needs %lld doubles, at most %lld fit (SU(2) <= %lld sites, SU(3) <= %lld sites)",
                      (long long)need, (long long)kNoAllocViolationCapacity,
                      (long long)(kNoAllocViolationCapacity / 3), (long long)(kNoAllocViolationCapacity / 8));
        return noalloc_fail(errbuf, errlen, TCYM_ERR_ARG, msg);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    double *scratch = nullptr;
    if (e == cudaSuccess) e = scratch_address(&scratch);
    if (e != cudaSuccess) {
        char msg[256];
        std::snprintf(msg, sizeof(msg), "tcym_gauss_restore_noalloc: scratch address on device %d: %s", dev,
                      cudaGetErrorString(e));
        return noalloc_fail(errbuf, errlen, TCYM_ERR_CUDA, msg);
    }
    const Geom g{nx, ny, nz, V};
    int it = 0;
    double mx = 0.0;
    bool bad = false;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = nc == 2 ? restore_aos<FMT_SU2_AOS64>(g, U_aos, E_aos, tol, maxit, scratch, st, &it, &mx, &bad)
                : restore_aos<FMT_SU3_AOS64>(g, U_aos, E_aos, tol, maxit, scratch, st, &it, &mx, &bad);
    if (e != cudaSuccess) {
        char msg[256];
        std::snprintf(msg, sizeof(msg), "tcym_gauss_restore_noalloc: %s", cudaGetErrorString(e));
        return noalloc_fail(errbuf, errlen, TCYM_ERR_CUDA, msg);
    }
    if (iters) *iters = it;
    if (final_max) *final_max = mx;
    if (bad)
        return noalloc_fail(errbuf, errlen, TCYM_ERR_NONFINITE,
                            "tcym_gauss_restore_noalloc: a reduction saw NaN or Inf (non-finite U or E)");
    return TCYM_OK;
}
