// C ABI (include/tcym.h): contexts, lattice handles and the host side of
// every call.  The host side only sizes launches and orders them on the
// lattice's stream; all arithmetic is in the kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "../../include/tcym.h"
#include "tcym_batch.cuh"
#include "tcym_internal.h"
#include "tcym_pipeline.h"

using namespace tcym;

// ------------------------------------------------------------------ errors
void tcym_set_error(tcym_ctx ctx, const char *fmt, ...) {
    if (!ctx) return;
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->last_error = buf;
}

static int cuda_fail(tcym_ctx ctx, cudaError_t e, const char *where) {
    tcym_set_error(ctx, "%s: %s", where, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TCYM_ERR_OOM : TCYM_ERR_CUDA;
}

#define CK(call)                                                 \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

// ------------------------------------------------------- format dispatching
// Runs `body` with the Launch<FMT> type of the lattice's storage format.
#define DISPATCH(fmt, body)                                                \
    switch (fmt) {                                                         \
        case FMT_SU2_F32: { using L = Launch<FMT_SU2_F32>; body; } break;  \
        case FMT_SU2_F64: { using L = Launch<FMT_SU2_F64>; body; } break;  \
        case FMT_SU3_F32: { using L = Launch<FMT_SU3_F32>; body; } break;  \
        case FMT_SU3_F64: { using L = Launch<FMT_SU3_F64>; body; } break;  \
        default: return TCYM_ERR_ARG;                                      \
    }

int tcym_format_of(int nc, int precision) {
    if (nc == 2) return precision == TCYM_FP32 ? FMT_SU2_F32 : FMT_SU2_F64;
    return precision == TCYM_FP32 ? FMT_SU3_F32 : FMT_SU3_F64;
}

size_t tcym_link_bytes(int fmt) {
    switch (fmt) {
        case FMT_SU2_F32: return 16;
        case FMT_SU2_F64: return 32;
        case FMT_SU3_F32: return 48;
        default: return 144;
    }
}
// sites stored per plane: the FP32 formats hold site pairs, padded to even V
size_t tcym_stored_sites(int fmt, int64_t V) {
    return (fmt == FMT_SU2_F32 || fmt == FMT_SU3_F32) ? 2 * (size_t)pair_sites(V) : (size_t)V;
}
size_t tcym_field_bytes(int fmt) {
    switch (fmt) {
        case FMT_SU2_F32: return 12;
        case FMT_SU2_F64: return 24;
        case FMT_SU3_F32: return 32;
        default: return 64;
    }
}

// Step coefficients of the reference for spacings a[3], Minkowski metric
// (gUp = gDown = sqrt(-g) = 1, Dynamics.cpp:40-48) and aScale = 1.
StepCoef<double> tcym_coef(const double *a, int mode, double dt, double gamma, double T, uint64_t seed,
                           uint64_t step) {
    StepCoef<double> c;
    std::memset(&c, 0, sizeof(c));
    c.mode = mode;
    c.seed = seed;
    c.step = step;
    const double acube = a[0] * a[1] * a[2];
    // leapfrog / Langevin: gamma = -2 dt sqrt(-g) a^3, cE = 1/a_mu^2 (Dynamics.cpp:150-155)
    // flow: gamma = -2 sqrt(-g) a^3 aScale (GradientFlow.cpp:40-46)
    const double g = mode == MODE_FLOW ? -2.0 * acube : -2.0 * dt * acube;
    for (int mu = 0; mu < 3; ++mu) {
        const double cE = 1.0 / (a[mu] * a[mu]);
        c.fc[mu] = g * cE;
        c.cnu[mu] = cE;
        // cU = -dt gDown a_mu^2 / (sqrt(-g) a^3) (Dynamics.cpp:100-104; flow: dt -> DcTau, GradientFlow.cpp:111-115)
        c.uc[mu] = -dt * a[mu] * a[mu] / acube;
        if (mode == MODE_LANGEVIN) {
            // cS = sqrt(-g) a^3 / a_mu^2 * dt, cR = sqrt(dt) / a_mu^2 (LangevinDynamics.cpp:182-188);
            // xi = sqrt(2/beta) N(0,1) = sqrt(2T) N(0,1); damping gamma generalises the reference's 1
            c.damp[mu] = gamma * acube * cE * dt;
            c.kick[mu] = std::sqrt(gamma) * std::sqrt(dt) * cE * std::sqrt(2.0 * T);
        }
    }
    return c;
}

// ------------------------------------------------------------------ context
extern "C" int tcym_version(void) { return TCYM_VERSION; }

extern "C" int tcym_ctx_create(int device, tcym_ctx *out) {
    if (!out) return TCYM_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return TCYM_ERR_CUDA;
    tcym_ctx ctx = new (std::nothrow) tcym_ctx_s();
    if (!ctx) return TCYM_ERR_OOM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return TCYM_ERR_CUDA; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
        ctx->sm_count = prop.multiProcessorCount;
        ctx->mem_pitch = prop.memPitch;
    }
    *out = ctx;
    return TCYM_OK;
}

extern "C" int tcym_ctx_destroy(tcym_ctx ctx) {
    if (!ctx) return TCYM_ERR_ARG;
    delete ctx;
    return TCYM_OK;
}

extern "C" const char *tcym_last_error(tcym_ctx ctx) {
    if (!ctx) return "null context";
    return ctx->last_error.c_str();
}

// ------------------------------------------------------------------ lattices
static void drop_host_graphs(tcym_lattice lat) {
    for (auto &h : lat->host_graph) {
        if (h.exec) cudaGraphExecDestroy(h.exec);
        h = tcym_lattice_s::HostStepGraph{};
    }
}

cudaError_t tcym_lattice_alloc(tcym_lattice lat, void **p, size_t bytes) {
    if (lat->pool) return cudaMallocFromPoolAsync(p, bytes, lat->pool, lat->stream);
    return cudaMalloc(p, bytes);
}
void tcym_lattice_free_mem(tcym_lattice lat, void *p) {
    if (!p) return;
    if (lat->pool) cudaFreeAsync(p, lat->stream);
    else cudaFree(p);
}

static void lattice_free(tcym_lattice lat) {
    cudaSetDevice(lat->ctx->device);
    if (lat->stream) cudaStreamSynchronize(lat->stream);
    drop_host_graphs(lat);
    tcym_lattice_free_mem(lat, lat->U[0]);
    tcym_lattice_free_mem(lat, lat->U[1]);
    tcym_lattice_free_mem(lat, lat->E);
    tcym_lattice_free_mem(lat, lat->partial);
    tcym_lattice_free_mem(lat, lat->result);
    tcym_lattice_free_mem(lat, lat->gauss);
    tcym_lattice_free_mem(lat, lat->staging);
    if (lat->host_result) {
        if (lat->pool) std::free(lat->host_result);
        else cudaFreeHost(lat->host_result);
    }
    for (int i = 0; i < 2; ++i)
        if (lat->side[i]) cudaStreamDestroy(lat->side[i]);
    for (int i = 0; i < 3; ++i)
        if (lat->ev[i]) cudaEventDestroy(lat->ev[i]);
    for (auto &st : lat->hs)
        if (st) cudaStreamDestroy(st);
    for (auto &ev : lat->hev)
        if (ev) cudaEventDestroy(ev);
    if (lat->stream) cudaStreamDestroy(lat->stream);
}

static int lattice_create(tcym_ctx ctx, int nc, int nx, int ny, int nz, const double a[3], int precision,
                          cudaMemPool_t pool, tcym_lattice *out) {
    if (!ctx || !out) return TCYM_ERR_ARG;
    *out = nullptr;
    if ((nc != 2 && nc != 3) || (precision != TCYM_FP32 && precision != TCYM_FP64) || nx < 2 || ny < 2 || nz < 2) {
        tcym_set_error(ctx, "tcym_lattice_create: nc must be 2 or 3, extents >= 2, precision FP32/FP64");
        return TCYM_ERR_ARG;
    }
    const int64_t V = (int64_t)nx * ny * nz;
    if (V >= (int64_t)1 << 32) {
        tcym_set_error(ctx, "tcym_lattice_create: at most 2^32-1 sites (the noise counter holds a 32-bit site)");
        return TCYM_ERR_ARG;
    }
    tcym_lattice lat = new (std::nothrow) tcym_lattice_s();
    if (!lat) return TCYM_ERR_OOM;
    lat->ctx = ctx;
    lat->nc = nc;
    lat->precision = precision;
    lat->fmt = tcym_format_of(nc, precision);
    lat->g = Geom{nx, ny, nz, V};
    for (int i = 0; i < 3; ++i) lat->a[i] = a ? a[i] : 1.0;
    lat->reunit_period = precision == TCYM_FP32 ? 100 : 0;
    cudaSetDevice(ctx->device);
    auto fail = [&](cudaError_t e, const char *w) {
        int r = cuda_fail(ctx, e, w);
        lattice_free(lat);
        delete lat;
        return r;
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&lat->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
    lat->pool = pool;
    const size_t nst = tcym_stored_sites(lat->fmt, V);
    const size_t ub = 3 * tcym_link_bytes(lat->fmt) * nst, eb = 3 * tcym_field_bytes(lat->fmt) * nst;
    auto alloc = [&](void **p, size_t n) { return tcym_lattice_alloc(lat, p, n); };
    if ((e = alloc(&lat->U[0], ub)) != cudaSuccess) return fail(e, "allocation of U");
    if ((e = alloc(&lat->U[1], ub)) != cudaSuccess) return fail(e, "allocation of U'");
    if ((e = alloc(&lat->E, eb)) != cudaSuccess) return fail(e, "allocation of E");
    lat->max_blocks = ctx->sm_count * 8;
    if ((e = alloc((void **)&lat->partial, sizeof(double) * P_WIDTH * lat->max_blocks)) != cudaSuccess)
        return fail(e, "allocation of the reduction records");
    if ((e = alloc((void **)&lat->result, sizeof(double) * R_WIDTH)) != cudaSuccess)
        return fail(e, "allocation of the result block");
    if ((e = cudaMemsetAsync(lat->result, 0, sizeof(double) * R_WIDTH, lat->stream)) != cudaSuccess)
        return fail(e, "memset(result)");
    if (pool) {
        lat->host_result = static_cast<double *>(std::calloc(R_WIDTH, sizeof(double)));
        if (!lat->host_result) return fail(cudaErrorMemoryAllocation, "host result block");
    } else if ((e = cudaMallocHost(&lat->host_result, sizeof(double) * R_WIDTH)) != cudaSuccess) {
        return fail(e, "cudaMallocHost(result)");
    }
    lat->bytes = 2 * ub + eb + sizeof(double) * (P_WIDTH * lat->max_blocks + R_WIDTH);
    *out = lat;
    return TCYM_OK;
}

extern "C" int tcym_lattice_create_ex(tcym_ctx ctx, int nc, int nx, int ny, int nz, const double a[3], int precision,
                                      tcym_lattice *out) {
    return lattice_create(ctx, nc, nx, ny, nz, a, precision, nullptr, out);
}

int tcym_lattice_create_pooled(tcym_ctx ctx, int nc, int nx, int ny, int nz, int precision, cudaMemPool_t pool,
                               tcym_lattice *out) {
    return lattice_create(ctx, nc, nx, ny, nz, nullptr, precision, pool, out);
}

extern "C" int tcym_lattice_create(tcym_ctx ctx, int nc, int nx, int ny, int nz, int precision, tcym_lattice *out) {
    return tcym_lattice_create_ex(ctx, nc, nx, ny, nz, nullptr, precision, out);
}

extern "C" int tcym_lattice_destroy(tcym_lattice lat) {
    if (!lat) return TCYM_ERR_ARG;
    lattice_free(lat);
    delete lat;
    return TCYM_OK;
}

// Doubles of a lattice's restore scratch: the violation array G[a*V + s] and the
// restore's control block (first iteration not to run, non-finite flag, spare).
static size_t gauss_scratch_doubles(const tcym_lattice_s *lat) {
    return (size_t)(lat->nc == 2 ? 3 : 8) * (size_t)lat->g.V + 4;
}

extern "C" int tcym_lattice_bytes(tcym_lattice lat, size_t *bytes) {
    if (!lat || !bytes) return TCYM_ERR_ARG;
    *bytes = lat->bytes + lat->staging_bytes + (lat->gauss ? sizeof(double) * gauss_scratch_doubles(lat) : 0);
    return TCYM_OK;
}

static int ensure_staging(tcym_lattice lat) {
    tcym_ctx ctx = lat->ctx;
    const int nmd = lat->nc == 2 ? 4 : 18, na = lat->nc == 2 ? 3 : 8;
    const size_t need = sizeof(double) * 3 * (size_t)(nmd + na) * (size_t)lat->g.V;
    for (int i = 0; i < 2; ++i)
        if (!lat->side[i]) CK(cudaStreamCreateWithFlags(&lat->side[i], cudaStreamNonBlocking));
    for (int i = 0; i < 3; ++i)
        if (!lat->ev[i]) CK(cudaEventCreateWithFlags(&lat->ev[i], cudaEventDisableTiming));
    if (lat->staging_bytes >= need) return TCYM_OK;
    drop_host_graphs(lat);
    tcym_lattice_free_mem(lat, lat->staging);
    lat->staging = nullptr;
    lat->staging_bytes = 0;
    CK(tcym_lattice_alloc(lat, (void **)&lat->staging, need));
    lat->staging_bytes = need;
    return TCYM_OK;
}

// host transfers in chunks of about 64 MB (at most 32), at least one
static int64_t transfer_chunks(tcym_lattice lat, bool u, bool e) {
    const int nmd = lat->nc == 2 ? 4 : 18, na = lat->nc == 2 ? 3 : 8;
    const int64_t bytes = (int64_t)sizeof(double) * 3 * ((u ? nmd : 0) + (e ? na : 0)) * lat->g.V;
    int64_t k = bytes / (64ll << 20);
    if (k < 1) k = 1;
    if (k > 32) k = 32;
    if (k > lat->g.V) k = lat->g.V;
    return k;
}
// the lattice's stream waits for both side streams
static cudaError_t join_side(tcym_lattice lat) {
    for (int i = 0; i < 2; ++i) {
        cudaError_t e = cudaEventRecord(lat->ev[1 + i], lat->side[i]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(lat->stream, lat->ev[1 + i], 0);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

extern "C" int tcym_lattice_upload(tcym_lattice lat, const double *U_aos, const double *E_aos) {
    TCYM_RANGE("tcym_lattice_upload");
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    int r = ensure_staging(lat);
    if (r) return r;
    const int nmd = lat->nc == 2 ? 4 : 18, na = lat->nc == 2 ? 3 : 8;
    const int64_t V = lat->g.V;
    double *du = lat->staging, *de = lat->staging + 3 * nmd * V;
    // chunks of sites alternate between two side streams, so that the copy of one
    // chunk overlaps the layout conversion of the previous one (and two copy engines run)
    const int64_t nchunk = transfer_chunks(lat, U_aos != nullptr, E_aos != nullptr);
    CK(cudaEventRecord(lat->ev[0], lat->stream));
    for (int i = 0; i < 2; ++i) CK(cudaStreamWaitEvent(lat->side[i], lat->ev[0], 0));
    for (int64_t k = 0; k < nchunk; ++k) {
        const int64_t s0 = V * k / nchunk, s1 = V * (k + 1) / nchunk;
        cudaStream_t st = lat->side[k & 1];
        if (U_aos)
            CK(cudaMemcpyAsync(du + 3 * nmd * s0, U_aos + 3 * nmd * s0, sizeof(double) * 3 * nmd * (s1 - s0),
                               cudaMemcpyHostToDevice, st));
        if (E_aos)
            CK(cudaMemcpyAsync(de + 3 * na * s0, E_aos + 3 * na * s0, sizeof(double) * 3 * na * (s1 - s0),
                               cudaMemcpyHostToDevice, st));
        DISPATCH(lat->fmt, CK(L::from_aos(lat->g, lat->U[lat->cur], lat->E, U_aos ? du : nullptr,
                                          E_aos ? de : nullptr, st, s0, s1 - s0)));
    }
    CK(join_side(lat));
    CK(cudaStreamSynchronize(lat->stream));
    return TCYM_OK;
}

extern "C" int tcym_lattice_download(tcym_lattice lat, double *U_aos, double *E_aos) {
    TCYM_RANGE("tcym_lattice_download");
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    int r = ensure_staging(lat);
    if (r) return r;
    const int nmd = lat->nc == 2 ? 4 : 18, na = lat->nc == 2 ? 3 : 8;
    const int64_t V = lat->g.V;
    double *du = lat->staging, *de = lat->staging + 3 * nmd * V;
    const int64_t nchunk = transfer_chunks(lat, U_aos != nullptr, E_aos != nullptr);
    CK(cudaEventRecord(lat->ev[0], lat->stream));
    for (int i = 0; i < 2; ++i) CK(cudaStreamWaitEvent(lat->side[i], lat->ev[0], 0));
    for (int64_t k = 0; k < nchunk; ++k) {
        const int64_t s0 = V * k / nchunk, s1 = V * (k + 1) / nchunk;
        cudaStream_t st = lat->side[k & 1];
        DISPATCH(lat->fmt, CK(L::to_aos(lat->g, lat->U[lat->cur], lat->E, U_aos ? du : nullptr,
                                        E_aos ? de : nullptr, st, s0, s1 - s0)));
        if (U_aos)
            CK(cudaMemcpyAsync(U_aos + 3 * nmd * s0, du + 3 * nmd * s0, sizeof(double) * 3 * nmd * (s1 - s0),
                               cudaMemcpyDeviceToHost, st));
        if (E_aos)
            CK(cudaMemcpyAsync(E_aos + 3 * na * s0, de + 3 * na * s0, sizeof(double) * 3 * na * (s1 - s0),
                               cudaMemcpyDeviceToHost, st));
    }
    CK(join_side(lat));
    CK(cudaStreamSynchronize(lat->stream));
    return TCYM_OK;
}

// Block(GaugeLinks**) and Block(ElectricFields**) (LATTICE/GaugeLinks.cpp:124-145,
// LATTICE/ElectricFields.cpp:113-127) into an existing lattice: dst has half the
// (even) extents of src, the same group and precision; it receives the blocked
// links U'_mu(x) = U_mu(2x) U_mu(2x + mu), zero fields and twice src's spacings.
extern "C" int tcym_lattice_block(const tcym_lattice src, tcym_lattice dst) {
    if (!dst || !src) return TCYM_ERR_ARG;
    tcym_ctx ctx = dst->ctx;
    const Geom &gs = src->g, &gd = dst->g;
    if (dst->fmt != src->fmt || ((gs.nx | gs.ny | gs.nz) & 1) || gd.nx * 2 != gs.nx || gd.ny * 2 != gs.ny ||
        gd.nz * 2 != gs.nz) {
        tcym_set_error(ctx, "tcym_lattice_block: dst must have the group and precision of src and half its even extents");
        return TCYM_ERR_ARG;
    }
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(src->stream));
    DISPATCH(dst->fmt, CK(L::block(gs, gd, src->U[src->cur], dst->U[dst->cur], dst->stream)));
    CK(cudaMemsetAsync(dst->E, 0, 3 * tcym_field_bytes(dst->fmt) * tcym_stored_sites(dst->fmt, gd.V), dst->stream));
    for (int i = 0; i < 3; ++i) dst->a[i] = 2.0 * src->a[i];
    drop_host_graphs(dst);  // their step coefficients hold the old spacings
    CK(cudaStreamSynchronize(dst->stream));
    return TCYM_OK;
}

extern "C" int tcym_lattice_copy(tcym_lattice dst, const tcym_lattice src) {
    if (!dst || !src) return TCYM_ERR_ARG;
    tcym_ctx ctx = dst->ctx;
    if (dst->nc != src->nc || dst->g.nx != src->g.nx || dst->g.ny != src->g.ny || dst->g.nz != src->g.nz) {
        tcym_set_error(ctx, "tcym_lattice_copy: group and extents must match");
        return TCYM_ERR_ARG;
    }
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(src->stream));
    if (dst->fmt == src->fmt) {
        const size_t nst = tcym_stored_sites(dst->fmt, dst->g.V);
        const size_t ub = 3 * tcym_link_bytes(dst->fmt) * nst, eb = 3 * tcym_field_bytes(dst->fmt) * nst;
        CK(cudaMemcpyAsync(dst->U[dst->cur], src->U[src->cur], ub, cudaMemcpyDeviceToDevice, dst->stream));
        CK(cudaMemcpyAsync(dst->E, src->E, eb, cudaMemcpyDeviceToDevice, dst->stream));
    } else {
        // through FP64 AoS on the device
        int r = ensure_staging(dst);
        if (r) return r;
        const int nmd = dst->nc == 2 ? 4 : 18;
        double *du = dst->staging, *de = dst->staging + 3 * nmd * (size_t)dst->g.V;
        DISPATCH(src->fmt, CK(L::to_aos(src->g, src->U[src->cur], src->E, du, de, dst->stream)));
        DISPATCH(dst->fmt, CK(L::from_aos(dst->g, dst->U[dst->cur], dst->E, du, de, dst->stream)));
    }
    // the spacings too, as Copy does (GaugeLinks.cpp:91-100)
    if (std::memcmp(dst->a, src->a, sizeof dst->a) != 0) {
        std::memcpy(dst->a, src->a, sizeof dst->a);
        drop_host_graphs(dst);  // their step coefficients hold the old spacings
    }
    CK(cudaStreamSynchronize(dst->stream));
    return TCYM_OK;
}

extern "C" int tcym_lattice_sync(tcym_lattice lat) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    CK(cudaStreamSynchronize(lat->stream));
    return TCYM_OK;
}

void tcym_lattice_release_scratch(tcym_lattice lat) {
    if (!lat) return;
    cudaSetDevice(lat->ctx->device);
    cudaStreamSynchronize(lat->stream);
    drop_host_graphs(lat);
    tcym_lattice_free_mem(lat, lat->gauss);
    tcym_lattice_free_mem(lat, lat->staging);
    lat->gauss = nullptr;
    lat->staging = nullptr;
    lat->staging_bytes = 0;
}

extern "C" int tcym_lattice_stream(tcym_lattice lat, void **stream) {
    if (!lat || !stream) return TCYM_ERR_ARG;
    *stream = (void *)lat->stream;
    return TCYM_OK;
}

extern "C" int tcym_host_alloc(size_t bytes, void **ptr) {
    if (!ptr) return TCYM_ERR_ARG;
    *ptr = nullptr;
    if (bytes == 0) return TCYM_OK;
    const cudaError_t e = cudaMallocHost(ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return e == cudaErrorMemoryAllocation ? TCYM_ERR_OOM : TCYM_ERR_CUDA;
    }
    return TCYM_OK;
}
extern "C" int tcym_host_free(void *ptr) {
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
        cudaGetLastError();
        return TCYM_ERR_ARG;
    }
    return TCYM_OK;
}

// ------------------------------------------------------- initial conditions
extern "C" int tcym_set_zero(tcym_lattice lat) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    DISPATCH(lat->fmt, CK(L::set_zero(lat->g, lat->U[lat->cur], lat->E, lat->stream)));
    return TCYM_OK;
}

extern "C" int tcym_gaussian_efield(tcym_lattice lat, double sigma, uint64_t seed) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    DISPATCH(lat->fmt, CK(L::gaussian_efield(lat->g, lat->E, sigma, seed, 0, lat->stream)));
    return TCYM_OK;
}

extern "C" int tcym_random_links(tcym_lattice lat, double sigma, uint64_t seed) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    DISPATCH(lat->fmt, CK(L::random_links(lat->g, lat->U[lat->cur], sigma, seed, lat->stream)));
    return TCYM_OK;
}

// Runs the observables reduction with `mask` and the finaliser; result on device.
int tcym_reduce(tcym_lattice lat, int mask, double ncs_dt) {
    tcym_ctx ctx = lat->ctx;
    int blocks = 0;
    DISPATCH(lat->fmt, {
        blocks = L::reduce_grid(lat->g, lat->max_blocks);
        CK(L::observables(lat->g, lat->U[lat->cur], lat->E, mask, lat->partial, blocks, lat->stream));
    });
    CK(finalize_obs(lat->partial, blocks, lat->nc == 2 ? 3 : 8, lat->g.V, ncs_dt, lat->result, lat->stream));
    return TCYM_OK;
}

static int fetch_result(tcym_lattice lat) {
    tcym_ctx ctx = lat->ctx;
    CK(cudaMemcpyAsync(lat->host_result, lat->result, sizeof(double) * R_WIDTH, cudaMemcpyDeviceToHost, lat->stream));
    CK(cudaStreamSynchronize(lat->stream));
    return TCYM_OK;
}

// GaussLawRestoration::Restore (GAUSSLAWFIXING/GaussRestore.cpp:131-167).  Each
// iteration is three (deviation, update) sub-steps; the reference stops once the
// signed maximum of the third deviation is <= tol (GaussRestore.cpp:150).  The
// iterations are queued in growing batches between host checks: the finaliser of
// the deciding deviation writes the stopping iteration into the device control
// block, and the kernels of later iterations return at once, so the result, the
// iteration count and the final maximum are those of the reference's loop, with
// one host synchronisation per batch instead of one per iteration.  The result
// block's non-finite flag (sticky) is cleared first: the restore judges only its
// own reductions, and their sums see a NaN that the signed maximum drops.
extern "C" int tcym_gauss_restore(tcym_lattice lat, double tol, int maxit, int *iters, double *final_max) {
    TCYM_RANGE("tcym_gauss_restore");
    if (!lat || maxit < 0) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    const int na = lat->nc == 2 ? 3 : 8;
    if (!lat->gauss) CK(tcym_lattice_alloc(lat, (void **)&lat->gauss, sizeof(double) * gauss_scratch_doubles(lat)));
    double *ctl = lat->gauss + (size_t)na * (size_t)lat->g.V;
    const double gam[3] = {7.0 / 24.0, 7.0 / 48.0, 7.0 / 72.0};
    int blocks = 0;
    DISPATCH(lat->fmt, blocks = L::reduce_grid(lat->g, lat->max_blocks));
    CK(cudaMemsetAsync(lat->result + R_NONFINITE, 0, sizeof(double), lat->stream));
    const double init[4] = {(double)maxit, 0.0, 0.0, 0.0};
    CK(cudaMemcpyAsync(ctl, init, sizeof(init), cudaMemcpyHostToDevice, lat->stream));
    auto deviation = [&](int it, bool check) -> int {
        DISPATCH(lat->fmt, CK(L::gauss_compute_it(lat->g, lat->U[lat->cur], lat->E, lat->gauss, lat->partial, blocks,
                                                  ctl, it, lat->stream)));
        CK(finalize_restore(lat->partial, blocks, na, lat->g.V, lat->result, ctl, tol, it, check, lat->stream));
        return TCYM_OK;
    };
    // initial deviation (GaussRestore.cpp:143)
    int r = deviation(-1, true);
    if (r) return r;
    double h[4];
    int queued = 0, batch = 4, stop = maxit;
    for (;;) {
        CK(cudaMemcpyAsync(h, ctl, sizeof(h), cudaMemcpyDeviceToHost, lat->stream));
        if ((r = fetch_result(lat))) return r;  // synchronises the stream
        stop = (int)h[0];
        if (h[1] != 0.0) {
            tcym_set_error(ctx, "tcym_gauss_restore: non-finite violation at iteration %d", stop - 1);
            return TCYM_ERR_NONFINITE;
        }
        if (stop <= queued || queued >= maxit) break;
        const int n = std::min(batch, maxit - queued);
        for (int it = queued; it < queued + n; ++it)
            for (int k = 0; k < 3; ++k) {
                if ((r = deviation(it, k == 2))) return r;
                DISPATCH(lat->fmt, CK(L::gauss_update_it(lat->g, lat->U[lat->cur], lat->E, lat->gauss, gam[k], ctl, it,
                                                         lat->stream)));
            }
        queued += n;
        batch = std::min(2 * batch, 64);
    }
    if (iters) *iters = std::min(stop, maxit);
    if (final_max) *final_max = lat->host_result[R_GMAX];
    return TCYM_OK;
}

// ThermalDynamics::Thermalize(rounds, max_time) (DYNAMICS/ThermalDynamics.cpp:260-314):
// each round redraws E = N(0,1)/sqrt(beta) (round r draws the field stream at
// step r, ReassignElectricFields :205-226), restores Gauss's law, and runs the
// leapfrog (ThermalDynamics::Update, :238-249) while t = steps * dt < max_time,
// the clock restarting each round (:274, :294).  Every `every` steps it appends
// the reference's ThermalEnergy record (:280-285): t + r max_time, T00, TXX,
// TYY, TZZ, ELECTRIC, MAGNETIC (BulkObservables.cpp:29-52).
extern "C" int tcym_thermalize(tcym_lattice lat, double beta, uint64_t seed, int rounds, double max_time, double dt,
                               double restore_tol, int every, double *series, int series_cap, int *records) {
    TCYM_RANGE("tcym_thermalize");
    if (!lat || !(beta > 0) || rounds < 0 || !(dt > 0) || every < 0 || series_cap < 0 ||
        (series_cap > 0 && !series))
        return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    // the reference restores to 1e-14 (GaussRestore.cpp:150); FP32 storage holds ~1e-6
    const double tol = restore_tol > 0 ? restore_tol : (lat->precision == TCYM_FP64 ? 1e-14 : 1e-6);
    int nrec = 0, rc = 0;
    if (records) *records = 0;
    for (int r = 0; r < rounds; ++r) {
        DISPATCH(lat->fmt, CK(L::gaussian_efield(lat->g, lat->E, 1.0 / std::sqrt(beta), seed, (uint64_t)r,
                                                 lat->stream)));
        if ((rc = tcym_gauss_restore(lat, tol, 10000, nullptr, nullptr))) return rc;
        long nsteps = 0;  // steps of the round: the reference's while (Time() < MaxTime)
        while ((double)nsteps * dt < max_time) ++nsteps;
        long done = 0;
        while (done < nsteps) {
            const long next = every > 0 ? std::min(nsteps, (done / every + 1) * every) : nsteps;
            if ((rc = tcym_run_steps(lat, MODE_LEAPFROG, dt, 0, 0, 0, 0, (int)(next - done)))) return rc;
            done = next;
            if (every > 0 && done % every == 0 && nrec < series_cap) {
                if ((rc = tcym_reduce(lat, OBS_BULK, 0.0)) || (rc = fetch_result(lat))) return rc;
                const double *h = lat->host_result;
                const double e0 = h[R_ESQ0], e1 = h[R_ESQ0 + 1], e2 = h[R_ESQ0 + 2];
                const double b0 = h[R_BSQ0], b1 = h[R_BSQ0 + 1], b2 = h[R_BSQ0 + 2];
                double *rec = series + 7 * (size_t)nrec++;
                rec[0] = (double)done * dt + r * max_time;
                rec[1] = 0.5 * (e0 + e1 + e2 + b0 + b1 + b2);
                rec[2] = 0.5 * ((e1 + e2 + b1 + b2) - (e0 + b0));
                rec[3] = 0.5 * ((e0 + e2 + b0 + b2) - (e1 + b1));
                rec[4] = 0.5 * ((e0 + e1 + b0 + b1) - (e2 + b2));
                rec[5] = 0.5 * (e0 + e1 + e2);
                rec[6] = 0.5 * (b0 + b1 + b2);
                if (records) *records = nrec;
            }
        }
    }
    return TCYM_OK;
}

// ------------------------------------------------------------------ dynamics
static int maybe_track(tcym_lattice lat, double dt, int64_t step_index) {
    if (lat->ncs_every > 0 && (step_index % lat->ncs_every) == 0)
        return tcym_reduce(lat, OBS_EDOTB, dt * lat->ncs_every);
    return TCYM_OK;
}

static int maybe_reunitarize(tcym_lattice lat) {
    tcym_ctx ctx = lat->ctx;
    ++lat->steps_since_reunit;
    if (lat->reunit_period > 0 && lat->steps_since_reunit >= lat->reunit_period) {
        DISPATCH(lat->fmt, CK(L::reunitarize(lat->g, lat->U[lat->cur], lat->stream)));
        lat->steps_since_reunit = 0;
    }
    return TCYM_OK;
}

int tcym_run_steps(tcym_lattice lat, int mode, double dt, double gamma, double T, uint64_t seed, uint64_t step0,
                   int nsteps) {
    TCYM_RANGE("tcym_steps");
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    for (int i = 0; i < nsteps; ++i) {
        StepCoef<double> c = tcym_coef(lat->a, mode, dt, gamma, T, seed, step0 + (uint64_t)i);
        const Tile &t = tcym_lattice_tile_of(lat);
        DISPATCH(lat->fmt,
                 CK(L::step(lat->g, lat->U[lat->cur], lat->U[1 - lat->cur], lat->E, c, true, true, lat->stream, t)));
        lat->cur ^= 1;
        ++lat->steps_done;
        int r = maybe_reunitarize(lat);
        if (r) return r;
        if ((r = maybe_track(lat, dt, lat->steps_done))) return r;
    }
    return TCYM_OK;
}

extern "C" int tcym_leapfrog(tcym_lattice lat, double dt, int nsteps) {
    if (!lat || nsteps < 0) return TCYM_ERR_ARG;
    return tcym_run_steps(lat, MODE_LEAPFROG, dt, 0, 0, 0, 0, nsteps);
}

// ------------------------------------------------------ host-resident step
// The pipeline of tcym_leapfrog_host (order in tcym_pipeline.h) on five
// streams, so that neither copy stream waits behind a kernel: host-to-device
// copies of each chunk (hs[0]); their conversion to the storage layout (hs[1]);
// the step of each chunk on the lattice's stream once its neighbour planes are
// converted; conversion of the stepped chunk back to AoS (hs[2]); its
// device-to-host copies (hs[3]).  Host data of a chunk of storage units
// [a, b): sites [a, b), and for site pairs also their partners [a + Vh,
// b + Vh), moved as one two-row copy per array.  The staging buffer holds the
// AoS state; a chunk's region is converted back into only after it was
// uploaded and converted, so one buffer serves both directions (and U_out
// may be U_in).  Each event is waited on right after it is recorded, so one
// event per edge of the chain suffices.
template <int FMT>
static cudaError_t host_step_pipeline(tcym_lattice lat, const StepCoef<double> &c, int64_t C, size_t max_pitch,
                                      const double *U_in, const double *E_in, double *U_out, double *E_out) {
    using L = Launch<FMT>;
    const int nmd = lat->nc == 2 ? 4 : 18, na = lat->nc == 2 ? 3 : 8;
    const Geom &g = lat->g;
    const int64_t V = g.V, Vh = pair_sites(V), P = (int64_t)g.nx * g.ny;
    const bool paired = L::paired_step(g);  // then V is even and both halves of a chunk are as long
    const int64_t N = paired ? Vh : V;
    double *du = lat->staging, *de = lat->staging + 3 * nmd * V;
    const void *Uin = lat->U[lat->cur];
    void *Uout = lat->U[1 - lat->cur];
    cudaStream_t cin = lat->hs[0], vin = lat->hs[1], vout = lat->hs[2], cout = lat->hs[3], cs = lat->stream;
    cudaEvent_t *ev = lat->hev;  // 0 start, 1 copied in, 2 converted in, 3 stepped, 4 converted out, 5 joins
    cudaError_t err = cudaEventRecord(ev[0], cs);
    for (cudaStream_t st : lat->hs)
        if (err == cudaSuccess) err = cudaStreamWaitEvent(st, ev[0], 0);
    // both halves of a chunk in one two-row copy (pitch Vh sites), or one range
    // copies wider than max_pitch (the device's: about 2 GB, lattices beyond ~200^3) take two
    auto copy = [&](double *dst, const double *src, int64_t a, int64_t n, int nd, cudaMemcpyKind kind,
                    cudaStream_t st) {
        if (err != cudaSuccess) return;
        const size_t w = sizeof(double) * 3 * nd * n, pitch = sizeof(double) * 3 * nd * Vh;
        const int64_t off = 3 * nd * a, half = 3 * nd * Vh;
        if (!paired) {
            err = cudaMemcpyAsync(dst + off, src + off, w, kind, st);
        } else if (pitch <= max_pitch) {
            err = cudaMemcpy2DAsync(dst + off, pitch, src + off, pitch, w, 2, kind, st);
        } else {
            err = cudaMemcpyAsync(dst + off, src + off, w, kind, st);
            if (err == cudaSuccess) err = cudaMemcpyAsync(dst + off + half, src + off + half, w, kind, st);
        }
    };
    auto link = [&](cudaEvent_t e, cudaStream_t from, cudaStream_t to) {
        if (err == cudaSuccess) err = cudaEventRecord(e, from);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(to, e, 0);
    };
    const std::vector<int64_t> bounds = pipeline_bounds(N, P, C);
    pipeline_schedule(bounds, P, [&](int op, int64_t j) {
        if (err != cudaSuccess) return;
        const int64_t a = bounds[j], n = bounds[j + 1] - a;
        if (op == PIPE_UPLOAD) {
            copy(du, U_in, a, n, nmd, cudaMemcpyHostToDevice, cin);
            copy(de, E_in, a, n, na, cudaMemcpyHostToDevice, cin);
            link(ev[1], cin, vin);
            for (int h = 0; h < (paired ? 2 : 1) && err == cudaSuccess; ++h)
                err = L::from_aos(g, lat->U[lat->cur], lat->E, du, de, vin, a + h * Vh, n);
            // the latest conversion covers this chunk's neighbourhood when a step follows
            link(ev[2], vin, cs);
        } else {
            if (err == cudaSuccess) err = L::step_range(g, Uin, Uout, lat->E, c, a, a + n, cs);
            link(ev[3], cs, vout);
            for (int h = 0; h < (paired ? 2 : 1) && err == cudaSuccess; ++h)
                err = L::to_aos(g, Uout, lat->E, du, de, vout, a + h * Vh, n);
            link(ev[4], vout, cout);
            copy(U_out, du, a, n, nmd, cudaMemcpyDeviceToHost, cout);
            copy(E_out, de, a, n, na, cudaMemcpyDeviceToHost, cout);
        }
    });
    // the lattice's stream waits for the last download (which follows every other operation)
    // and for the other side streams, which are idle by then but must join a capture
    for (cudaStream_t st : lat->hs) link(ev[5], st, cs);
    return err;
}

// Units per middle chunk of the host-step pipeline (the ends take one z-plane
// chunks, pipeline_bounds): about 64 MB of host data, a multiple of 128
// (TCYM_HOST_STEP_CHUNK overrides, in units).  Measured on GB300 at 128^3
// SU(3) with uniform chunks: 8.9 ms per step with 64 MB, 9.5-14 ms with 16 MB,
// 12 ms with 5 MB (more, smaller copies), 9.3 ms with 128 MB, against 14.1 ms
// for the three calls upload, step, download; the one-plane ends then took the
// 64 MB case to 8.75 ms.
static int64_t host_step_chunk(tcym_lattice lat, bool paired) {
    const int nmd = lat->nc == 2 ? 4 : 18, na = lat->nc == 2 ? 3 : 8;
    const int64_t unit_bytes = (int64_t)sizeof(double) * 3 * (nmd + na) * (paired ? 2 : 1);
    int64_t C = ((64ll << 20) / unit_bytes) / 128 * 128;
    if (const char *env = getenv("TCYM_HOST_STEP_CHUNK")) {
        const long long v = atoll(env);
        if (v > 0) C = (v + 127) / 128 * 128;
    }
    return C < 128 ? 128 : C;
}
// the largest pitch of the pipeline's two-row copies: the device's, or less
// (TCYM_HOST_STEP_MAX_PITCH, bytes) so that tests reach the two-copy path
static size_t host_step_max_pitch(tcym_lattice lat) {
    size_t p = lat->ctx->mem_pitch;
    if (const char *env = getenv("TCYM_HOST_STEP_MAX_PITCH")) {
        const long long v = atoll(env);
        if (v > 0 && (size_t)v < p) p = (size_t)v;
    }
    return p;
}
static bool pinned_host(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// One leapfrog step of a state held in host memory (reference AoS FP64 arrays
// as tcym_lattice_upload / _download take them), the two transfer directions
// overlapped with each other and with the step.  The lattice holds the new
// state afterwards, exactly as after upload + tcym_leapfrog(lat, dt, 1) +
// download; when a reunitarisation falls due after this step (it must precede
// the download) those three calls run instead.  With pinned host arrays the
// pipeline (about a hundred copies, conversions and step chunks tied by
// events) is captured once as a graph per ping-pong parity and replayed while
// the arrays, dt and the chunk size stay the same: one launch per step instead
// of host-issued operations whose issue order would tie the two directions.
extern "C" int tcym_leapfrog_host(tcym_lattice lat, double dt, const double *U_in, const double *E_in,
                                  double *U_out, double *E_out) {
    TCYM_RANGE("tcym_leapfrog_host");
    if (!lat || !U_in || !E_in || !U_out || !E_out) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    if (lat->reunit_period > 0 && lat->steps_since_reunit + 1 >= lat->reunit_period) {
        int r = tcym_lattice_upload(lat, U_in, E_in);
        if (!r) r = tcym_leapfrog(lat, dt, 1);
        if (!r) r = tcym_lattice_download(lat, U_out, E_out);
        return r;
    }
    int r = ensure_staging(lat);
    if (r) return r;
    for (auto &st : lat->hs)
        if (!st) CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (auto &ev : lat->hev)
        if (!ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    bool paired = false;
    DISPATCH(lat->fmt, paired = L::paired_step(lat->g));
    const int64_t C = host_step_chunk(lat, paired);
    const size_t max_pitch = host_step_max_pitch(lat);
    const StepCoef<double> c = tcym_coef(lat->a, MODE_LEAPFROG, dt, 0, 0, 0, 0);
    const void *io[4] = {U_in, E_in, U_out, E_out};
    const bool graph = pinned_host(U_in) && pinned_host(E_in) && pinned_host(U_out) && pinned_host(E_out);
    if (!graph) {
        DISPATCH(lat->fmt, CK(host_step_pipeline<L::FMT_ID>(lat, c, C, max_pitch, U_in, E_in, U_out, E_out)));
    } else {
        auto &h = lat->host_graph[lat->cur];
        if (!h.exec || h.dt != dt || h.chunk != C || h.max_pitch != max_pitch || h.staging != lat->staging ||
            memcmp(h.io, io, sizeof io) != 0) {
            if (h.exec) cudaGraphExecDestroy(h.exec);
            h = tcym_lattice_s::HostStepGraph{};
            cudaGraph_t gr = nullptr;
            CK(cudaStreamBeginCapture(lat->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            DISPATCH(lat->fmt, e = host_step_pipeline<L::FMT_ID>(lat, c, C, max_pitch, U_in, E_in, U_out, E_out));
            const cudaError_t e2 = cudaStreamEndCapture(lat->stream, &gr);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&h.exec, gr, 0);
            if (gr) cudaGraphDestroy(gr);
            if (e != cudaSuccess) {
                h = tcym_lattice_s::HostStepGraph{};
                return cuda_fail(ctx, e, "tcym_leapfrog_host: capture of the pipeline");
            }
            memcpy(h.io, io, sizeof io);
            h.dt = dt;
            h.chunk = C;
            h.max_pitch = max_pitch;
            h.staging = lat->staging;
        }
        CK(cudaGraphLaunch(h.exec, lat->stream));
    }
    lat->cur ^= 1;
    ++lat->steps_done;
    if ((r = maybe_reunitarize(lat))) return r;
    if ((r = maybe_track(lat, dt, lat->steps_done))) return r;
    CK(cudaStreamSynchronize(lat->stream));
    return TCYM_OK;
}

extern "C" int tcym_langevin(tcym_lattice lat, double dt, double gamma, double T, uint64_t seed, uint64_t step0,
                             int nsteps) {
    if (!lat || nsteps < 0 || gamma < 0 || T < 0 || dt < 0) return TCYM_ERR_ARG;
    const int r = tcym_run_steps(lat, MODE_LANGEVIN, dt, gamma, T, seed, step0, nsteps);
    if (r == TCYM_OK) {
        lat->noise_seed = seed;
        lat->noise_next = step0 + (uint64_t)nsteps;
        lat->noise_valid = true;
    }
    return r;
}

extern "C" int tcym_update_e(tcym_lattice lat, double dt) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    StepCoef<double> c = tcym_coef(lat->a, MODE_LEAPFROG, dt, 0, 0, 0, 0);
    DISPATCH(lat->fmt, CK(L::step(lat->g, lat->U[lat->cur], lat->U[lat->cur], lat->E, c, true, false, lat->stream)));
    return TCYM_OK;
}

extern "C" int tcym_update_u(tcym_lattice lat, double dt) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    StepCoef<double> c = tcym_coef(lat->a, MODE_LEAPFROG, dt, 0, 0, 0, 0);
    DISPATCH(lat->fmt, CK(L::step(lat->g, lat->U[lat->cur], lat->U[lat->cur], lat->E, c, false, true, lat->stream)));
    return TCYM_OK;
}

// FP32 gradient flows reunitarise their links (in FP64, rounded once) at least every
// this many sweeps.  A late flow's updates are small enough that their second-order,
// inward part rounds away in FP32 and the norms grow; a cooled field's magnetic energy
// (N (1 - Re tr U_p / N) a plaquette) follows the norms to first order.  Measured with
// the site code on the host, SU(3) 8^3 cooled to 3e-4 a site in 250 sweeps: 0.28 off the
// FP64 flow without, 8.5e-2 reunitarising every 100 sweeps, 3.8e-6 every 25.
constexpr int kFlowReunitSweeps = 10;
extern "C" int tcym_flow(tcym_lattice lat, double dtau, int nsteps, int mode, int calibrate, double *dncs) {
    TCYM_RANGE("tcym_flow");
    if (!lat || nsteps < 0 || (mode != TCYM_FLOW_SIMULTANEOUS && mode != TCYM_FLOW_CHECKERBOARD) || calibrate < 0 ||
        calibrate > 2)
        return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    // NCsDot operator: the reference's default is the O(a^2)-improved one (ChernSimonsDerivative.cpp:44)
    const int op = calibrate == TCYM_NCS_CLOVER ? OBS_EDOTB : OBS_EDOTB_IMP;
    cudaSetDevice(ctx->device);
    if (mode == TCYM_FLOW_CHECKERBOARD && ((lat->g.nx | lat->g.ny | lat->g.nz) & 1)) {
        tcym_set_error(ctx, "tcym_flow: checkerboard sweeps need even extents");
        return TCYM_ERR_ARG;
    }
    const double inv8pi2 = 0.125 / (M_PI * M_PI);
    double acc = 0.0;
    StepCoef<double> c = tcym_coef(lat->a, MODE_FLOW, dtau, 0, 0, 0, 0);
    int r;
    for (int s = 0; s < nsteps; ++s) {
        if (mode == TCYM_FLOW_SIMULTANEOUS) {
            // F into E and U' = exp(-i dtau F) U into the other buffer; U stays intact
            const Tile &t = tcym_lattice_tile_of(lat);
            DISPATCH(lat->fmt, CK(L::step(lat->g, lat->U[lat->cur], lat->U[1 - lat->cur], lat->E, c, true, true,
                                          lat->stream, t)));
        } else {
            if (calibrate)  // the force of the state before the sweep, for the trapezoid rule
                DISPATCH(lat->fmt, CK(L::step(lat->g, lat->U[lat->cur], lat->U[lat->cur], lat->E, c, true, false,
                                              lat->stream)));
        }
        if (calibrate) {
            if ((r = tcym_reduce(lat, op, 0.0))) return r;
            if ((r = fetch_result(lat))) return r;
            acc += 0.5 * dtau * inv8pi2 * lat->host_result[R_EDB];
        }
        if (mode == TCYM_FLOW_SIMULTANEOUS) {
            lat->cur ^= 1;
        } else {
            for (int p = 0; p < 2; ++p)
                for (int mu = 0; mu < 3; ++mu)
                    DISPATCH(lat->fmt, CK(L::flow_cb(lat->g, lat->U[lat->cur], p, mu, c.fc, c.cnu, c.uc, lat->stream)));
        }
        // FP32 storage: sweeps count toward the links' FP64 reunitarisation, at least
        // every kFlowReunitSweeps (a period of 0 switches it off, as for the dynamics)
        if (lat->precision == TCYM_FP32 && lat->reunit_period > 0 &&
            ++lat->steps_since_reunit >= std::min(lat->reunit_period, kFlowReunitSweeps)) {
            DISPATCH(lat->fmt, CK(L::reunitarize(lat->g, lat->U[lat->cur], lat->stream)));
            lat->steps_since_reunit = 0;
        }
        if (calibrate) {
            if ((r = tcym_reduce(lat, op, 0.0))) return r;
            if ((r = fetch_result(lat))) return r;
            acc += 0.5 * dtau * inv8pi2 * lat->host_result[R_EDB];
        }
    }
    if (dncs) *dncs = acc;
    return TCYM_OK;
}

extern "C" int tcym_reunitarize(tcym_lattice lat) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    cudaSetDevice(ctx->device);
    DISPATCH(lat->fmt, CK(L::reunitarize(lat->g, lat->U[lat->cur], lat->stream)));
    lat->steps_since_reunit = 0;
    return TCYM_OK;
}

extern "C" int tcym_set_reunitarize_period(tcym_lattice lat, int period) {
    if (!lat || period < 0) return TCYM_ERR_ARG;
    lat->reunit_period = period;
    lat->steps_since_reunit = 0;
    return TCYM_OK;
}

// ---------------------------------------------------------------- observables
extern "C" int tcym_observables(tcym_lattice lat, tcym_obs *out) {
    TCYM_RANGE("tcym_observables");
    if (!lat || !out) return TCYM_ERR_ARG;
    cudaSetDevice(lat->ctx->device);
    int r = tcym_reduce(lat, OBS_ALL, 0.0);
    if (r) return r;
    if ((r = fetch_result(lat))) return r;
    const double *h = lat->host_result;
    std::memset(out, 0, sizeof(*out));
    for (int m = 0; m < 3; ++m) { out->esqr[m] = h[R_ESQ0 + m]; out->bsqr[m] = h[R_BSQ0 + m]; }
    // Bulk::ELECTRIC/MAGNETIC/T00 with cE = cB = 1 (BulkObservables.cpp:17-51)
    out->electric = 0.5 * (out->esqr[0] + out->esqr[1] + out->esqr[2]);
    out->magnetic = 0.5 * (out->bsqr[0] + out->bsqr[1] + out->bsqr[2]);
    out->T00 = out->electric + out->magnetic;
    out->gauss_max = h[R_GMAX];
    out->gauss_rms = h[R_GRMS];
    out->gauss_absmax = h[R_GABS];
    out->unit_max = h[R_UMAX];
    out->unit_rms = h[R_URMS];
    out->edotb = h[R_EDB];
    out->ncs_dot = 0.125 * out->edotb / (M_PI * M_PI);
    out->ncs = h[R_NCS];
    out->nonfinite = h[R_NONFINITE] != 0.0;
    if (out->nonfinite) {
        tcym_set_error(lat->ctx, "tcym_observables: non-finite reduction");
        return TCYM_ERR_NONFINITE;
    }
    return TCYM_OK;
}

extern "C" int tcym_edotb(tcym_lattice lat, double *out) {
    if (!lat || !out) return TCYM_ERR_ARG;
    cudaSetDevice(lat->ctx->device);
    int r = tcym_reduce(lat, OBS_EDOTB, 0.0);
    if (r) return r;
    if ((r = fetch_result(lat))) return r;
    *out = lat->host_result[R_EDB];
    return TCYM_OK;
}

extern "C" int tcym_edotb_improved(tcym_lattice lat, double *out) {
    if (!lat || !out) return TCYM_ERR_ARG;
    cudaSetDevice(lat->ctx->device);
    int r = tcym_reduce(lat, OBS_EDOTB_IMP, 0.0);
    if (r) return r;
    if ((r = fetch_result(lat))) return r;
    *out = lat->host_result[R_EDB];
    return TCYM_OK;
}

extern "C" int tcym_ncs_track(tcym_lattice lat, int every) {
    if (!lat || every < 0) return TCYM_ERR_ARG;
    lat->ncs_every = every;
    return TCYM_OK;
}

extern "C" int tcym_ncs_get(tcym_lattice lat, double *ncs) {
    if (!lat || !ncs) return TCYM_ERR_ARG;
    int r = fetch_result(lat);
    if (r) return r;
    *ncs = lat->host_result[R_NCS];
    return TCYM_OK;
}

extern "C" int tcym_ncs_reset(tcym_lattice lat) {
    if (!lat) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    CK(cudaMemsetAsync(lat->result + R_NCS, 0, 2 * sizeof(double), lat->stream));
    CK(cudaStreamSynchronize(lat->stream));
    return TCYM_OK;
}
