// Internal state behind the opaque handles of include/tcym.h.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <map>
#include <mutex>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "../../include/tcym.h"
#include "tcym_site.cuh"

// An NVTX range over the rest of the scope: the library's entry points show by
// name on an nsys or ncu timeline (a few nanoseconds when no tool listens).
struct TcymRange {
    explicit TcymRange(const char *name) { nvtxRangePushA(name); }
    ~TcymRange() { nvtxRangePop(); }
    TcymRange(const TcymRange &) = delete;
    TcymRange &operator=(const TcymRange &) = delete;
};
#define TCYM_RANGE(name) TcymRange tcym_range_scope_(name)

struct tcym_ctx_s {
    int device = 0;
    int sm_count = 152;
    size_t mem_pitch = (size_t)1 << 31;  // largest pitch of a 2D copy (cudaDeviceProp::memPitch)
    std::mutex mu;
    std::string last_error;
    std::mutex tune_mu;
    std::map<std::array<int, 4>, tcym::Tile> tiles;  // autotuned paired-step tiling per (format, nx, ny, nz)
};

struct tcym_lattice_s {
    tcym_ctx ctx = nullptr;
    int nc = 0, precision = 0, fmt = 0;
    tcym::Geom g{};
    double a[3] = {1, 1, 1};
    void *U[2] = {nullptr, nullptr};  // ping-pong link buffers; U[cur] is the state
    int cur = 0;
    void *E = nullptr;
    double *partial = nullptr;  // per-block reduction records
    int max_blocks = 0;
    double *result = nullptr;   // device result block (also holds the Kahan N_CS)
    double *host_result = nullptr;
    double *gauss = nullptr;    // Gauss violation scratch, allocated by the first restore
    double *staging = nullptr;  // AoS FP64 staging for upload/download, allocated on first use
    size_t staging_bytes = 0;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    int reunit_period = 0, steps_since_reunit = 0;
    int ncs_every = 0;
    int64_t steps_done = 0;
    // the Langevin noise stream of the last tcym_langevin call: its Philox key and
    // the first step it has not drawn yet (kept so a snapshot can resume the stream)
    uint64_t noise_seed = 0, noise_next = 0;
    bool noise_valid = false;
    // device memory from a stream-ordered pool (cudaMallocFromPoolAsync / cudaFreeAsync
    // on the lattice's stream): creating and destroying such a lattice never waits for
    // the rest of the device (the request loop's lattices); nullptr: cudaMalloc
    cudaMemPool_t pool = nullptr;
    tcym::Tile tile{};   // block tiling of the paired step
    bool tile_chosen = false;
    cudaStream_t side[2] = {nullptr, nullptr};  // pipelined host transfers (created with the staging)
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    // tcym_leapfrog_host's pipeline: streams for the host-to-device copies, their
    // conversion, the conversion for the download and the device-to-host copies,
    // and the events tying them (created on first use)
    cudaStream_t hs[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t hev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // tcym_leapfrog_host's pipeline captured as a graph, one per ping-pong parity,
    // with what it was captured for (host arrays, dt, chunk, staging)
    struct HostStepGraph {
        cudaGraphExec_t exec = nullptr;
        const void *io[4] = {nullptr, nullptr, nullptr, nullptr};
        double dt = 0;
        int64_t chunk = 0;
        size_t max_pitch = 0;
        const void *staging = nullptr;
    } host_graph[2];
};

void tcym_set_error(tcym_ctx ctx, const char *fmt, ...);
int tcym_format_of(int nc, int precision);
size_t tcym_link_bytes(int fmt);
size_t tcym_field_bytes(int fmt);
size_t tcym_stored_sites(int fmt, int64_t V);
tcym::StepCoef<double> tcym_coef(const double *a, int mode, double dt, double gamma, double T, uint64_t seed,
                                 uint64_t step);
int tcym_reduce(tcym_lattice lat, int mask, double ncs_dt);
// frees the Gauss-restore and AoS staging scratch of a lattice (reallocated on next use)
void tcym_lattice_release_scratch(tcym_lattice lat);
// a lattice whose device memory comes from `pool` on its own stream (see tcym_lattice_s::pool);
// its host result block is pageable, so neither creation nor destruction synchronises the device
int tcym_lattice_create_pooled(tcym_ctx ctx, int nc, int nx, int ny, int nz, int precision, cudaMemPool_t pool,
                               tcym_lattice *out);
// device allocation and release for a lattice: from its pool when it has one
cudaError_t tcym_lattice_alloc(tcym_lattice lat, void **p, size_t bytes);
void tcym_lattice_free_mem(tcym_lattice lat, void *p);
// the block tiling of lat's paired step, autotuned on first use (tcym_autotune.cu)
const tcym::Tile &tcym_lattice_tile_of(tcym_lattice lat);
int tcym_run_steps(tcym_lattice lat, int mode, double dt, double gamma, double T, uint64_t seed, uint64_t step0,
                   int nsteps);
