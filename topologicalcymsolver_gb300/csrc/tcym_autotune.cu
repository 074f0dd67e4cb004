// Autotuner of the paired step's block tiling (FP32 formats, even nz).
//
// A block of 128 threads covers either 128 consecutive pair indices or a
// tx x ty tile of one z-plane (Tile, tcym_site.cuh); the tile decides how many
// of a pair's +-x and +-y neighbour links the block itself has just loaded,
// i.e. the L1 reuse, and what share of the threads idle on ragged planes.  The
// best choice depends on nx and ny, so the first step of a lattice times the
// candidates on a proxy lattice of the same format, nx and ny (at most 1 GiB;
// best of three trials of ~2 ms each, CUDA events on the proxy's stream), and
// the context keeps the winner per (format, nx, ny, nz); a tile must beat the
// linear mapping by 3% to be taken.  A site's arithmetic does
// not depend on the tiling, only the speed does.
//
// TCYM_TILE=linear or TCYM_TILE=<tx>x<ty> in the environment, or
// tcym_lattice_set_tile, fixes the tiling instead.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/tcym.h"
#include "tcym_batch.cuh"
#include "tcym_internal.h"

using namespace tcym;

namespace {

bool paired_step(tcym_lattice lat) {
    return (lat->fmt == FMT_SU2_F32 || lat->fmt == FMT_SU3_F32) && lat->g.nz % 2 == 0;
}

// TCYM_TILE from the environment: linear -> tx 0; "<tx>x<ty>" with tx * ty = 128
bool tile_from_env(const Geom &g, Tile &t) {
    const char *s = std::getenv("TCYM_TILE");
    if (!s || !*s) return false;
    if (std::strcmp(s, "linear") == 0) {
        t = make_tile(g, 0);
        return true;
    }
    int tx = 0, ty = 0;
    if (std::sscanf(s, "%dx%d", &tx, &ty) == 2 && tx > 0 && (tx & (tx - 1)) == 0 && tx <= 128 && tx * ty == 128) {
        t = make_tile(g, tx);
        return true;
    }
    return false;
}

std::vector<Tile> candidates(const Geom &g) {
    std::vector<Tile> c{make_tile(g, 0)};
    for (int tx = 128; tx >= 8; tx /= 2)
        if (tx <= g.nx && 128 / tx <= g.ny) c.push_back(make_tile(g, tx));
    return c;
}

template <int FMT> cudaError_t step_with(tcym_lattice p, const Tile &t) {
    const StepCoef<double> c = tcym_coef(p->a, MODE_LEAPFROG, 0.05, 0, 0, 0, 0);
    return Launch<FMT>::step(p->g, p->U[0], p->U[1], p->E, c, true, true, p->stream, t);
}

// milliseconds for `reps` steps of the proxy with tiling t (negative: failed)
float time_tile(tcym_lattice p, const Tile &t, int reps) {
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return -1.f;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return -1.f;
    }
    float ms = -1.f;
    bool ok = true;
    for (int r = 0; r < reps + 2 && ok; ++r) {  // two untimed launches first
        if (r == 2) ok = cudaEventRecord(e0, p->stream) == cudaSuccess;
        if (ok) ok = (p->fmt == FMT_SU2_F32 ? step_with<FMT_SU2_F32>(p, t) : step_with<FMT_SU3_F32>(p, t)) == cudaSuccess;
    }
    if (ok && cudaEventRecord(e1, p->stream) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess)
        cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

// The fastest candidate on a proxy lattice; linear unless a tile beats it by 3%
// (timing noise must not pick a slower tiling), and linear when anything fails.
// The proxy has the lattice's nx and ny and as many z-planes as keep it under
// 1 GiB, so that a lattice larger than L2 is timed out of HBM as it runs.
Tile tune(tcym_lattice lat) {
    const Tile linear = make_tile(lat->g, 0);
    const std::vector<Tile> cand = candidates(lat->g);
    if (cand.size() < 2) return linear;
    const size_t per_plane = 3 * (2 * tcym_link_bytes(lat->fmt) + tcym_field_bytes(lat->fmt)) *
                             (size_t)lat->g.nx * (size_t)lat->g.ny;
    int nzp = (int)std::min<size_t>((size_t)lat->g.nz, ((size_t)1 << 30) / per_plane);
    nzp = std::max(2, nzp & ~1);
    tcym_lattice p = nullptr;
    if (tcym_lattice_create_ex(lat->ctx, lat->nc, lat->g.nx, lat->g.ny, nzp, lat->a, lat->precision, &p))
        return linear;
    if (tcym_random_links(p, 0.5, 1) || tcym_gaussian_efield(p, 0.7, 2)) {
        tcym_lattice_destroy(p);
        return linear;
    }
    // launches per trial: about 2 ms of work at ~1e10 link-updates/s
    const int reps = (int)std::max<int64_t>(5, std::min<int64_t>(200, 20000000 / (3 * p->g.V)));
    std::vector<float> ms(cand.size(), -1.f);
    for (int trial = 0; trial < 3; ++trial)  // best of three, candidates interleaved
        for (size_t i = 0; i < cand.size(); ++i) {
            const float t = time_tile(p, cand[i], reps);
            if (t > 0.f && (ms[i] < 0.f || t < ms[i])) ms[i] = t;
        }
    cudaGetLastError();  // a failed candidate leaves nothing behind but its error
    tcym_lattice_destroy(p);
    size_t best = 0;
    for (size_t i = 1; i < cand.size(); ++i)
        if (ms[i] > 0.f && (ms[best] < 0.f || ms[i] < ms[best])) best = i;
    if (best != 0 && ms[0] > 0.f && ms[best] > 0.97f * ms[0]) best = 0;
    return make_tile(lat->g, cand[best].tx);
}

}  // namespace

const Tile &tcym_lattice_tile_of(tcym_lattice lat) {
    if (lat->tile_chosen) return lat->tile;
    lat->tile = make_tile(lat->g, 0);
    lat->tile_chosen = true;
    if (!paired_step(lat) || tile_from_env(lat->g, lat->tile)) return lat->tile;
    const std::array<int, 4> key{lat->fmt, lat->g.nx, lat->g.ny, lat->g.nz};
    std::lock_guard<std::mutex> lock(lat->ctx->tune_mu);
    auto it = lat->ctx->tiles.find(key);
    if (it == lat->ctx->tiles.end()) it = lat->ctx->tiles.emplace(key, tune(lat)).first;
    lat->tile = it->second;
    return lat->tile;
}

extern "C" int tcym_lattice_tile(tcym_lattice lat, int *tx, int *ty) {
    if (!lat || !tx || !ty) return TCYM_ERR_ARG;
    cudaSetDevice(lat->ctx->device);
    const Tile &t = tcym_lattice_tile_of(lat);
    *tx = t.tx;
    *ty = t.ty;
    return TCYM_OK;
}

extern "C" int tcym_lattice_set_tile(tcym_lattice lat, int tx, int ty) {
    if (!lat) return TCYM_ERR_ARG;
    if (tx < 0) {  // back to the autotuner
        lat->tile_chosen = false;
        return TCYM_OK;
    }
    if (tx > 0 && (tx > 128 || (tx & (tx - 1)) != 0 || tx * ty != 128)) return TCYM_ERR_ARG;
    lat->tile = make_tile(lat->g, tx);
    lat->tile_chosen = true;
    return TCYM_OK;
}
