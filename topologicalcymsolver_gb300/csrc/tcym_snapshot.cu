// Binary snapshot of a lattice's device state, for an exact resume.
//
// The reference checkpoints through its configuration text files
// (IO/SaveConfiguration.cpp:3-56, 15 significant digits), which cannot carry
// FP32 storage bit for bit, the Kahan-compensated N_CS or the position of the
// Langevin noise stream.  A snapshot holds the state in the device's own storage
// format plus every counter the next step reads:
//
//   header (kHeaderBytes, little-endian, fixed layout: SnapHeader below)
//   links  U[cur], 3 * link_bytes(fmt) * stored_sites bytes
//   fields E,      3 * field_bytes(fmt) * stored_sites bytes
//
// The header carries the group, precision, extents and spacings, the step
// count, the reunitarisation period and phase, the N_CS tracking period, the
// Kahan pair (sum, compensation) and the sticky non-finite flag, the ping-pong
// parity, the Langevin noise key (seed) and next step, and a 64-bit checksum of
// the payload.  Restoring into a lattice of the same group, precision and
// extents and stepping on is bit-identical to never having stopped.
#include <cstdio>
#include <cstring>

#include "tcym_kernels.cuh"
#include "tcym_internal.h"

using namespace tcym;

namespace {

constexpr char kMagic[8] = {'T', 'C', 'Y', 'M', 'S', 'N', 'A', 'P'};
constexpr uint32_t kVersion = 1;
constexpr size_t kHeaderBytes = 256;

struct SnapHeader {
    char magic[8];
    uint32_t version, header_bytes;
    int32_t nc, precision, fmt, nx, ny, nz;
    double a[3];
    int32_t cur, reunit_period, steps_since_reunit, ncs_every;
    int64_t steps_done;
    uint64_t noise_seed, noise_next;
    uint32_t noise_valid, pad0;
    double ncs, ncs_comp, nonfinite;
    uint64_t link_payload, field_payload, checksum;
};
static_assert(sizeof(SnapHeader) <= kHeaderBytes, "snapshot header grew past its fixed size");

// 64-bit checksum of the payload: a sum of rotated words (order-dependent), fast
// enough to run over GB-sized snapshots on the host.
uint64_t payload_checksum(const unsigned char *p, size_t n, uint64_t h) {
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        std::memcpy(&w, p + i, 8);
        h = ((h << 7) | (h >> 57)) + (w ^ 0x9E3779B97F4A7C15ull);
    }
    for (; i < n; ++i) h = ((h << 7) | (h >> 57)) + p[i];
    return h;
}

size_t link_payload(const tcym_lattice_s *lat) {
    return 3 * tcym_link_bytes(lat->fmt) * tcym_stored_sites(lat->fmt, lat->g.V);
}
size_t field_payload(const tcym_lattice_s *lat) {
    return 3 * tcym_field_bytes(lat->fmt) * tcym_stored_sites(lat->fmt, lat->g.V);
}

int cuda_error(tcym_ctx ctx, cudaError_t e, const char *where) {
    tcym_set_error(ctx, "%s: %s", where, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TCYM_ERR_OOM : TCYM_ERR_CUDA;
}

}  // namespace

extern "C" int tcym_lattice_snapshot_bytes(tcym_lattice lat, size_t *bytes) {
    if (!lat || !bytes) return TCYM_ERR_ARG;
    *bytes = kHeaderBytes + link_payload(lat) + field_payload(lat);
    return TCYM_OK;
}

extern "C" int tcym_lattice_snapshot(tcym_lattice lat, void *buf, size_t bytes) {
    TCYM_RANGE("tcym_lattice_snapshot");
    if (!lat || !buf) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    const size_t lb = link_payload(lat), fb = field_payload(lat);
    if (bytes < kHeaderBytes + lb + fb) {
        tcym_set_error(ctx, "tcym_lattice_snapshot: buffer of %zu bytes, %zu needed", bytes, kHeaderBytes + lb + fb);
        return TCYM_ERR_ARG;
    }
    cudaSetDevice(ctx->device);
    unsigned char *out = static_cast<unsigned char *>(buf);
    double res[R_WIDTH];
    cudaError_t e;
    if ((e = cudaMemcpyAsync(out + kHeaderBytes, lat->U[lat->cur], lb, cudaMemcpyDeviceToHost, lat->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out + kHeaderBytes + lb, lat->E, fb, cudaMemcpyDeviceToHost, lat->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(res, lat->result, sizeof(res), cudaMemcpyDeviceToHost, lat->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(lat->stream)) != cudaSuccess)
        return cuda_error(ctx, e, "tcym_lattice_snapshot");
    SnapHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.header_bytes = (uint32_t)kHeaderBytes;
    h.nc = lat->nc; h.precision = lat->precision; h.fmt = lat->fmt;
    h.nx = lat->g.nx; h.ny = lat->g.ny; h.nz = lat->g.nz;
    for (int i = 0; i < 3; ++i) h.a[i] = lat->a[i];
    h.cur = lat->cur;
    h.reunit_period = lat->reunit_period;
    h.steps_since_reunit = lat->steps_since_reunit;
    h.ncs_every = lat->ncs_every;
    h.steps_done = lat->steps_done;
    h.noise_seed = lat->noise_seed;
    h.noise_next = lat->noise_next;
    h.noise_valid = lat->noise_valid ? 1u : 0u;
    h.ncs = res[R_NCS];
    h.ncs_comp = res[R_NCS_COMP];
    h.nonfinite = res[R_NONFINITE];
    h.link_payload = lb;
    h.field_payload = fb;
    h.checksum = payload_checksum(out + kHeaderBytes, lb + fb, 0x6A09E667F3BCC908ull);
    std::memset(out, 0, kHeaderBytes);
    std::memcpy(out, &h, sizeof(h));
    return TCYM_OK;
}

extern "C" int tcym_lattice_restore(tcym_lattice lat, const void *buf, size_t bytes) {
    TCYM_RANGE("tcym_lattice_restore");
    if (!lat || !buf) return TCYM_ERR_ARG;
    tcym_ctx ctx = lat->ctx;
    if (bytes < kHeaderBytes) {
        tcym_set_error(ctx, "tcym_lattice_restore: %zu bytes is shorter than a snapshot header", bytes);
        return TCYM_ERR_ARG;
    }
    const unsigned char *in = static_cast<const unsigned char *>(buf);
    SnapHeader h;
    std::memcpy(&h, in, sizeof(h));
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion || h.header_bytes != kHeaderBytes) {
        tcym_set_error(ctx, "tcym_lattice_restore: not a version-%u lattice snapshot", kVersion);
        return TCYM_ERR_ARG;
    }
    if (h.nc != lat->nc || h.precision != lat->precision || h.nx != lat->g.nx || h.ny != lat->g.ny ||
        h.nz != lat->g.nz) {
        tcym_set_error(ctx, "tcym_lattice_restore: snapshot of SU(%d) %dx%dx%d precision %d, lattice SU(%d) %dx%dx%d "
                            "precision %d",
                       h.nc, h.nx, h.ny, h.nz, h.precision, lat->nc, lat->g.nx, lat->g.ny, lat->g.nz,
                       lat->precision);
        return TCYM_ERR_ARG;
    }
    const size_t lb = link_payload(lat), fb = field_payload(lat);
    if (h.link_payload != lb || h.field_payload != fb || bytes < kHeaderBytes + lb + fb) {
        tcym_set_error(ctx, "tcym_lattice_restore: truncated snapshot (%zu bytes, %zu expected)", bytes,
                       kHeaderBytes + lb + fb);
        return TCYM_ERR_ARG;
    }
    if (payload_checksum(in + kHeaderBytes, lb + fb, 0x6A09E667F3BCC908ull) != h.checksum) {
        tcym_set_error(ctx, "tcym_lattice_restore: payload checksum mismatch (corrupt snapshot)");
        return TCYM_ERR_ARG;
    }
    if (h.cur != 0 && h.cur != 1) {
        tcym_set_error(ctx, "tcym_lattice_restore: bad ping-pong parity %d", h.cur);
        return TCYM_ERR_ARG;
    }
    cudaSetDevice(ctx->device);
    // the state goes to the buffer of the saved parity; the Kahan pair and the
    // non-finite flag back into the result block
    double res[R_WIDTH];
    cudaError_t e;
    if ((e = cudaMemcpyAsync(res, lat->result, sizeof(res), cudaMemcpyDeviceToHost, lat->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(lat->stream)) != cudaSuccess)
        return cuda_error(ctx, e, "tcym_lattice_restore");
    res[R_NCS] = h.ncs;
    res[R_NCS_COMP] = h.ncs_comp;
    res[R_NONFINITE] = h.nonfinite;
    if ((e = cudaMemcpyAsync(lat->U[h.cur], in + kHeaderBytes, lb, cudaMemcpyHostToDevice, lat->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(lat->E, in + kHeaderBytes + lb, fb, cudaMemcpyHostToDevice, lat->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(lat->result, res, sizeof(res), cudaMemcpyHostToDevice, lat->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(lat->stream)) != cudaSuccess)
        return cuda_error(ctx, e, "tcym_lattice_restore");
    lat->cur = h.cur;
    for (int i = 0; i < 3; ++i) lat->a[i] = h.a[i];
    lat->reunit_period = h.reunit_period;
    lat->steps_since_reunit = h.steps_since_reunit;
    lat->ncs_every = h.ncs_every;
    lat->steps_done = h.steps_done;
    lat->noise_seed = h.noise_seed;
    lat->noise_next = h.noise_next;
    lat->noise_valid = h.noise_valid != 0;
    return TCYM_OK;
}

extern "C" int tcym_lattice_noise_state(tcym_lattice lat, uint64_t *seed, uint64_t *next_step, int *valid) {
    if (!lat) return TCYM_ERR_ARG;
    if (seed) *seed = lat->noise_seed;
    if (next_step) *next_step = lat->noise_next;
    if (valid) *valid = lat->noise_valid ? 1 : 0;
    return TCYM_OK;
}

extern "C" int tcym_lattice_steps(tcym_lattice lat, int64_t *steps) {
    if (!lat || !steps) return TCYM_ERR_ARG;
    *steps = lat->steps_done;
    return TCYM_OK;
}

extern "C" int tcym_lattice_snapshot_file(tcym_lattice lat, const char *path) {
    if (!lat || !path) return TCYM_ERR_ARG;
    size_t n = 0;
    int r = tcym_lattice_snapshot_bytes(lat, &n);
    if (r) return r;
    void *buf = nullptr;
    // page-locked staging so the device-to-host copies run at full rate
    if (cudaMallocHost(&buf, n) != cudaSuccess) {
        tcym_set_error(lat->ctx, "tcym_lattice_snapshot_file: cannot allocate %zu bytes of host staging", n);
        return TCYM_ERR_OOM;
    }
    r = tcym_lattice_snapshot(lat, buf, n);
    if (r == TCYM_OK) {
        FILE *f = std::fopen(path, "wb");
        if (!f || std::fwrite(buf, 1, n, f) != n) {
            tcym_set_error(lat->ctx, "tcym_lattice_snapshot_file: cannot write %s", path);
            r = TCYM_ERR_ARG;
        }
        if (f && std::fclose(f) != 0 && r == TCYM_OK) {
            tcym_set_error(lat->ctx, "tcym_lattice_snapshot_file: cannot close %s", path);
            r = TCYM_ERR_ARG;
        }
    }
    cudaFreeHost(buf);
    return r;
}

extern "C" int tcym_lattice_restore_file(tcym_lattice lat, const char *path) {
    if (!lat || !path) return TCYM_ERR_ARG;
    size_t n = 0;
    int r = tcym_lattice_snapshot_bytes(lat, &n);
    if (r) return r;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        tcym_set_error(lat->ctx, "tcym_lattice_restore_file: cannot open %s", path);
        return TCYM_ERR_ARG;
    }
    void *buf = nullptr;
    if (cudaMallocHost(&buf, n) != cudaSuccess) {
        std::fclose(f);
        tcym_set_error(lat->ctx, "tcym_lattice_restore_file: cannot allocate %zu bytes of host staging", n);
        return TCYM_ERR_OOM;
    }
    const size_t got = std::fread(buf, 1, n, f);
    std::fclose(f);
    r = tcym_lattice_restore(lat, buf, got);
    cudaFreeHost(buf);
    return r;
}
