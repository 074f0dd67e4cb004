// Cooled real-time Chern-Simons number: ChernSimonsNumber::CoolingMethod
// (TOPOLOGY/CoolingMethod.cpp) at any standard blocking level.
//
// The object keeps UOld and UNew (the last two cooled configurations, Init
// :19-32), at the caller's extents divided by 2^level, and a scratch lattice
// of that size holding UMid/EMid of the geodesic between them.  Cooling
// (Cooling::CoolNSave and Perform, GRADIENTFLOW/Cooling.cpp:69-175) copies the
// caller's links, sets E to zero and runs max_steps simultaneous flow steps
// (GradientFlow::StandardUpdate, GradientFlow.cpp:150-165) through tcym_flow;
// with blocking, the b-th Block of links and fields (Cooling.cpp:123-143)
// comes after step block_frequency * 8^b, onto a lattice of half the extents
// and twice the spacings, until the level is reached.  Each flow step has
// DcTau = sqrt_dctau^2 (a_x a_y a_z)^(2/3) of the lattice it runs on
// (GradientFlow.cpp:150).  The geodesic (SUNc/AdvancedOperations.cpp:432-442)
// runs per link in FP64 (k_geodesic), and NCsDot = improved E.B / (8 pi^2)
// (ChernSimonsDerivative.cpp:31-49) through tcym_edotb_improved, so every
// reduction is the library's fixed-order FP64 one.  EMid's conversion to
// field units (cE_mu = a^3 / a_mu^2, CoolingMethod.cpp:39-45) and E.B's
// weights (cS_mu = a_mu^2 / a^3, ChernSimonsOperators.cpp:91-95) multiply to
// one, so neither is applied at any spacing.
#include <cmath>
#include <new>
#include <utility>
#include <vector>

#include "../../include/tcym.h"
#include "tcym_batch.cuh"
#include "tcym_internal.h"

using namespace tcym;

struct tcym_cooling_s {
    tcym_lattice hot = nullptr;
    tcym_lattice uold = nullptr, unew = nullptr, mid = nullptr;
    // blocking: work[b] holds the cooled links at blocking number b < level
    // (work[0] the caller's extents); the last Block writes into unew
    static constexpr int kMaxLevel = 8;
    tcym_lattice work[kMaxLevel] = {};
    int level = 0, block_frequency = 0;
    int max_steps = 0;
    double sqrt_dctau = 0.0;
    double real_time = 0.0;  // DeltaNCsCoolRealTime
    bool started = false;
};

namespace {

#define CKC(ctx, x)                                                  \
    do {                                                             \
        cudaError_t e_ = (x);                                        \
        if (e_ != cudaSuccess) {                                     \
            tcym_set_error(ctx, "%s: %s", #x, cudaGetErrorString(e_)); \
            return TCYM_ERR_CUDA;                                    \
        }                                                            \
    } while (0)

size_t link_bytes(tcym_lattice l) { return 3 * tcym_link_bytes(l->fmt) * tcym_stored_sites(l->fmt, l->g.V); }
size_t field_bytes(tcym_lattice l) { return 3 * tcym_field_bytes(l->fmt) * tcym_stored_sites(l->fmt, l->g.V); }

// the current links of src into the current link buffer of dst (same format and extents)
int copy_links(tcym_lattice dst, tcym_lattice src) {
    CKC(dst->ctx, cudaStreamSynchronize(src->stream));
    CKC(dst->ctx, cudaMemcpyAsync(dst->U[dst->cur], src->U[src->cur], link_bytes(dst), cudaMemcpyDeviceToDevice,
                                  dst->stream));
    return TCYM_OK;
}

// GradientFlow's DcTau on lattice l (GradientFlow.cpp:150, aScale = 1)
double dctau(tcym_cooling c, tcym_lattice l) {
    return c->sqrt_dctau * c->sqrt_dctau * std::cbrt(l->a[0] * l->a[1] * l->a[2] * l->a[0] * l->a[1] * l->a[2]);
}

// Cooling::CoolNSave: UNew = the hot links cooled from E = 0 with level Blocks
// (Perform, Cooling.cpp:69-143: the b-th after step block_frequency 8^b)
int cool(tcym_cooling c) {
    tcym_lattice cur = c->level ? c->work[0] : c->unew;
    int r = copy_links(cur, c->hot);
    if (r) return r;
    CKC(c->hot->ctx, cudaMemsetAsync(cur->E, 0, field_bytes(cur), cur->stream));
    double unused = 0.0;
    int steps = 0;
    for (int b = 0;; ++b) {
        // flow up to the next Block, or to the end
        const int upto = b < c->level ? c->block_frequency << (3 * b) : c->max_steps;
        if ((r = tcym_flow(cur, dctau(c, cur), upto - steps, TCYM_FLOW_SIMULTANEOUS, 0, &unused))) return r;
        steps = upto;
        if (b == c->level) return TCYM_OK;
        tcym_lattice next = b + 1 < c->level ? c->work[b + 1] : c->unew;
        if ((r = tcym_lattice_block(cur, next))) return r;
        cur = next;
    }
}

int ncs_dot(tcym_lattice l, double *out) {
    double edb = 0.0;
    int r = tcym_edotb_improved(l, &edb);
    if (r) return r;
    *out = 0.125 * edb / (M_PI * M_PI);
    return TCYM_OK;
}

template <int FMT> cudaError_t launch_geodesic(tcym_cooling c, double x) {
    tcym_lattice m = c->mid;
    return Launch<FMT>::geodesic(m->g, c->uold->U[c->uold->cur], c->unew->U[c->unew->cur], x, m->U[m->cur], m->E,
                                 m->stream);
}

// UMid, EMid at geodesic position x in [0, 1]
int geodesic(tcym_cooling c, double x) {
    tcym_lattice m = c->mid;
    CKC(m->ctx, cudaStreamSynchronize(c->uold->stream));
    CKC(m->ctx, cudaStreamSynchronize(c->unew->stream));
    switch (m->fmt) {
        case FMT_SU2_F32: CKC(m->ctx, launch_geodesic<FMT_SU2_F32>(c, x)); break;
        case FMT_SU2_F64: CKC(m->ctx, launch_geodesic<FMT_SU2_F64>(c, x)); break;
        case FMT_SU3_F32: CKC(m->ctx, launch_geodesic<FMT_SU3_F32>(c, x)); break;
        default: CKC(m->ctx, launch_geodesic<FMT_SU3_F64>(c, x)); break;
    }
    return TCYM_OK;
}

// CoolingMethod::GetDeltaNCs(NOrder) (CoolingMethod.cpp:77-120): Simpson's rule on
// the geodesic UOld -> UNew; interior points ip / 2N with weights 2 + 2 (ip mod 2),
// end points with weight 1, all with the geodesic's field EMid.
int delta_ncs(tcym_cooling c, int norder, double *out) {
    double value = 0.0, weight = 0.0, v = 0.0;
    int r;
    for (int ip = 1; ip < 2 * norder; ++ip) {
        const double x = ip / (2.0 * norder), w = 2.0 + 2.0 * (ip % 2);
        if ((r = geodesic(c, x)) || (r = ncs_dot(c->mid, &v))) return r;
        value += w * v;
        weight += w;
    }
    if (norder == 0 && (r = geodesic(c, 0.5))) return r;
    if ((r = copy_links(c->mid, c->uold)) || (r = ncs_dot(c->mid, &v))) return r;
    value += v;
    if ((r = copy_links(c->mid, c->unew)) || (r = ncs_dot(c->mid, &v))) return r;
    value += v;
    weight += 2.0;
    *out = value / weight;
    return TCYM_OK;
}

}  // namespace

extern "C" int tcym_cooling_create_ex(tcym_lattice lat, int max_steps, double sqrt_dctau, int blocking_level,
                                      int block_frequency, tcym_cooling *out) {
    if (!lat || !out || max_steps < 0 || !(sqrt_dctau >= 0) || blocking_level < 0 ||
        blocking_level >= tcym_cooling_s::kMaxLevel)
        return TCYM_ERR_ARG;
    *out = nullptr;
    if (blocking_level > 0) {
        // every Block must fall within the cooling steps, on extents divisible by 2^level
        const int f = 1 << blocking_level;
        const long long last = block_frequency > 0 ? (long long)block_frequency << (3 * (blocking_level - 1)) : 0;
        if (block_frequency <= 0 || last > max_steps || lat->g.nx % f || lat->g.ny % f || lat->g.nz % f) {
            tcym_set_error(lat->ctx, "tcym_cooling_create_ex: blocking level %d needs extents divisible by %d and "
                                     "block_frequency * 8^(level-1) <= max_steps", blocking_level, f);
            return TCYM_ERR_ARG;
        }
    }
    tcym_cooling c = new (std::nothrow) tcym_cooling_s;
    if (!c) return TCYM_ERR_OOM;
    c->hot = lat;
    c->max_steps = max_steps;
    c->sqrt_dctau = sqrt_dctau;
    c->level = blocking_level;
    c->block_frequency = block_frequency;
    // UOld, UNew, UMid at the blocked extents (spacings are set by the Blocks); work lattices per level
    std::vector<std::pair<tcym_lattice *, int>> ls = {{&c->uold, blocking_level}, {&c->unew, blocking_level},
                                                      {&c->mid, blocking_level}};
    for (int b = 0; b < blocking_level; ++b) ls.push_back({&c->work[b], b});
    for (auto &[l, b] : ls) {
        double a[3];
        for (int i = 0; i < 3; ++i) a[i] = lat->a[i] * (1 << b);
        int r = tcym_lattice_create_ex(lat->ctx, lat->nc, lat->g.nx >> b, lat->g.ny >> b, lat->g.nz >> b, a,
                                       lat->precision, l);
        if (r) {
            tcym_cooling_destroy(c);
            return r;
        }
        (*l)->reunit_period = lat->reunit_period;
    }
    *out = c;
    return TCYM_OK;
}

extern "C" int tcym_cooling_create(tcym_lattice lat, int max_steps, double sqrt_dctau, tcym_cooling *out) {
    return tcym_cooling_create_ex(lat, max_steps, sqrt_dctau, 0, 0, out);
}

extern "C" int tcym_cooling_destroy(tcym_cooling c) {
    if (!c) return TCYM_ERR_ARG;
    if (c->uold) tcym_lattice_destroy(c->uold);
    if (c->unew) tcym_lattice_destroy(c->unew);
    if (c->mid) tcym_lattice_destroy(c->mid);
    for (tcym_lattice w : c->work)
        if (w) tcym_lattice_destroy(w);
    delete c;
    return TCYM_OK;
}

// CoolingMethod::Start (:124-135)
extern "C" int tcym_cooling_start(tcym_cooling c) {
    if (!c) return TCYM_ERR_ARG;
    cudaSetDevice(c->hot->ctx->device);
    int r = cool(c);
    if (r || (r = copy_links(c->uold, c->unew))) return r;
    CKC(c->hot->ctx, cudaStreamSynchronize(c->uold->stream));
    c->started = true;
    return TCYM_OK;
}

// CoolingMethod::Update(Measure) (:141-166)
extern "C" int tcym_cooling_update(tcym_cooling c, int measure, double *delta) {
    TCYM_RANGE("tcym_cooling_update");
    if (!c) return TCYM_ERR_ARG;
    if (!c->started) {
        tcym_set_error(c->hot->ctx, "tcym_cooling_update: call tcym_cooling_start first");
        return TCYM_ERR_STATE;
    }
    cudaSetDevice(c->hot->ctx->device);
    int r = cool(c);
    if (r) return r;
    double d = 0.0;
    if (measure) {
        if ((r = delta_ncs(c, 1, &d))) return r;
        c->real_time += d;
    }
    if (delta) *delta = d;
    if ((r = copy_links(c->uold, c->unew))) return r;
    CKC(c->hot->ctx, cudaStreamSynchronize(c->uold->stream));
    return TCYM_OK;
}

extern "C" int tcym_cooling_delta_ncs(tcym_cooling c, int norder, double *out) {
    if (!c || !out || norder < 0) return TCYM_ERR_ARG;
    if (!c->started) return TCYM_ERR_STATE;
    cudaSetDevice(c->hot->ctx->device);
    return delta_ncs(c, norder, out);
}

// the cooled links UOld (after start / update: the latest cooled copy) in the
// reference's AoS layout, on the extents divided by 2^level
extern "C" int tcym_cooling_links(tcym_cooling c, double *U_aos) {
    if (!c || !U_aos) return TCYM_ERR_ARG;
    if (!c->started) return TCYM_ERR_STATE;
    return tcym_lattice_download(c->uold, U_aos, nullptr);
}

extern "C" int tcym_cooling_total(tcym_cooling c, double *out) {
    if (!c || !out) return TCYM_ERR_ARG;
    *out = c->real_time;
    return TCYM_OK;
}
