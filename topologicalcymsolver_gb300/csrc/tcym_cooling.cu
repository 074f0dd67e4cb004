// Cooled real-time Chern-Simons number: ChernSimonsNumber::CoolingMethod
// (TOPOLOGY/CoolingMethod.cpp) at blocking level 0, the level its real-time
// measurement runs at (StandardBlockingLevel, SphaleronSimulation.cpp:236).
//
// The object keeps three lattices of the caller's format and extents: UOld
// and UNew (the last two cooled configurations, Init :19-32) and a scratch
// lattice holding UMid/EMid of the geodesic between them.  Cooling
// (Cooling::CoolNSave, GRADIENTFLOW/Cooling.cpp:156-175) copies the caller's
// links into UNew, sets its E to zero and runs max_steps simultaneous flow
// steps of dtau = sqrt_dctau^2 (GradientFlow::StandardUpdate,
// GradientFlow.cpp:150-165) through tcym_flow.  The geodesic
// (SUNc/AdvancedOperations.cpp:432-442) runs per link in FP64 (k_geodesic), and
// NCsDot = improved E.B / (8 pi^2) (ChernSimonsDerivative.cpp:31-49) through
// tcym_edotb_improved, so every reduction is the library's fixed-order FP64 one.
#include <cmath>
#include <new>

#include "../../include/tcym.h"
#include "tcym_batch.cuh"
#include "tcym_internal.h"

using namespace tcym;

struct tcym_cooling_s {
    tcym_lattice hot = nullptr;
    tcym_lattice uold = nullptr, unew = nullptr, mid = nullptr;
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

// Cooling::CoolNSave at blocking level 0: UNew = the hot links cooled from E = 0
int cool(tcym_cooling c) {
    int r = copy_links(c->unew, c->hot);
    if (r) return r;
    CKC(c->hot->ctx, cudaMemsetAsync(c->unew->E, 0, field_bytes(c->unew), c->unew->stream));
    double unused = 0.0;
    return tcym_flow(c->unew, c->sqrt_dctau * c->sqrt_dctau, c->max_steps, TCYM_FLOW_SIMULTANEOUS, 0, &unused);
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

extern "C" int tcym_cooling_create(tcym_lattice lat, int max_steps, double sqrt_dctau, tcym_cooling *out) {
    if (!lat || !out || max_steps < 0 || !(sqrt_dctau >= 0)) return TCYM_ERR_ARG;
    *out = nullptr;
    tcym_cooling c = new (std::nothrow) tcym_cooling_s;
    if (!c) return TCYM_ERR_OOM;
    c->hot = lat;
    c->max_steps = max_steps;
    c->sqrt_dctau = sqrt_dctau;
    tcym_lattice *ls[3] = {&c->uold, &c->unew, &c->mid};
    for (tcym_lattice *l : ls) {
        int r = tcym_lattice_create_ex(lat->ctx, lat->nc, lat->g.nx, lat->g.ny, lat->g.nz, lat->a, lat->precision, l);
        if (r) {
            tcym_cooling_destroy(c);
            return r;
        }
        (*l)->reunit_period = lat->reunit_period;
    }
    *out = c;
    return TCYM_OK;
}

extern "C" int tcym_cooling_destroy(tcym_cooling c) {
    if (!c) return TCYM_ERR_ARG;
    if (c->uold) tcym_lattice_destroy(c->uold);
    if (c->unew) tcym_lattice_destroy(c->unew);
    if (c->mid) tcym_lattice_destroy(c->mid);
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

extern "C" int tcym_cooling_total(tcym_cooling c, double *out) {
    if (!c || !out) return TCYM_ERR_ARG;
    *out = c->real_time;
    return TCYM_OK;
}
