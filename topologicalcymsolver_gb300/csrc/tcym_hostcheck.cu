// TEST-ONLY host build of the per-site device code (not part of libtcym.so).
//
// Compiled by nvcc for the host only (no kernels), it runs the exact
// __host__ __device__ site functions the CUDA kernels call, in a loop over
// sites, on host arrays in the device storage layout.  tests/ use it to check
// the device arithmetic (both FP64 and FP32 formats) against the FP64 oracle
// on machines without a GPU.
#include <cstdint>
#include <cstring>
#include <vector>

#include "tcym_pipeline.h"
#include "tcym_site.cuh"

using namespace tcym;

namespace {

StepCoef<double> coef(int mode, double dt, double gamma, double T, uint64_t seed, uint64_t step) {
    // unit spacings (the same folding as tcym_coef in tcym_capi.cu)
    StepCoef<double> c;
    std::memset(&c, 0, sizeof(c));
    c.mode = mode;
    c.seed = seed;
    c.step = step;
    for (int mu = 0; mu < 3; ++mu) {
        c.fc[mu] = mode == MODE_FLOW ? -2.0 : -2.0 * dt;
        c.cnu[mu] = 1.0;
        c.uc[mu] = -dt;
        if (mode == MODE_LANGEVIN) {
            c.damp[mu] = gamma * dt;
            c.kick[mu] = std::sqrt(gamma) * std::sqrt(dt) * std::sqrt(2.0 * T);
        }
    }
    return c;
}

template <class T> StepCoef<T> cast(const StepCoef<double> &c) {
    StepCoef<T> r;
    r.mode = c.mode; r.seed = c.seed; r.step = c.step;
    for (int i = 0; i < 3; ++i) {
        r.fc[i] = (T)c.fc[i]; r.cnu[i] = (T)c.cnu[i]; r.uc[i] = (T)c.uc[i];
        r.damp[i] = (T)c.damp[i]; r.kick[i] = (T)c.kick[i];
    }
    return r;
}

template <int FMT> struct H {
    using F = Fmt<FMT>;
    using T = typename F::T;
    // pairs: 0 per-site step; 1 + tx: the paired step with tiling tx (0: linear)
    static void step(const Geom &g, const void *Uin, void *Uout, void *E, const StepCoef<double> &cd, int doE,
                     int doU, int pairs) {
        StepCoef<T> c = cast<T>(cd);
        if constexpr (F::PAIRED) {
            // the device's paired step, block by block and thread by thread as the kernel runs it
            if (pairs && doE && doU && g.nz % 2 == 0) {
                const Tile t = make_tile(g, pairs - 1);
                for (int64_t b = 0; b < tile_blocks(g, t); ++b)
                    for (int tid = 0; tid < 128; ++tid) {
                        int64_t p;
                        bool seam;
                        if (!tile_pair(g, t, b, tid, p, seam)) continue;
                        f2 sm[3 * F::NA];
                        if (seam) site_step_pair<F, true>(g, Uin, Uout, E, c, p, 0, sm, 1);
                        else site_step_pair<F, false>(g, Uin, Uout, E, c, p, 0, sm, 1);
                    }
                return;
            }
        }
        for (int64_t s = 0; s < g.V; ++s) {
            T sm[3 * F::NA];
            if (doE && doU) site_step<F, true, true>(g, Uin, Uout, E, c, s, 0, sm, 1);
            else if (doE) site_step<F, true, false>(g, Uin, Uout, E, c, s, 0, sm, 1);
            else site_step<F, false, true>(g, Uin, Uout, E, c, s, 0, sm, 1);
        }
    }
    // one fused step of the storage indices [i0, i1) as Launch::step_range runs it: the
    // paired step's linear blocks from block i0 / 128 (Tile::b0), or sites
    static void step_range(const Geom &g, const void *Uin, void *Uout, void *E, const StepCoef<double> &cd,
                           int64_t i0, int64_t i1) {
        StepCoef<T> c = cast<T>(cd);
        if constexpr (F::PAIRED) {
            if (g.nz % 2 == 0) {
                const Tile t{0, 0, 0, 0, 0, (int)(i0 / 128)};
                for (int64_t b = 0; b < (i1 - i0 + 127) / 128; ++b)
                    for (int tid = 0; tid < 128; ++tid) {
                        int64_t p;
                        bool seam;
                        if (!tile_pair(g, t, b, tid, p, seam)) continue;
                        f2 sm[3 * F::NA];
                        if (seam) site_step_pair<F, true>(g, Uin, Uout, E, c, p, 0, sm, 1);
                        else site_step_pair<F, false>(g, Uin, Uout, E, c, p, 0, sm, 1);
                    }
                return;
            }
        }
        for (int64_t s = i0; s < i1; ++s) {
            T sm[3 * F::NA];
            site_step<F, true, true>(g, Uin, Uout, E, c, s, 0, sm, 1);
        }
    }
    static void flow_cb(const Geom &g, void *U, double dtau, int nsweeps) {
        const T fc[3] = {T(-2), T(-2), T(-2)}, cn[3] = {T(1), T(1), T(1)}, uc[3] = {T(-dtau), T(-dtau), T(-dtau)};
        for (int sw = 0; sw < nsweeps; ++sw)
            for (int p = 0; p < 2; ++p)
                for (int mu = 0; mu < 3; ++mu)
                    for (int64_t s = 0; s < g.V; ++s) {
                        Nbhd nb(g, s);
                        if (nb.parity() == p) link_flow<F>(g, U, mu, fc, cn, uc, s);
                    }
    }
    static void observables(const Geom &g, const void *U, const void *E, int mask, double *out) {
        double esq[3] = {0, 0, 0}, bsq[3] = {0, 0, 0}, gsq = 0, usq = 0, edb = 0, gmax = 0, gabs = 0, umax = 0;
        for (int64_t s = 0; s < g.V; ++s) {
            SiteObs<F> o;
            site_observables<F>(g, U, E, mask, s, o);
            for (int m = 0; m < 3; ++m) { esq[m] += o.esq[m]; bsq[m] += o.bsq[m]; usq += o.un[m] * o.un[m]; umax = std::fmax(umax, o.un[m]); }
            for (int a = 0; a < F::NA; ++a) { gsq += o.g[a] * o.g[a]; gmax = std::fmax(gmax, o.g[a]); gabs = std::fmax(gabs, std::fabs(o.g[a])); }
            edb += o.edotb;
        }
        const double V = (double)g.V;
        for (int m = 0; m < 3; ++m) { out[3 + m] = esq[m] / V; out[6 + m] = bsq[m] / V; }
        out[1] = 0.5 * (out[3] + out[4] + out[5]);
        out[2] = 0.5 * (out[6] + out[7] + out[8]);
        out[0] = out[1] + out[2];
        out[9] = gmax;
        out[10] = std::sqrt(gsq / (F::NA * V));
        out[11] = umax;
        out[12] = std::sqrt(usq / (3 * V));
        out[13] = edb;
        out[14] = 0;
        out[15] = gabs;
    }
    // the N_CS sample through the paired code (FP32 pair storage, even nz): the
    // E^2, plaquette B^2 and clover E.B slots of observables(); false if not paired
    static bool edotb_pair(const Geom &g, const void *U, const void *E, double *out) {
        if constexpr (F::PAIRED) {
            if (g.nz % 2) return false;
            double esq[3] = {0, 0, 0}, bsq[3] = {0, 0, 0}, edb = 0;
            const int64_t Vh = g.V >> 1, plane = (int64_t)g.nx * g.ny;
            for (int64_t p = 0; p < Vh; ++p)
                for (int mu = 0; mu < 3; ++mu) {
                    f2 e2, b2;
                    const f2 d = (p < plane || p >= Vh - plane) ? pair_edotb_obs<F, true>(g, U, E, p, mu, e2, b2)
                                                                : pair_edotb_obs<F, false>(g, U, E, p, mu, e2, b2);
                    esq[mu] += (double)e2.v.x + (double)e2.v.y;
                    bsq[mu] += (double)b2.v.x + (double)b2.v.y;
                    edb += (double)d.v.x + (double)d.v.y;
                }
            const double V = (double)g.V;
            for (int k = 0; k < 16; ++k) out[k] = 0;
            for (int m = 0; m < 3; ++m) { out[3 + m] = esq[m] / V; out[6 + m] = bsq[m] / V; }
            out[1] = 0.5 * (out[3] + out[4] + out[5]);
            out[2] = 0.5 * (out[6] + out[7] + out[8]);
            out[0] = out[1] + out[2];
            out[13] = edb;
            return true;
        }
        return false;
    }
    static void iexp_aos(double c, const double *alpha, double *out) {
        T e[F::NA];
        for (int a = 0; a < F::NA; ++a) e[a] = (T)alpha[a];
        auto m = F::G::iexp((T)c, e);
        if constexpr (F::NA == 3) {
            for (int k = 0; k < 4; ++k) out[k] = (double)m.q[k];
        } else {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    out[2 * (i + 3 * j)] = (double)m.m[i][j].re;
                    out[2 * (i + 3 * j) + 1] = (double)m.m[i][j].im;
                }
        }
    }
    // A with exp(i c A^a t^a) = V, V given in the reference AoS link layout
    static void ilog_aos(double c, const double *v, double *out) {
        typename F::G::Mat m;
        if constexpr (F::NA == 3) {
            for (int k = 0; k < 4; ++k) m.q[k] = (T)v[k];
        } else {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) m.m[i][j] = cx<T>{(T)v[2 * (i + 3 * j)], (T)v[2 * (i + 3 * j) + 1]};
        }
        T o[F::NA];
        F::G::ilog((T)c, m, o);
        for (int a = 0; a < F::NA; ++a) out[a] = (double)o[a];
    }
    static void geodesic(const Geom &g, const void *Uold, const void *Unew, double c, void *Umid, void *Emid) {
        for (int64_t s = 0; s < g.V; ++s) site_geodesic<F>(g, Uold, Unew, c, Umid, Emid, s);
    }
    static int gauss_restore(const Geom &g, const void *U, void *E, double tol, int maxit) {
        std::vector<double> G((size_t)F::NA * g.V);
        const double gam[3] = {7.0 / 24.0, 7.0 / 48.0, 7.0 / 72.0};
        auto dev = [&]() {
            double m = 0;
            for (int64_t s = 0; s < g.V; ++s) {
                double gv[F::NA];
                site_gauss<F>(g, U, E, s, gv);
                for (int a = 0; a < F::NA; ++a) { G[a * g.V + s] = gv[a]; m = std::fmax(m, gv[a]); }
            }
            return m;
        };
        double gmax = dev();
        int it = 0;
        while (it < maxit && gmax > tol) {
            for (int k = 0; k < 3; ++k) {
                gmax = dev();
                for (int64_t s = 0; s < g.V; ++s) site_gauss_update<F>(g, U, E, G.data(), gam[k], s);
            }
            ++it;
        }
        return it;
    }
};

Geom geom(const int *n) { return Geom{n[0], n[1], n[2], (int64_t)n[0] * n[1] * n[2]}; }

#define HC_DISPATCH(fmt, body)                                  \
    switch (fmt) {                                              \
        case FMT_SU2_F32: { using HH = H<FMT_SU2_F32>; body; } break; \
        case FMT_SU2_F64: { using HH = H<FMT_SU2_F64>; body; } break; \
        case FMT_SU3_F32: { using HH = H<FMT_SU3_F32>; body; } break; \
        case FMT_SU3_F64: { using HH = H<FMT_SU3_F64>; body; } break; \
        default: return -1;                                     \
    }

}  // namespace

extern "C" {

int hc_from_aos(int fmt, const int *n, const double *Ua, const double *Ea, void *U, void *E) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, for (int64_t s = 0; s < g.V; ++s) site_from_aos<HH::F>(g, U, E, Ua, Ea, s));
    return 0;
}
// sites [s0, s0 + cnt) of full AoS arrays into the storage
int hc_from_aos_range(int fmt, const int *n, const double *Ua, const double *Ea, void *U, void *E, int64_t s0,
                      int64_t cnt) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, for (int64_t s = s0; s < s0 + cnt; ++s) site_from_aos<HH::F>(g, U, E, Ua, Ea, s));
    return 0;
}
// one leapfrog step of the storage indices [i0, i1) (site pairs when the format pairs and nz is even)
int hc_step_range(int fmt, const int *n, const void *Uin, void *Uout, void *E, double dt, int64_t i0, int64_t i1) {
    Geom g = geom(n);
    StepCoef<double> c = coef(MODE_LEAPFROG, dt, 0, 0, 0, 0);
    HC_DISPATCH(fmt, HH::step_range(g, Uin, Uout, E, c, i0, i1));
    return 0;
}
int hc_to_aos(int fmt, const int *n, const void *U, const void *E, double *Ua, double *Ea) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, for (int64_t s = 0; s < g.V; ++s) site_to_aos<HH::F>(g, U, E, Ua, Ea, s));
    return 0;
}
// pairs: 0 the per-site step; 1 + tx: the paired step where the device takes it (FP32
// formats, even nz, fused step) with block tiling tx (0: linear)
int hc_step(int fmt, const int *n, const void *Uin, void *Uout, void *E, int mode, double dt, double gamma, double T,
            uint64_t seed, uint64_t step, int doE, int doU, int pairs) {
    Geom g = geom(n);
    StepCoef<double> c = coef(mode, dt, gamma, T, seed, step);
    HC_DISPATCH(fmt, HH::step(g, Uin, Uout, E, c, doE, doU, pairs));
    return 0;
}
int hc_flow_cb(int fmt, const int *n, void *U, double dtau, int nsweeps) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, HH::flow_cb(g, U, dtau, nsweeps));
    return 0;
}
int hc_observables(int fmt, const int *n, const void *U, const void *E, int mask, double *out) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, HH::observables(g, U, E, mask, out));
    return 0;
}
int hc_edotb_pair(int fmt, const int *n, const void *U, const void *E, double *out) {
    Geom g = geom(n);
    int ok = 0;
    HC_DISPATCH(fmt, ok = HH::edotb_pair(g, U, E, out));
    return ok;
}
int hc_gauss_restore(int fmt, const int *n, const void *U, void *E, double tol, int maxit) {
    Geom g = geom(n);
    int it = 0;
    HC_DISPATCH(fmt, it = HH::gauss_restore(g, U, E, tol, maxit));
    return it;
}
int hc_reunitarize(int fmt, const int *n, void *U) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, for (int64_t s = 0; s < g.V; ++s) site_reunitarize<HH::F>(g, U, s));
    return 0;
}
// Block of the links of extents n into Ub (extents n / 2, the same format)
int hc_block(int fmt, const int *n, const void *U, void *Ub) {
    const Geom gs = geom(n);
    const int h[3] = {n[0] / 2, n[1] / 2, n[2] / 2};
    const Geom gd = geom(h);
    HC_DISPATCH(fmt, for (int64_t s = 0; s < gd.V; ++s) site_block<HH::F>(gs, gd, U, Ub, s));
    return 0;
}
int hc_init(int fmt, const int *n, void *U, void *E, int what, double sigma, uint64_t seed) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, for (int64_t s = 0; s < g.V; ++s) {
        if (what == 0) site_set_zero<HH::F>(g, U, E, s);
        else if (what == 1) site_gaussian_efield<HH::F>(g, E, sigma, seed, s);
        else site_random_links<HH::F>(g, U, sigma, seed, s);
    });
    return 0;
}
int hc_ilog(int fmt, double c, const double *v, double *out) {
    HC_DISPATCH(fmt, HH::ilog_aos(c, v, out));
    return 0;
}
int hc_geodesic(int fmt, const int *n, const void *Uold, const void *Unew, double c, void *Umid, void *Emid) {
    Geom g = geom(n);
    HC_DISPATCH(fmt, HH::geodesic(g, Uold, Unew, c, Umid, Emid));
    return 0;
}
// exp(i c t^a alpha^a) in the format's precision, returned in the reference AoS link layout
int hc_iexp(int fmt, double c, const double *alpha, double *out) {
    HC_DISPATCH(fmt, HH::iexp_aos(c, alpha, out));
    return 0;
}
// the host-resident step's pipeline for N units in planes of P, chunk size C:
// its chunk bounds (at most cap written) and the issue order, kinds[i] (0
// upload, 1 step) of chunks[i]; returns the number of operations
int64_t hc_pipeline_schedule(int64_t N, int64_t P, int64_t C, int64_t *bounds, int64_t bcap, int *kinds,
                             int64_t *chunks, int64_t cap) {
    const std::vector<int64_t> b = pipeline_bounds(N, P, C);
    for (int64_t i = 0; i < (int64_t)b.size() && i < bcap; ++i) bounds[i] = b[i];
    int64_t n = 0;
    pipeline_schedule(b, P, [&](int op, int64_t j) {
        if (n < cap) { kinds[n] = op; chunks[n] = j; }
        ++n;
    });
    return n;
}
double hc_normal(uint64_t seed, uint32_t stream, uint64_t step, uint32_t site, uint32_t mu, uint32_t a, int single) {
    double z0, z1;
    if (single) {
        float f0, f1;
        normal_pair<float>(seed, stream, step, site, mu, a >> 1, &f0, &f1);
        z0 = f0; z1 = f1;
    } else {
        normal_pair<double>(seed, stream, step, site, mu, a >> 1, &z0, &z1);
    }
    return (a & 1) ? z1 : z0;
}

}  // extern "C"
