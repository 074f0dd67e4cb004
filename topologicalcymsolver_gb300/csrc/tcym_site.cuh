// Per-site work of every kernel, as __host__ __device__ functions of one site.
//
// A CUDA kernel maps one thread to one site and calls these; the test-only
// host build calls them in a loop over sites, so CPU tests see the exact
// arithmetic of the device path.
#pragma once

#include <type_traits>

#include "tcym_layout.cuh"
#include "tcym_rng.cuh"

namespace tcym {

// Step kinds: how the colour force f enters E before the link update.
enum StepMode : int {
    MODE_LEAPFROG = 0,  // E += fc f                              (Dynamics.cpp:184-188)
    MODE_LANGEVIN = 1,  // E += fc f - damp E + kick xi           (LangevinDynamics.cpp:222-234)
    MODE_FLOW = 2,      // E  = fc f  (the flow force, stored)    (GradientFlow.cpp:77-84)
};

// Coefficients of one step, per direction mu (metric factors of the reference
// folded in; for unit spacings: fc = -2 dt (leapfrog/Langevin) or -2 (flow),
// cnu = 1, uc = -dt or -dtau, damp = gamma dt, kick = sqrt(gamma dt) sqrt(2T)).
template <class T> struct StepCoef {
    int mode;
    T fc[3], cnu[3], uc[3], damp[3], kick[3];
    uint64_t seed, step;
};

// Staple sum around U_mu(x): A = sum_{nu != mu} cnu[nu] (S+ + S-) with
//   S+ = U_nu(x+mu) U_mu^dag(x+nu) U_nu^dag(x)        (upper staple)
//   S- = U_nu^dag(x+mu-nu) U_mu^dag(x-nu) U_nu(x-nu)  (lower staple)
// so that U_mu(x) S+ is the plaquette U_{mu nu}(x) of Plaquettes.cpp:28 and
// proj(U_mu S-) = -proj(U_{mu,-nu}(x)) (Plaquettes.cpp:30); the reference's
// bracket [c_nu1 (P_{mu nu1} - P_{mu,-nu1}) - c_nu2 (P_{nu2 mu} - P_{-nu2,mu})]
// (Dynamics.cpp:184-188) equals proj(U_mu A).
template <class F>
TCYM_HD typename F::Mat staple_sum(const void *U, int64_t V, const Nbhd &nb, int mu,
                                  const typename F::T (&cnu)[3]) {
    using G = typename F::G;
    using M = typename F::Mat;
    M A = G::zero();
#pragma unroll
    for (int k = 1; k <= 2; ++k) {
        const int nu = mu + k >= 3 ? mu + k - 3 : mu + k;
        // staples are group elements: mulu forms rows 0 and 1 and rebuilds row 2
        M a1 = F::load(U, V, nu, nb.at(mu, 1));
        M a2 = F::load(U, V, mu, nb.at(nu, 1));
        M a3 = F::load(U, V, nu, nb.s);
        M up = G::template mulu<false, true>(G::template mulu<false, true>(a1, a2), a3);
        M b1 = F::load(U, V, nu, nb.at(mu, 1, nu, -1));
        const int64_t sb = nb.at(nu, -1);
        M b2 = F::load(U, V, mu, sb);
        M b3 = F::load(U, V, nu, sb);
        M lo = G::template mulu<false, false>(G::template mulu<true, true>(b1, b2), b3);
        A = G::add(A, G::scale(sel3(cnu, nu), G::add(up, lo)));
    }
    return A;
}

// Sum of the lower staples around U_mu(x), sum_{nu != mu} cnu[nu] S-, S- as above.
template <class F>
TCYM_HD typename F::Mat lower_staple_sum(const void *U, int64_t V, const Nbhd &nb, int mu,
                                         const typename F::T (&cnu)[3]) {
    using G = typename F::G;
    using M = typename F::Mat;
    M A = G::zero();
#pragma unroll
    for (int k = 1; k <= 2; ++k) {
        const int nu = mu + k >= 3 ? mu + k - 3 : mu + k;
        M b1 = F::load(U, V, nu, nb.at(mu, 1, nu, -1));
        const int64_t sb = nb.at(nu, -1);
        M b2 = F::load(U, V, mu, sb);
        M b3 = F::load(U, V, nu, sb);
        M lo = G::template mulu<false, false>(G::template mulu<true, true>(b1, b2), b3);
        A = G::add(A, G::scale(sel3(cnu, nu), lo));
    }
    return A;
}

// the group arithmetic of a format in the working type T: packed pairs (f2) or scalars
template <class F, class T, bool PACKED = std::is_same<T, f2>::value> struct GroupOf { using type = typename F::G; };
template <class F, class T> struct GroupOf<F, T, true> { using type = typename F::G2; };

// The step's force with the plaquettes shared between directions.  The force on
// U_mu(x) sums, over nu != mu, the projections of the plaquette above the link
// (corner x) and of the one below it (corner x - nu).  The plaquette above is
// P_{mu nu}(x) = U_mu(x) S+_{mu nu}, and P_{nu mu}(x) = P_{mu nu}(x)^dag, whose
// projection is the negative, so the upper staples of all six (mu, nu) come from
// the three plaquettes P_01, P_12, P_20 at x, each formed once:
//   f_mu = c_{mu+1} p_{mu,mu+1} - c_{mu+2} p_{mu+2,mu} + proj(U_mu sum_nu c_nu S-_{mu nu})
// with p_{mu nu} = proj(P_{mu nu}(x)).  That is the reference's bracket
// (Dynamics.cpp:184-188) in the staple form above, with 18 instead of 24 SU(3)
// products per site.  plaquette_projections writes p_01, p_12, p_20 to
// sm[(k * NA + a) * stride], the caller's slots for this site (shared memory
// on the device), where the per-direction phase reads them back.
template <class F, class M, class T, class LOAD>
TCYM_HD void plaquette_projections(LOAD load, T *sm, int stride) {
    using G = typename GroupOf<F, T>::type;
#pragma unroll 1
    for (int mu = 0; mu < 3; ++mu) {
        const int nu = mu == 2 ? 0 : mu + 1;
        // P_{mu nu}(x) = [U_mu(x) U_nu(x+mu)] [U_nu(x) U_mu(x+nu)]^dag
        const M t1 = G::template mulu<false, false>(load(mu, 0, mu), load(nu, 1, mu));
        const M t2 = G::template mulu<false, false>(load(nu, 0, mu), load(mu, 1, nu));
        T pr[F::NA];
        G::proj_mul_dag(t1, t2, pr);
#pragma unroll
        for (int a = 0; a < F::NA; ++a) sm[(mu * F::NA + a) * stride] = pr[a];
    }
}
// f[a] += c_{mu+1} p_{mu,mu+1} - c_{mu+2} p_{mu+2,mu}
template <int NA, class T, class C>
TCYM_HD void add_plaquette_force(const T *sm, int stride, int mu, const C (&cnu)[3], T *f) {
    const int n1 = mu == 2 ? 0 : mu + 1, n2 = mu == 0 ? 2 : mu - 1;
    const T cp(sel3(cnu, n1)), cm(sel3(cnu, n2));
#pragma unroll
    for (int a = 0; a < NA; ++a) f[a] = fma(cp, sm[(mu * NA + a) * stride], fma(-cm, sm[(n2 * NA + a) * stride], f[a]));
}

// One site of a step.  DO_E: compute the force and update E; DO_U: move the
// links by exp(i uc E) and write them to Uout (Uout may alias Uin only when
// DO_E is false, i.e. for the pointwise link update).  sm: 3 * NA slots of T
// for this site, stride apart (used when DO_E).
template <class F, bool DO_E, bool DO_U>
TCYM_HD void site_step(const Geom &g, const void *Uin, void *Uout, void *E, const StepCoef<typename F::T> &c,
                       int64_t s, uint64_t step_add, typename F::T *sm, int stride) {
    using G = typename F::G;
    using T = typename F::T;
    using M = typename F::Mat;
    constexpr int NA = F::NA;
    const int64_t V = g.V;
    Nbhd nb(g, s);
    if (DO_E) {
        // link along d at x (a = 0) or at x + e_dir (a = 1)
        auto load = [&](int d, int a, int dir) { return F::load(Uin, V, d, a ? nb.at(dir, 1) : s); };
        plaquette_projections<F, M>(load, sm, stride);
    }
#pragma unroll 1
    for (int mu = 0; mu < 3; ++mu) {
        T e[NA];
        M u;
        if (DO_E) {
            const M A = lower_staple_sum<F>(Uin, V, nb, mu, c.cnu);
            u = F::load(Uin, V, mu, s);
            F::load_e(E, V, mu, s, e);
            T f[NA];
            G::proj_mul(u, A, f);
            add_plaquette_force<NA>(sm, stride, mu, c.cnu, f);
            const T fc = sel3(c.fc, mu);
            if (c.mode == MODE_LANGEVIN) {
                T xi[NA];
                normals<T, NA>(c.seed, STREAM_NOISE, c.step + step_add, (uint32_t)s, (uint32_t)mu, xi);
                const T damp = sel3(c.damp, mu), kick = sel3(c.kick, mu);
#pragma unroll
                for (int a = 0; a < NA; ++a) e[a] = e[a] + (fc * f[a] - damp * e[a] + kick * xi[a]);
            } else if (c.mode == MODE_FLOW) {
#pragma unroll
                for (int a = 0; a < NA; ++a) e[a] = fc * f[a];
            } else {
#pragma unroll
                for (int a = 0; a < NA; ++a) e[a] = e[a] + fc * f[a];
            }
            F::store_e(E, V, mu, s, e);
        } else {
            u = F::load(Uin, V, mu, s);
            F::load_e(E, V, mu, s, e);
        }
        if (DO_U) {
            F::store(Uout, V, mu, s, G::iexp_mul(sel3(c.uc, mu), e, u));
        }
    }
}

// ------------------------------------------------------------------ site pairs
// E += fc f - damp E + kick xi for both sites of pair p (Philox noise of sites p, p + Vh)
template <int NA>
TCYM_COLD void langevin_kick_pair(const StepCoef<float> &c, int mu, int64_t p, int64_t Vh, uint64_t step_add, f2 fc,
                                  const f2 *f, f2 *e) {
    float x0[NA], x1[NA];
    normals<float, NA>(c.seed, STREAM_NOISE, c.step + step_add, (uint32_t)p, (uint32_t)mu, x0);
    normals<float, NA>(c.seed, STREAM_NOISE, c.step + step_add, (uint32_t)(p + Vh), (uint32_t)mu, x1);
    const f2 damp(sel3(c.damp, mu)), kick(sel3(c.kick, mu));
#pragma unroll
    for (int a = 0; a < NA; ++a) e[a] = e[a] + fma(kick, f2(x0[a], x1[a]), fma(-damp, e[a], fc * f[a]));
}

// site_step for both sites of pair p of an FP32 lattice with even nz, (x,y,z)
// and (x,y,z+nz/2), in packed FP32 (f2): the same plaquettes, staples,
// projections, E update and exponential per lane, at half the instructions.
// SEAM: the pair may touch the seam z = nz/2, across which neighbour pairs
// arrive with their lanes swapped; pairs away from it skip the swap tests.
// cn: the Langevin noise's coefficients (seed, step, damping, kick), which may
// sit apart from the step's (a batched member's own, beside coefficients the
// members share).  MODE >= 0 fixes the step kind at compile time (c.mode is
// then ignored); -1 reads it from c.  sm: 3 * NA f2 slots for this pair,
// stride apart (shared memory on the device).
// The plaquette form (see plaquette_projections) took the SU(3) step from
// 0.366 to 0.331 ms per 128^3 step on GB300 and, needing fewer registers,
// runs 4 blocks of 128 per SM without spills (the staple form: 3).
// 1: the two lower staples of a direction in a rolled loop (half the code of
// the direction's phase), 0: unrolled
#ifndef TCYM_PAIR_STAPLE_ROLLED
#define TCYM_PAIR_STAPLE_ROLLED 0
#endif
template <class F, bool SEAM, int MODE = -1>
TCYM_HD void site_step_pair(const Geom &g, const void *Uin, void *Uout, void *E, const StepCoef<float> &c,
                            const StepCoef<float> &cn, int64_t p, uint64_t step_add, f2 *sm, int stride) {
    using G2 = typename F::G2;
    using M2 = typename F::Mat2;
    constexpr int NA = F::NA;
    const int64_t Vh = g.V >> 1;
    const PairNbhd nb(g, p);
    auto load = [&](int d, int a, int dir) {
        return a ? F::load2(Uin, Vh, d, nb.at(dir, 1), SEAM && nb.swapped(dir, 1)) : F::load2(Uin, Vh, d, p, false);
    };
    plaquette_projections<F, M2>(load, sm, stride);
#pragma unroll 1
    for (int mu = 0; mu < 3; ++mu) {
        // lower staples S- = U_nu^dag(x+mu-nu) U_mu^dag(x-nu) U_nu(x-nu)
        M2 A = G2::zero();
#if TCYM_PAIR_STAPLE_ROLLED
#pragma unroll 1
#else
#pragma unroll
#endif
        for (int k = 1; k <= 2; ++k) {
            const int nu = mu + k >= 3 ? mu + k - 3 : mu + k;
            const M2 b1 = F::load2(Uin, Vh, nu, nb.at(mu, 1, nu, -1), SEAM && nb.swapped(mu, 1, nu, -1));
            const int64_t sb = nb.at(nu, -1);
            const bool wb = SEAM && nb.swapped(nu, -1);
            const M2 b2 = F::load2(Uin, Vh, mu, sb, wb);
            const M2 b3 = F::load2(Uin, Vh, nu, sb, wb);
            const M2 lo = G2::template mulu<false, false>(G2::template mulu<true, true>(b1, b2), b3);
            A = G2::add(A, G2::scale(f2(sel3(c.cnu, nu)), lo));
        }
        // the link and its field are read after the staple sum, so that they are
        // not live while it runs
        const M2 u = F::load2(Uin, Vh, mu, p, false);
        f2 e[NA];
        F::load_e2(E, Vh, mu, p, e);
        f2 f[NA];
        G2::proj_mul(u, A, f);
        add_plaquette_force<NA>(sm, stride, mu, c.cnu, f);
        const f2 fc(sel3(c.fc, mu));
        const int mode = MODE >= 0 ? MODE : c.mode;
        if (mode == MODE_LANGEVIN) {
            langevin_kick_pair<NA>(cn, mu, p, Vh, step_add, fc, f, e);
        } else if (mode == MODE_FLOW) {
#pragma unroll
            for (int a = 0; a < NA; ++a) e[a] = fc * f[a];
        } else {
#pragma unroll
            for (int a = 0; a < NA; ++a) e[a] = fma(fc, f[a], e[a]);
        }
        F::store_e2(E, Vh, mu, p, e);
        F::store2(Uout, Vh, mu, p, G2::iexp_mul(f2(sel3(c.uc, mu)), e, u));
    }
}

template <class F, bool SEAM, int MODE = -1>
TCYM_HD void site_step_pair(const Geom &g, const void *Uin, void *Uout, void *E, const StepCoef<float> &c, int64_t p,
                            uint64_t step_add, f2 *sm, int stride) {
    site_step_pair<F, SEAM, MODE>(g, Uin, Uout, E, c, c, p, step_add, sm, stride);
}

// Does the block of pairs [p0, p0 + n) touch the seam planes z = 0 or z = nz/2 - 1?
TCYM_HD bool pairs_touch_seam(const Geom &g, int64_t p0, int64_t n) {
    const int64_t Vh = g.V >> 1, plane = (int64_t)g.nx * g.ny;
    const int64_t last = (p0 + n < Vh ? p0 + n : Vh) - 1;
    return p0 < plane || last >= Vh - plane;
}

// How the paired step's blocks of 128 threads cover the pairs: tx = 0, 128
// consecutive pair indices (rows run on); otherwise a tx x ty tile (tx = 2^lx,
// tx * ty = 128) of one z-plane, so the +-y neighbours of most pairs are in the
// block's own L1 working set.  Chosen per lattice shape by the autotuner.
struct Tile {
    int tx, ty, lx;          // tile extents; lx = log2(tx)
    int tiles_x, tiles_y;    // tiles per z-plane
    int b0;                  // linear mapping: the launch starts at pair 128 b0 (a range of pairs)
};
// tx = 0: linear; else a tx x (128 / tx) tile, tx a power of two from 1 to 128
TCYM_HD Tile make_tile(const Geom &g, int tx) {
    if (tx <= 0) return Tile{0, 0, 0, 0, 0, 0};
    int lx = 0;
    while ((1 << lx) < tx) ++lx;
    const int ty = 128 / tx;
    return Tile{tx, ty, lx, (g.nx + tx - 1) / tx, (g.ny + ty - 1) / ty, 0};
}
TCYM_HD int64_t tile_blocks(const Geom &g, const Tile &t) {
    const int64_t Vh = g.V >> 1;
    if (t.tx == 0) return (Vh + 127) / 128;
    return (int64_t)t.tiles_x * t.tiles_y * (g.nz >> 1);
}
// Pair of thread `tid` in block `b`, and whether the block touches the seam;
// false: the thread has no pair (a partial tile or the last linear block).
TCYM_HD bool tile_pair(const Geom &g, const Tile &t, int64_t b, int tid, int64_t &p, bool &seam) {
    if (t.tx == 0) {
        p = (b + t.b0) * 128 + tid;
        seam = pairs_touch_seam(g, (b + t.b0) * 128, 128);
        return p < (g.V >> 1);
    }
    const int64_t per_plane = (int64_t)t.tiles_x * t.tiles_y;
    const int z = (int)(b / per_plane);
    const int r = (int)(b - (int64_t)z * per_plane);
    const int by = r / t.tiles_x, bx = r - by * t.tiles_x;
    const int x = bx * t.tx + (tid & (t.tx - 1)), y = by * t.ty + (tid >> t.lx);
    seam = z == 0 || z == (g.nz >> 1) - 1;
    p = x + (int64_t)g.nx * (y + (int64_t)g.ny * z);
    return x < g.nx && y < g.ny;
}

// Checkerboard flow: one link U_mu(x) of the active parity moved in place by
// exp(-i dtau F_mu(x)), F = fc proj(U_mu A) (no reference counterpart; the
// reference flows all links at once, GradientFlow.cpp:150-165).
template <class F>
TCYM_HD void link_flow(const Geom &g, void *U, int mu, const typename F::T (&fc)[3], const typename F::T (&cnu)[3],
                       const typename F::T (&uc)[3], int64_t s) {
    using G = typename F::G;
    using T = typename F::T;
    using M = typename F::Mat;
    Nbhd nb(g, s);
    M A = staple_sum<F>(U, g.V, nb, mu, cnu);
    M u = F::load(U, g.V, mu, s);
    T f[F::NA];
    G::proj_mul(u, A, f);
    const T fm = sel3(fc, mu);
#pragma unroll
    for (int a = 0; a < F::NA; ++a) f[a] *= fm;
    F::store(U, g.V, mu, s, G::iexp_mul(sel3(uc, mu), f, u));
}

// ----------------------------------------------------------------- observables
// Plaquette P_{mu nu}(x) in the four quadrants around x, each a loop from x
// (Plaquettes.cpp:28-31):
//   Q0 = U_{mu nu}(x), Q1 = U_{-mu nu}(x), Q2 = U_{mu -nu}(x), Q3 = U_{-mu -nu}(x)
template <class F>
TCYM_HD void clover_leaves(const void *U, int64_t V, const Nbhd &nb, int mu, int nu, typename F::Mat *Q) {
    using G = typename F::G;
    using M = typename F::Mat;
    // link along d at x + a e_mu + b e_nu
    auto L = [&](int d, int a, int b) { return F::load(U, V, d, nb.at(mu, a, nu, b)); };
    // Q0 = U_mu(x) U_nu(x+mu) U_mu^dag(x+nu) U_nu^dag(x)
    M a = L(mu, 0, 0), b = L(nu, 1, 0), c = L(mu, 0, 1), d = L(nu, 0, 0);
    Q[0] = G::mul(G::mul(a, b), G::template mulx<true, true>(c, d));
    // Q1 = U_nu(x) U_mu^dag(x+nu-mu) U_nu^dag(x-mu) U_mu(x-mu)
    a = L(nu, 0, 0);
    b = L(mu, -1, 1);
    c = L(nu, -1, 0);
    d = L(mu, -1, 0);
    Q[1] = G::mul(G::template mulx<false, true>(a, b), G::template mulx<true, false>(c, d));
    // Q2 = U_nu^dag(x-nu) U_mu(x-nu) U_nu(x-nu+mu) U_mu^dag(x)
    a = L(nu, 0, -1);
    b = L(mu, 0, -1);
    c = L(nu, 1, -1);
    d = L(mu, 0, 0);
    Q[2] = G::mul(G::template mulx<true, false>(a, b), G::template mulx<false, true>(c, d));
    // Q3 = U_mu^dag(x-mu) U_nu^dag(x-mu-nu) U_mu(x-mu-nu) U_nu(x-nu)
    a = L(mu, -1, 0);
    b = L(nu, -1, -1);
    c = L(mu, -1, -1);
    d = L(nu, 0, -1);
    Q[3] = G::mul(G::template mulx<true, true>(a, b), G::mul(c, d));
}

// Site at (x,y,z) + (dx,dy,dz) with periodic wrap, offsets in [-2, 2].
TCYM_HD int64_t site_offset(const Geom &g, int x, int y, int z, int dx, int dy, int dz) {
    int a = x + dx, b = y + dy, c = z + dz;
    a = a < 0 ? a + g.nx : (a >= g.nx ? a - g.nx : a);
    b = b < 0 ? b + g.ny : (b >= g.ny ? b - g.ny : b);
    c = c < 0 ? c + g.nz : (c >= g.nz ? c - g.nz : c);
    a = a < 0 ? a + g.nx : (a >= g.nx ? a - g.nx : a);  // extents of 2 wrap twice
    b = b < 0 ? b + g.ny : (b >= g.ny ? b - g.ny : b);
    c = c < 0 ? c + g.nz : (c >= g.nz ? c - g.nz : c);
    return (int64_t)a + (int64_t)g.nx * ((int64_t)b + (int64_t)g.ny * c);
}

// Product of links around a closed path from (x,y,z): step +(d+1) moves along
// U_d, step -(d+1) moves back along U_d^dag.
template <class F, int NS>
TCYM_HD typename F::Mat path_product(const void *U, const Geom &g, int x, int y, int z, const int (&steps)[NS]) {
    using G = typename F::G;
    typename F::Mat acc = G::identity();
    int p[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        const int d = (steps[k] > 0 ? steps[k] : -steps[k]) - 1;
        if (steps[k] > 0) {
            acc = G::mul(acc, F::load(U, g.V, d, site_offset(g, x, y, z, p[0], p[1], p[2])));
            p[d] += 1;
        } else {
            p[d] -= 1;
            acc = G::template mulx<false, true>(acc, F::load(U, g.V, d, site_offset(g, x, y, z, p[0], p[1], p[2])));
        }
    }
    return acc;
}

// O(a^2)-improved E.B at one site, ImprovedOperators::ComputeEDotB
// (CALC/ChernSimonsOperators.cpp:72-382), written with loops from x:
//   B_i = 2 proj(5/12 sum(4 boxes) - 1/24 sum(8 rectangles)) in the plane (i+1, i+2)
//   E_i = -1/12 Ad(U_i(x)) E_i(x+i) + 7/12 E_i(x) + 7/12 Ad^-1(U_i(x-i)) E_i(x-i)
//         - 1/12 Ad^-1(U_i(x-2i) U_i(x-i)) E_i(x-2i)
// (the reference builds the off-site loops at their own corner and transports
// them to x, :53-62 and :226-318; the loops from x are the same matrices).
template <class F> TCYM_HD double site_edotb_improved(const Geom &g, const void *U, const void *E, int64_t s) {
    using G = typename F::G;
    using T = typename F::T;
    using M = typename F::Mat;
    constexpr int NA = F::NA;
    const int x = (int)(s % g.nx), y = (int)((s / g.nx) % g.ny), z = (int)(s / ((int64_t)g.nx * g.ny));
    double sum = 0.0;
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        const int J = (i + 1) % 3 + 1, K = (i + 2) % 3 + 1;
        const int b0[4] = {J, K, -J, -K}, b1[4] = {K, -J, -K, J}, b2[4] = {-K, J, K, -J}, b3[4] = {-J, -K, J, K};
        const int r0[6] = {J, J, K, -J, -J, -K}, r1[6] = {J, K, K, -J, -K, -K}, r2[6] = {K, -J, -J, -K, J, J},
                  r3[6] = {K, K, -J, -K, -K, J}, r4[6] = {-J, -J, -K, J, J, K}, r5[6] = {-J, -K, -K, J, K, K},
                  r6[6] = {-K, J, J, K, -J, -J}, r7[6] = {-K, -K, J, K, K, -J};
        M boxes = G::add(G::add(path_product<F>(U, g, x, y, z, b0), path_product<F>(U, g, x, y, z, b1)),
                         G::add(path_product<F>(U, g, x, y, z, b2), path_product<F>(U, g, x, y, z, b3)));
        M rects = G::add(G::add(path_product<F>(U, g, x, y, z, r0), path_product<F>(U, g, x, y, z, r1)),
                         G::add(path_product<F>(U, g, x, y, z, r2), path_product<F>(U, g, x, y, z, r3)));
        rects = G::add(rects, G::add(G::add(path_product<F>(U, g, x, y, z, r4), path_product<F>(U, g, x, y, z, r5)),
                                     G::add(path_product<F>(U, g, x, y, z, r6), path_product<F>(U, g, x, y, z, r7))));
        M avg = G::add(G::scale(T(5.0 / 12.0), boxes), G::scale(T(-1.0 / 24.0), rects));
        T b[NA];
        G::proj(avg, b);
        const int dx = i == 0, dy = i == 1, dz = i == 2;
        const int64_t sp = site_offset(g, x, y, z, dx, dy, dz);
        const int64_t sm = site_offset(g, x, y, z, -dx, -dy, -dz);
        const int64_t sm2 = site_offset(g, x, y, z, -2 * dx, -2 * dy, -2 * dz);
        T e0[NA], ep[NA], em[NA], em2[NA], t1[NA], t2[NA], t3[NA];
        F::load_e(E, g.V, i, s, e0);
        F::load_e(E, g.V, i, sp, ep);
        F::load_e(E, g.V, i, sm, em);
        F::load_e(E, g.V, i, sm2, em2);
        G::adjoint(F::load(U, g.V, i, s), ep, t1);
        M um = F::load(U, g.V, i, sm);
        G::inverse_adjoint(um, em, t2);
        G::inverse_adjoint(G::mul(F::load(U, g.V, i, sm2), um), em2, t3);
        for (int a = 0; a < NA; ++a) {
            double ei = -(1.0 / 12.0) * (double)t1[a] + (7.0 / 12.0) * (double)e0[a] + (7.0 / 12.0) * (double)t2[a] -
                        (1.0 / 12.0) * (double)t3[a];
            sum += ei * 2.0 * (double)b[a];
        }
    }
    return sum;
}

// Everything the observables reduce, for one site (FP64 accumulators):
//   esq[mu]   sum_a E^a_mu(x)^2                        (BulkObservables.cpp:99-130)
//   bsq[i]    4 Re tr(1 - P_jk(x)), (i,j,k) cyclic      (BulkObservables.cpp:55-88)
//   g[a]      Gauss violation G^a(x)                    (CALC/GaussViolation.cpp:13-23)
//   un[mu]    ||U_mu U_mu^dag - 1||                     (UnitarityViolation.cpp:13-51)
//   edotb     sum_i E_i^clover . B_i^clover             (ChernSimonsOperators.cpp:4-47)
// OBS_EDOTB_IMP puts the O(a^2)-improved E.B in the edotb slot instead of the clover one.
enum ObsMask : int { OBS_BULK = 1, OBS_GAUSS = 2, OBS_UNIT = 4, OBS_EDOTB = 8, OBS_ALL = 15, OBS_EDOTB_IMP = 16 };

template <class F> struct SiteObs {
    double esq[3], bsq[3], g[F::NA], un[3], edotb;
};

template <class F>
TCYM_HD void site_observables(const Geom &g, const void *U, const void *E, int mask, int64_t s, SiteObs<F> &o) {
    using G = typename F::G;
    using T = typename F::T;
    using M = typename F::Mat;
    constexpr int NA = F::NA;
    const int64_t V = g.V;
    Nbhd nb(g, s);
    for (int mu = 0; mu < 3; ++mu) { o.esq[mu] = 0; o.bsq[mu] = 0; o.un[mu] = 0; }
    for (int a = 0; a < NA; ++a) o.g[a] = 0;
    o.edotb = 0;
    if (mask & OBS_EDOTB_IMP) {
        o.edotb = site_edotb_improved<F>(g, U, E, s);
        mask &= ~(OBS_EDOTB | OBS_EDOTB_IMP);
    }
    T et[3][NA];  // U_mu^dag(x-mu) E_mu(x-mu) U_mu(x-mu): shared by Gauss and clover E
    if (mask & (OBS_GAUSS | OBS_EDOTB)) {
#pragma unroll
        for (int mu = 0; mu < 3; ++mu) {
            const int64_t sm = nb.at(mu, -1);
            T e[NA];
            F::load_e(E, V, mu, sm, e);
            G::inverse_adjoint(F::load(U, V, mu, sm), e, et[mu]);
        }
    }
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
        T e[NA];
        F::load_e(E, V, mu, s, e);
        double sq = 0;
        for (int a = 0; a < NA; ++a) sq += (double)e[a] * (double)e[a];
        o.esq[mu] = sq;
        if (mask & OBS_GAUSS)
            for (int a = 0; a < NA; ++a) o.g[a] += (double)e[a] - (double)et[mu][a];
        if (mask & OBS_UNIT) o.un[mu] = (double)G::unitarity_norm(F::load(U, V, mu, s));
        if (mask & (OBS_BULK | OBS_EDOTB)) {
            // plane (j,k) = (mu+1, mu+2): B_mu
            const int j = (mu + 1) % 3, k = (mu + 2) % 3;
            M Q[4];
            if (mask & OBS_EDOTB) {
                clover_leaves<F>(U, V, nb, j, k, Q);
            } else {
                M a = F::load(U, V, j, s), b = F::load(U, V, k, nb.at(j, 1)), c = F::load(U, V, j, nb.at(k, 1)),
                  d = F::load(U, V, k, s);
                Q[0] = G::mul(G::mul(a, b), G::template mulx<true, true>(c, d));
            }
            o.bsq[mu] = 4.0 * (double)G::retr_one_minus(Q[0]);
            if (mask & OBS_EDOTB) {
                M avg = G::scale(T(0.25), G::add(G::add(Q[0], Q[1]), G::add(Q[2], Q[3])));
                T b[NA];
                G::proj(avg, b);
                double dot = 0;
                for (int a = 0; a < NA; ++a) dot += 0.5 * ((double)e[a] + (double)et[mu][a]) * 2.0 * (double)b[a];
                o.edotb += dot;
            }
        }
    }
}

// The N_CS sample's observables (mask OBS_EDOTB) of direction mu for both sites of
// pair p of FP32 pair storage (even nz), in packed FP32 (lane 0: site p, lane 1:
// its partner p + Vh): E_mu^2 into esq, the plaquette term of B_mu^2 into bsq, and
// the clover E_mu . B_mu returned, as site_observables forms them.  SEAM: the pair
// may step across the z seam, where a neighbour's lanes come swapped.  The clover
// average's projection is the average of the leaves' projections (proj is linear),
// so each leaf is a left-to-right chain of products whose last one is projected
// at once (proj_mul, proj_mul_dag) and no 3x3 sum is held; E.B accumulates in FP32.
template <class F, bool SEAM>
TCYM_HD f2 pair_edotb_obs(const Geom &g, const void *U, const void *E, int64_t p, int mu, f2 &esq, f2 &bsq) {
    using G2 = typename F::G2;
    using M2 = typename F::Mat2;
    constexpr int NA = F::NA;
    const int64_t Vh = g.V >> 1;
    const PairNbhd nb(g, p);
    // clover of plane (j, k) = (mu+1, mu+2): the leaves of clover_leaves(j, k)
    const int j = mu == 2 ? 0 : mu + 1, k = mu == 0 ? 2 : mu - 1;
    auto L = [&](int d, int a, int b) {
        return F::load2(U, Vh, d, nb.at(j, a, k, b), SEAM && nb.swapped(j, a, k, b));
    };
    f2 b[NA], pr[NA];
    {
        // Q0 = U_j(x) U_k(x+j) U_j^dag(x+k) U_k^dag(x), whole: its trace is the plaquette term
        M2 t = G2::mul(L(j, 0, 0), L(k, 1, 0));
        t = G2::template mulx<false, true>(t, L(j, 0, 1));
        const M2 q0 = G2::template mulx<false, true>(t, L(k, 0, 0));
        bsq = f2(4.0) * G2::retr_one_minus(q0);
        G2::proj(q0, b);
    }
    {
        // Q1 = U_k(x) U_j^dag(x+k-j) U_k^dag(x-j) U_j(x-j)
        M2 t = G2::template mulx<false, true>(L(k, 0, 0), L(j, -1, 1));
        t = G2::template mulx<false, true>(t, L(k, -1, 0));
        G2::proj_mul(t, L(j, -1, 0), pr);
#pragma unroll
        for (int a = 0; a < NA; ++a) b[a] = b[a] + pr[a];
    }
    {
        // Q2 = U_k^dag(x-k) U_j(x-k) U_k(x-k+j) U_j^dag(x)
        M2 t = G2::template mulx<true, false>(L(k, 0, -1), L(j, 0, -1));
        t = G2::mul(t, L(k, 1, -1));
        G2::proj_mul_dag(t, L(j, 0, 0), pr);
#pragma unroll
        for (int a = 0; a < NA; ++a) b[a] = b[a] + pr[a];
    }
    {
        // Q3 = U_j^dag(x-j) U_k^dag(x-j-k) U_j(x-j-k) U_k(x-k)
        M2 t = G2::template mulx<true, true>(L(j, -1, 0), L(k, -1, -1));
        t = G2::mul(t, L(j, -1, -1));
        G2::proj_mul(t, L(k, 0, -1), pr);
#pragma unroll
        for (int a = 0; a < NA; ++a) b[a] = f2(0.25) * (b[a] + pr[a]);
    }
    // E_mu(x) and U_mu^dag(x-mu) E_mu(x-mu) U_mu(x-mu)
    f2 e[NA], et[NA];
    {
        f2 em[NA];
        const int64_t pm = nb.at(mu, -1);
        const bool sw = SEAM && nb.swapped(mu, -1);
        F::load_e2(E, Vh, mu, pm, em);
        if (sw) {
#pragma unroll
            for (int a = 0; a < NA; ++a) em[a] = swap_f2(em[a]);
        }
        G2::inverse_adjoint(F::load2(U, Vh, mu, pm, sw), em, et);
    }
    F::load_e2(E, Vh, mu, p, e);
    f2 sq(0.0), dot(0.0);
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        sq = fma(e[a], e[a], sq);
        dot = fma(e[a] + et[a], b[a], dot);
    }
    esq = sq;
    return dot;
}

// Gauss violation G(x) in working precision T, for the restore iteration.
template <class F>
TCYM_HD void site_gauss(const Geom &g, const void *U, const void *E, int64_t s, double *gv) {
    using G = typename F::G;
    using T = typename F::T;
    constexpr int NA = F::NA;
    Nbhd nb(g, s);
    for (int a = 0; a < NA; ++a) gv[a] = 0;
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
        const int64_t sm = nb.at(mu, -1);
        T e[NA], em[NA], t[NA];
        F::load_e(E, g.V, mu, s, e);
        F::load_e(E, g.V, mu, sm, em);
        G::inverse_adjoint(F::load(U, g.V, mu, sm), em, t);
        for (int a = 0; a < NA; ++a) gv[a] += (double)e[a] - (double)t[a];
    }
}

// E_mu(x) -= gam (G(x) - U_mu(x) G(x+mu) U_mu^dag(x))   (GaussRestore.cpp:73-113)
// G is an FP64 SoA scratch array G[a*V + site].
template <class F>
TCYM_HD void site_gauss_update(const Geom &g, const void *U, void *E, const double *Gs, double gam, int64_t s) {
    using G = typename F::G;
    using T = typename F::T;
    constexpr int NA = F::NA;
    Nbhd nb(g, s);
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
        const int64_t sp = nb.at(mu, 1);
        T gp[NA], t[NA], e[NA];
        for (int a = 0; a < NA; ++a) gp[a] = (T)Gs[a * g.V + sp];
        G::adjoint(F::load(U, g.V, mu, s), gp, t);
        F::load_e(E, g.V, mu, s, e);
        for (int a = 0; a < NA; ++a) e[a] = (T)((double)e[a] - gam * (Gs[a * g.V + s] - (double)t[a]));
        F::store_e(E, g.V, mu, s, e);
    }
}

// ------------------------------------------------------------ initial conditions
template <class F> TCYM_HD void site_set_zero(const Geom &g, void *U, void *E, int64_t s) {
    using T = typename F::T;
    T z[F::NA];
    for (int a = 0; a < F::NA; ++a) z[a] = T(0);
    for (int mu = 0; mu < 3; ++mu) {
        F::store(U, g.V, mu, s, F::G::identity());
        F::store_e(E, g.V, mu, s, z);
    }
}

// E^a_mu(x) = sigma N(0,1) (field stream); computed in FP64 and rounded.
template <class F>
TCYM_HD void site_gaussian_efield(const Geom &g, void *E, double sigma, uint64_t seed, int64_t s, uint64_t step = 0) {
    using T = typename F::T;
    for (int mu = 0; mu < 3; ++mu) {
        double z[F::NA];
        normals<double, F::NA>(seed, STREAM_EFIELD, step, (uint32_t)s, (uint32_t)mu, z);
        T e[F::NA];
        for (int a = 0; a < F::NA; ++a) e[a] = (T)(sigma * z[a]);
        F::store_e(E, g.V, mu, s, e);
    }
}

// U_mu(x) = exp(i t^a theta^a), theta^a = sigma N(0,1) (link stream); FP64 then rounded.
// a link in another precision
template <class T, class S> TCYM_HD Q4<T> recast(const Q4<S> &m) {
    return Q4<T>{{(T)m.q[0], (T)m.q[1], (T)m.q[2], (T)m.q[3]}};
}
template <class T, class S> TCYM_HD M3<T> recast(const M3<S> &m) {
    M3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = cx<T>{(T)m.m[i][j].re, (T)m.m[i][j].im};
    return r;
}
template <class F> using Group64 = typename std::conditional<F::NA == 3, SU2<double>, SU3<double>>::type;

template <class F> TCYM_HD void site_random_links(const Geom &g, void *U, double sigma, uint64_t seed, int64_t s) {
    using G64 = Group64<F>;
    using T = typename F::T;
    for (int mu = 0; mu < 3; ++mu) {
        double th[F::NA];
        normals<double, F::NA>(seed, STREAM_LINKS, 0, (uint32_t)s, (uint32_t)mu, th);
        for (int a = 0; a < F::NA; ++a) th[a] *= sigma;
        F::store(U, g.V, mu, s, recast<T>(G64::iexp(1.0, th)));
    }
}

// Block (LATTICE/GaugeLinks.cpp:124-145) for site s of the blocked lattice gd
// (half the even extents of gs): U'_mu(x) = U_mu(2x) U_mu(2x + mu), the product
// in FP64 whatever the storage.
template <class F> TCYM_HD void site_block(const Geom &gs, const Geom &gd, const void *Us, void *Ud, int64_t s) {
    using T = typename F::T;
    using G64 = Group64<F>;
    const int x = (int)(s % gd.nx), y = (int)((s / gd.nx) % gd.ny), z = (int)(s / ((int64_t)gd.nx * gd.ny));
    const int64_t s0 = 2 * x + (int64_t)gs.nx * (2 * y + (int64_t)gs.ny * (2 * z));
    const int64_t step[3] = {1, gs.nx, (int64_t)gs.nx * gs.ny};  // 2x + mu stays inside: extents are even
    for (int mu = 0; mu < 3; ++mu) {
        const auto a = recast<double>(F::load(Us, gs.V, mu, s0));
        const auto b = recast<double>(F::load(Us, gs.V, mu, s0 + step[mu]));
        F::store(Ud, gd.V, mu, s, recast<T>(G64::mul(a, b)));
    }
}

// FP64 reunitarisation of the stored links (new: the reference only monitors
// unitarity).  Links are widened to FP64, projected and rounded back.
template <class F> TCYM_HD void site_reunitarize(const Geom &g, void *U, int64_t s) {
    using T = typename F::T;
    for (int mu = 0; mu < 3; ++mu)
        F::store(U, g.V, mu, s, recast<T>(Group64<F>::reunitarize(recast<double>(F::load(U, g.V, mu, s)))));
}

// GeodesicInterpolation (SUNc/AdvancedOperations.cpp:432-442) on the links of
// site s, in FP64 whatever the storage: EMid = ILog(-1, UNew UOld^dag) and
// UMid = IExp(-c, EMid) UOld, so UMid runs from UOld (c = 0) to UNew (c = 1);
// EMid in field units (CoolingMethod.cpp:39-70: cE = 1 at unit spacing).
template <class F>
TCYM_HD void site_geodesic(const Geom &g, const void *Uold, const void *Unew, double c, void *Umid, void *Emid,
                           int64_t s) {
    using G64 = Group64<F>;
    using T = typename F::T;
    for (int mu = 0; mu < 3; ++mu) {
        const typename G64::Mat uo = recast<double>(F::load(Uold, g.V, mu, s));
        const typename G64::Mat un = recast<double>(F::load(Unew, g.V, mu, s));
        double e[F::NA];
        G64::ilog(-1.0, G64::template mulx<false, true>(un, uo), e);
        F::store(Umid, g.V, mu, s, recast<T>(G64::mul(G64::iexp(-c, e), uo)));
        T et[F::NA];
        for (int a = 0; a < F::NA; ++a) et[a] = (T)e[a];
        F::store_e(Emid, g.V, mu, s, et);
    }
}

// ----------------------------------------------------------- AoS conversion
template <class F> TCYM_HD void site_from_aos(const Geom &g, void *U, void *E, const double *Ua, const double *Ea, int64_t s) {
    using T = typename F::T;
    constexpr int NMD = F::NA == 3 ? 4 : 18;
    for (int mu = 0; mu < 3; ++mu) {
        if (Ua) {
            typename F::Mat m;
            if constexpr (F::NA == 3) {
                for (int k = 0; k < 4; ++k) m.q[k] = (T)Ua[NMD * (mu + 3 * s) + k];
            } else {
                const double *a = Ua + NMD * (mu + 3 * s);
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) m.m[i][j] = cx<T>{(T)a[2 * (i + 3 * j)], (T)a[2 * (i + 3 * j) + 1]};
            }
            F::store(U, g.V, mu, s, m);
        }
        if (Ea) {
            T e[F::NA];
            for (int a = 0; a < F::NA; ++a) e[a] = (T)Ea[F::NA * (mu + 3 * s) + a];
            F::store_e(E, g.V, mu, s, e);
        }
    }
}

// One link (mu) of site s from / to AoS records held at slot k of a staging area
// (the AoS arrays themselves when k = s), for the shared-memory conversion kernels.
template <class F>
TCYM_HD void site_link_from_aos(const Geom &g, void *U, void *E, const double *Ua, const double *Ea, int64_t k,
                                int64_t s, int mu) {
    using T = typename F::T;
    constexpr int NMD = F::NA == 3 ? 4 : 18;
    if (Ua) {
        typename F::Mat m;
        const double *a = Ua + NMD * (mu + 3 * k);
        if constexpr (F::NA == 3) {
            for (int q = 0; q < 4; ++q) m.q[q] = (T)a[q];
        } else {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) m.m[i][j] = cx<T>{(T)a[2 * (i + 3 * j)], (T)a[2 * (i + 3 * j) + 1]};
        }
        F::store(U, g.V, mu, s, m);
    }
    if (Ea) {
        T e[F::NA];
        for (int a = 0; a < F::NA; ++a) e[a] = (T)Ea[F::NA * (mu + 3 * k) + a];
        F::store_e(E, g.V, mu, s, e);
    }
}
template <class F>
TCYM_HD void site_link_to_aos(const Geom &g, const void *U, const void *E, double *Ua, double *Ea, int64_t k,
                              int64_t s, int mu) {
    using T = typename F::T;
    constexpr int NMD = F::NA == 3 ? 4 : 18;
    if (Ua) {
        const typename F::Mat m = F::load(U, g.V, mu, s);
        double *a = Ua + NMD * (mu + 3 * k);
        if constexpr (F::NA == 3) {
            for (int q = 0; q < 4; ++q) a[q] = (double)m.q[q];
        } else {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    a[2 * (i + 3 * j)] = (double)m.m[i][j].re;
                    a[2 * (i + 3 * j) + 1] = (double)m.m[i][j].im;
                }
        }
    }
    if (Ea) {
        T e[F::NA];
        F::load_e(E, g.V, mu, s, e);
        for (int a = 0; a < F::NA; ++a) Ea[F::NA * (mu + 3 * k) + a] = (double)e[a];
    }
}

template <class F> TCYM_HD void site_to_aos(const Geom &g, const void *U, const void *E, double *Ua, double *Ea, int64_t s) {
    using T = typename F::T;
    constexpr int NMD = F::NA == 3 ? 4 : 18;
    for (int mu = 0; mu < 3; ++mu) {
        if (Ua) {
            typename F::Mat m = F::load(U, g.V, mu, s);
            if constexpr (F::NA == 3) {
                for (int k = 0; k < 4; ++k) Ua[NMD * (mu + 3 * s) + k] = (double)m.q[k];
            } else {
                double *a = Ua + NMD * (mu + 3 * s);
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        a[2 * (i + 3 * j)] = (double)m.m[i][j].re;
                        a[2 * (i + 3 * j) + 1] = (double)m.m[i][j].im;
                    }
            }
        }
        if (Ea) {
            T e[F::NA];
            F::load_e(E, g.V, mu, s, e);
            for (int a = 0; a < F::NA; ++a) Ea[F::NA * (mu + 3 * s) + a] = (double)e[a];
        }
    }
}

}  // namespace tcym
