// Device storage formats: structure-of-arrays planes of 16-byte vectors.
//
// A lattice of V = nx*ny*nz sites (site = x + nx*(y + ny*z), the reference's
// Index3D, LATTICE/GaugeLinks.cpp:27-31) stores, per direction mu, a fixed
// number of planes; plane p of direction mu is a contiguous array of vectors
// at offset (mu*P + p)*N.  A warp of consecutive sites (or site pairs) reads
// every plane as one coalesced 512-byte (float4, double2) or 256-byte
// (float2) transaction.
//
// The FP32 formats hold site pairs (s, s + Vh), Vh = ceil(V/2), N = Vh, each
// component packed as {site, partner} (see "site pairs" below); the FP64
// formats hold single sites, N = V.
//
//   format        link planes (per mu)                       E planes (per mu)
//   SU2 FP32      2 x float4 {q0,q0',q1,q1'},{q2,q2',q3,q3'} 3 x float2 {E^a,E^a'}
//   SU2 FP64      2 x double2 (q0,q1),(q2,q3)                3 x double
//   SU3 FP32      6 x float4 {re,re',im,im'}, rows 0 and 1:  4 x float4
//                 entries u00,u01,u02,u10,u11,u12;           {E^2q,E^2q',E^2q+1,E^2q+1'}
//                 row 2 = conj(row0 x row1) on load
//   SU3 FP64      9 x double2, all entries, row-major        4 x double2
//
// Bytes per link (U + E): SU2 FP32 16+12, SU2 FP64 32+24, SU3 FP32 48+32,
// SU3 FP64 144+64 (FP32 formats: one padding site when V is odd).
#pragma once

#include "tcym_math.cuh"

namespace tcym {

struct Geom {
    int nx, ny, nz;
    int64_t V;
};

// a[i] for a direction i known only at run time, by selects: indexing a small
// array with a run-time index would place it in local memory.
template <class T> TCYM_HD T sel3(const T (&a)[3], int i) { return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]); }

// Periodic neighbourhood of one site: the signed site-index offsets of its
// forward and backward neighbour along each axis (the wrap folded in), so a
// neighbour of a run-time direction is s + a select, all in registers.
// Extents stay below 2^31 sites per plane, so offsets fit 32 bits.
struct Nbhd {
    int64_t s;
    int fx, fy, fz, bx, by, bz;
    int par;
    TCYM_HD Nbhd(const Geom &g, int64_t site) : s(site) {
        const int x = (int)(site % g.nx);
        const int64_t r = site / g.nx;
        const int y = (int)(r % g.ny);
        const int z = (int)(r / g.ny);
        const int sy = g.nx, sz = g.nx * g.ny;
        fx = x == g.nx - 1 ? 1 - g.nx : 1;
        bx = x == 0 ? g.nx - 1 : -1;
        fy = y == g.ny - 1 ? (1 - g.ny) * sy : sy;
        by = y == 0 ? (g.ny - 1) * sy : -sy;
        fz = z == g.nz - 1 ? (1 - g.nz) * sz : sz;
        bz = z == 0 ? (g.nz - 1) * sz : -sz;
        par = (x + y + z) & 1;
    }
    // offset of one step along axis d, a in {-1, 0, 1} (a is a constant at every call site)
    TCYM_HD int step(int d, int a) const {
        if (a == 0) return 0;
        return a > 0 ? (d == 0 ? fx : (d == 1 ? fy : fz)) : (d == 0 ? bx : (d == 1 ? by : bz));
    }
    // the site s + a e_d
    TCYM_HD int64_t at(int d, int a) const { return s + step(d, a); }
    // the site s + a e_mu + b e_nu, mu != nu
    TCYM_HD int64_t at(int mu, int a, int nu, int b) const { return s + step(mu, a) + step(nu, b); }
    TCYM_HD int parity() const { return par; }
};

enum Format : int { FMT_SU2_F32 = 0, FMT_SU2_F64 = 1, FMT_SU3_F32 = 2, FMT_SU3_F64 = 3 };

template <int FMT> struct Fmt;

// ------------------------------------------------------------------ site pairs
// The FP32 formats store sites in pairs: site s < Vh = ceil(V/2) and site
// s + Vh share every 16-byte vector, as lane 0 and lane 1 of each packed
// component {a0, a1, b0, b1}, so that one thread can advance both with packed
// FP32 instructions.  For even nz the partner of (x, y, z) is (x, y, z + nz/2).
// Scalar access (any kernel working per site) reads or writes one lane.
TCYM_HD int64_t pair_sites(int64_t V) { return (V + 1) >> 1; }
// pair index and lane of site s
TCYM_HD int64_t pair_of(int64_t s, int64_t Vh, int &l) {
    l = s >= Vh;
    return l ? s - Vh : s;
}

// Neighbourhood of the pair p = x + nx (y + ny z), z < nz/2, of a lattice with
// even nz, in pair indices.  A step across the seam (z = nz/2 - 1 -> nz/2, or
// z = 0 -> -1) lands on the partner sites, i.e. on a pair whose lanes are
// swapped; swapped() says when.
struct PairNbhd {
    int64_t p;
    int fx, fy, fz, bx, by, bz;
    bool zf, zb;
    TCYM_HD PairNbhd(const Geom &g, int64_t pair) : p(pair) {
        const int nzh = g.nz >> 1;
        const int x = (int)(pair % g.nx);
        const int64_t r = pair / g.nx;
        const int y = (int)(r % g.ny);
        const int z = (int)(r / g.ny);
        const int sy = g.nx, sz = g.nx * g.ny;
        fx = x == g.nx - 1 ? 1 - g.nx : 1;
        bx = x == 0 ? g.nx - 1 : -1;
        fy = y == g.ny - 1 ? (1 - g.ny) * sy : sy;
        by = y == 0 ? (g.ny - 1) * sy : -sy;
        zf = z == nzh - 1;
        zb = z == 0;
        fz = zf ? (1 - nzh) * sz : sz;
        bz = zb ? (nzh - 1) * sz : -sz;
    }
    TCYM_HD int step(int d, int a) const {
        if (a == 0) return 0;
        return a > 0 ? (d == 0 ? fx : (d == 1 ? fy : fz)) : (d == 0 ? bx : (d == 1 ? by : bz));
    }
    TCYM_HD bool swapped(int d, int a) const { return a != 0 && d == 2 && (a > 0 ? zf : zb); }
    TCYM_HD int64_t at(int d, int a) const { return p + step(d, a); }
    TCYM_HD int64_t at(int mu, int a, int nu, int b) const { return p + step(mu, a) + step(nu, b); }
    TCYM_HD bool swapped(int mu, int a, int nu, int b) const { return swapped(mu, a) != swapped(nu, b); }
};

TCYM_HD float4 swap_lanes(float4 v) { return make_float4(v.y, v.x, v.w, v.z); }

// SU(2) FP32, per direction: links in 2 planes of float4 {q0, q0', q1, q1'} and
// {q2, q2', q3, q3'} (primes: the partner site); fields in 3 planes of float2 {e, e'}.
template <> struct Fmt<FMT_SU2_F32> {
    using T = float;
    using G = SU2<float>;
    using Mat = G::Mat;
    using G2 = SU2<f2>;
    using Mat2 = G2::Mat;
    static constexpr int NA = 3;
    static constexpr bool PAIRED = true;
    static TCYM_HD Mat load(const void *U, int64_t V, int mu, int64_t s) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        const float *f = static_cast<const float *>(U);
        const float *a = f + 4 * ((mu * 2) * Vh + p), *b = f + 4 * ((mu * 2 + 1) * Vh + p);
        return Mat{{a[l], a[2 + l], b[l], b[2 + l]}};
    }
    static TCYM_HD void store(void *U, int64_t V, int mu, int64_t s, const Mat &m) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        float *f = static_cast<float *>(U);
        float *a = f + 4 * ((mu * 2) * Vh + p), *b = f + 4 * ((mu * 2 + 1) * Vh + p);
        a[l] = m.q[0]; a[2 + l] = m.q[1]; b[l] = m.q[2]; b[2 + l] = m.q[3];
    }
    static TCYM_HD void load_e(const void *E, int64_t V, int mu, int64_t s, T *e) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        const float *f = static_cast<const float *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) e[a] = f[2 * ((mu * 3 + a) * Vh + p) + l];
    }
    static TCYM_HD void store_e(void *E, int64_t V, int mu, int64_t s, const T *e) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        float *f = static_cast<float *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) f[2 * ((mu * 3 + a) * Vh + p) + l] = e[a];
    }
    // both sites of pair p; swap: the pair is read with its lanes exchanged
    static TCYM_HD Mat2 load2(const void *U, int64_t Vh, int mu, int64_t p, bool swap) {
        const float4 *q = static_cast<const float4 *>(U);
        float4 a = q[(mu * 2) * Vh + p], b = q[(mu * 2 + 1) * Vh + p];
        if (swap) { a = swap_lanes(a); b = swap_lanes(b); }
        return Mat2{{f2(a.x, a.y), f2(a.z, a.w), f2(b.x, b.y), f2(b.z, b.w)}};
    }
    static TCYM_HD void store2(void *U, int64_t Vh, int mu, int64_t p, const Mat2 &m) {
        float4 *q = static_cast<float4 *>(U);
        q[(mu * 2) * Vh + p] = make_float4(m.q[0].v.x, m.q[0].v.y, m.q[1].v.x, m.q[1].v.y);
        q[(mu * 2 + 1) * Vh + p] = make_float4(m.q[2].v.x, m.q[2].v.y, m.q[3].v.x, m.q[3].v.y);
    }
    static TCYM_HD void load_e2(const void *E, int64_t Vh, int mu, int64_t p, f2 *e) {
        const float2 *q = static_cast<const float2 *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) e[a] = f2_of(q[(mu * 3 + a) * Vh + p]);
    }
    static TCYM_HD void store_e2(void *E, int64_t Vh, int mu, int64_t p, const f2 *e) {
        float2 *q = static_cast<float2 *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) q[(mu * 3 + a) * Vh + p] = e[a].v;
    }
};

template <> struct Fmt<FMT_SU2_F64> {
    using T = double;
    using G = SU2<double>;
    using Mat = G::Mat;
    static constexpr int NA = 3;
    static constexpr bool PAIRED = false;
    static TCYM_HD Mat load(const void *U, int64_t V, int mu, int64_t s) {
        const double2 *p = static_cast<const double2 *>(U);
        double2 a = p[(mu * 2) * V + s], b = p[(mu * 2 + 1) * V + s];
        return Mat{{a.x, a.y, b.x, b.y}};
    }
    static TCYM_HD void store(void *U, int64_t V, int mu, int64_t s, const Mat &m) {
        double2 *p = static_cast<double2 *>(U);
        p[(mu * 2) * V + s] = make_double2(m.q[0], m.q[1]);
        p[(mu * 2 + 1) * V + s] = make_double2(m.q[2], m.q[3]);
    }
    static TCYM_HD void load_e(const void *E, int64_t V, int mu, int64_t s, T *e) {
        const double *p = static_cast<const double *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) e[a] = p[(mu * 3 + a) * V + s];
    }
    static TCYM_HD void store_e(void *E, int64_t V, int mu, int64_t s, const T *e) {
        double *p = static_cast<double *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) p[(mu * 3 + a) * V + s] = e[a];
    }
};

// SU(3) FP32, per direction: rows 0 and 1 of the link (row 2 = conj(row0 x row1)
// on load), entry k = 3 i + j in plane k as float4 {re, re', im, im'}; fields in
// 4 planes of float4 {e_2q, e_2q', e_2q+1, e_2q+1'}.
template <> struct Fmt<FMT_SU3_F32> {
    using T = float;
    using G = SU3<float>;
    using Mat = G::Mat;
    using G2 = SU3<f2>;
    using Mat2 = G2::Mat;
    static constexpr int NA = 8;
    static constexpr bool PAIRED = true;
    static TCYM_HD Mat load(const void *U, int64_t V, int mu, int64_t s) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        const float *f = static_cast<const float *>(U);
        Mat m;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float *q = f + 4 * ((mu * 6 + k) * Vh + p);
            m.m[k / 3][k % 3] = cx<float>{q[l], q[2 + l]};
        }
        G::complete_row2(m);
        return m;
    }
    static TCYM_HD void store(void *U, int64_t V, int mu, int64_t s, const Mat &m) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        float *f = static_cast<float *>(U);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            float *q = f + 4 * ((mu * 6 + k) * Vh + p);
            q[l] = m.m[k / 3][k % 3].re;
            q[2 + l] = m.m[k / 3][k % 3].im;
        }
    }
    static TCYM_HD void load_e(const void *E, int64_t V, int mu, int64_t s, T *e) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        const float *f = static_cast<const float *>(E);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float *r = f + 4 * ((mu * 4 + q) * Vh + p);
            e[2 * q] = r[l];
            e[2 * q + 1] = r[2 + l];
        }
    }
    static TCYM_HD void store_e(void *E, int64_t V, int mu, int64_t s, const T *e) {
        int l;
        const int64_t Vh = pair_sites(V), p = pair_of(s, Vh, l);
        float *f = static_cast<float *>(E);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float *r = f + 4 * ((mu * 4 + q) * Vh + p);
            r[l] = e[2 * q];
            r[2 + l] = e[2 * q + 1];
        }
    }
    // both sites of pair p; swap: the pair is read with its lanes exchanged
    static TCYM_HD Mat2 load2(const void *U, int64_t Vh, int mu, int64_t p, bool swap) {
        const float4 *q = static_cast<const float4 *>(U);
        Mat2 m;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            float4 v = q[(mu * 6 + k) * Vh + p];
            if (swap) v = swap_lanes(v);
            m.m[k / 3][k % 3] = cx<f2>{f2(v.x, v.y), f2(v.z, v.w)};
        }
        G2::complete_row2(m);
        return m;
    }
    static TCYM_HD void store2(void *U, int64_t Vh, int mu, int64_t p, const Mat2 &m) {
        float4 *q = static_cast<float4 *>(U);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const cx<f2> z = m.m[k / 3][k % 3];
            q[(mu * 6 + k) * Vh + p] = make_float4(z.re.v.x, z.re.v.y, z.im.v.x, z.im.v.y);
        }
    }
    static TCYM_HD void load_e2(const void *E, int64_t Vh, int mu, int64_t p, f2 *e) {
        const float4 *q = static_cast<const float4 *>(E);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 v = q[(mu * 4 + k) * Vh + p];
            e[2 * k] = f2(v.x, v.y);
            e[2 * k + 1] = f2(v.z, v.w);
        }
    }
    static TCYM_HD void store_e2(void *E, int64_t Vh, int mu, int64_t p, const f2 *e) {
        float4 *q = static_cast<float4 *>(E);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            q[(mu * 4 + k) * Vh + p] = make_float4(e[2 * k].v.x, e[2 * k].v.y, e[2 * k + 1].v.x, e[2 * k + 1].v.y);
    }
};

template <> struct Fmt<FMT_SU3_F64> {
    using T = double;
    using G = SU3<double>;
    using Mat = G::Mat;
    static constexpr int NA = 8;
    static constexpr bool PAIRED = false;
    static TCYM_HD Mat load(const void *U, int64_t V, int mu, int64_t s) {
        const double2 *p = static_cast<const double2 *>(U);
        Mat m;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                double2 v = p[(mu * 9 + 3 * i + j) * V + s];
                m.m[i][j] = cx<double>{v.x, v.y};
            }
        return m;
    }
    static TCYM_HD void store(void *U, int64_t V, int mu, int64_t s, const Mat &m) {
        double2 *p = static_cast<double2 *>(U);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) p[(mu * 9 + 3 * i + j) * V + s] = make_double2(m.m[i][j].re, m.m[i][j].im);
    }
    static TCYM_HD void load_e(const void *E, int64_t V, int mu, int64_t s, T *e) {
        const double2 *p = static_cast<const double2 *>(E);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double2 v = p[(mu * 4 + q) * V + s];
            e[2 * q] = v.x; e[2 * q + 1] = v.y;
        }
    }
    static TCYM_HD void store_e(void *E, int64_t V, int mu, int64_t s, const T *e) {
        double2 *p = static_cast<double2 *>(E);
#pragma unroll
        for (int q = 0; q < 4; ++q) p[(mu * 4 + q) * V + s] = make_double2(e[2 * q], e[2 * q + 1]);
    }
};

}  // namespace tcym
