// Device storage formats: structure-of-arrays planes of 16-byte vectors.
//
// A lattice of V = nx*ny*nz sites (site = x + nx*(y + ny*z), the reference's
// Index3D, LATTICE/GaugeLinks.cpp:27-31) stores, per direction mu, a fixed
// number of planes; plane p of direction mu is a contiguous array of V vectors
// at offset (mu*P + p)*V.  A warp of consecutive sites therefore reads every
// plane as one coalesced 512-byte (float4) or 512-byte (double2) transaction.
//
//   format        link planes (per mu)                       E planes (per mu)
//   SU2 FP32      1 x float4  (q0,q1,q2,q3)                  3 x float  (E^0..E^2)
//   SU2 FP64      2 x double2 (q0,q1),(q2,q3)                3 x double
//   SU3 FP32      3 x float4, rows 0 and 1 only:             2 x float4 (E^0..3),(E^4..7)
//                 (u00,u01),(u02,u10),(u11,u12);
//                 row 2 = conj(row0 x row1) on load
//   SU3 FP64      9 x double2, all entries, row-major        4 x double2
//
// Bytes per link (U + E): SU2 FP32 16+12, SU2 FP64 32+24, SU3 FP32 48+32,
// SU3 FP64 144+64.
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

template <> struct Fmt<FMT_SU2_F32> {
    using T = float;
    using G = SU2<float>;
    using Mat = G::Mat;
    static constexpr int NA = 3, U_REALS = 4, E_REALS = 3, U_PLANE_BYTES = 16, E_PLANE_BYTES = 12;
    static TCYM_HD Mat load(const void *U, int64_t V, int mu, int64_t s) {
        float4 v = static_cast<const float4 *>(U)[mu * V + s];
        return Mat{{v.x, v.y, v.z, v.w}};
    }
    static TCYM_HD void store(void *U, int64_t V, int mu, int64_t s, const Mat &m) {
        static_cast<float4 *>(U)[mu * V + s] = make_float4(m.q[0], m.q[1], m.q[2], m.q[3]);
    }
    static TCYM_HD void load_e(const void *E, int64_t V, int mu, int64_t s, T *e) {
        const float *p = static_cast<const float *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) e[a] = p[(mu * 3 + a) * V + s];
    }
    static TCYM_HD void store_e(void *E, int64_t V, int mu, int64_t s, const T *e) {
        float *p = static_cast<float *>(E);
#pragma unroll
        for (int a = 0; a < 3; ++a) p[(mu * 3 + a) * V + s] = e[a];
    }
};

template <> struct Fmt<FMT_SU2_F64> {
    using T = double;
    using G = SU2<double>;
    using Mat = G::Mat;
    static constexpr int NA = 3, U_REALS = 4, E_REALS = 3;
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

template <> struct Fmt<FMT_SU3_F32> {
    using T = float;
    using G = SU3<float>;
    using Mat = G::Mat;
    static constexpr int NA = 8, U_REALS = 12, E_REALS = 8;
    static TCYM_HD Mat load(const void *U, int64_t V, int mu, int64_t s) {
        const float4 *p = static_cast<const float4 *>(U);
        float4 a = p[(mu * 3) * V + s], b = p[(mu * 3 + 1) * V + s], c = p[(mu * 3 + 2) * V + s];
        Mat m;
        m.m[0][0] = cx<float>{a.x, a.y}; m.m[0][1] = cx<float>{a.z, a.w};
        m.m[0][2] = cx<float>{b.x, b.y}; m.m[1][0] = cx<float>{b.z, b.w};
        m.m[1][1] = cx<float>{c.x, c.y}; m.m[1][2] = cx<float>{c.z, c.w};
        G::complete_row2(m);
        return m;
    }
    static TCYM_HD void store(void *U, int64_t V, int mu, int64_t s, const Mat &m) {
        float4 *p = static_cast<float4 *>(U);
        p[(mu * 3) * V + s] = make_float4(m.m[0][0].re, m.m[0][0].im, m.m[0][1].re, m.m[0][1].im);
        p[(mu * 3 + 1) * V + s] = make_float4(m.m[0][2].re, m.m[0][2].im, m.m[1][0].re, m.m[1][0].im);
        p[(mu * 3 + 2) * V + s] = make_float4(m.m[1][1].re, m.m[1][1].im, m.m[1][2].re, m.m[1][2].im);
    }
    static TCYM_HD void load_e(const void *E, int64_t V, int mu, int64_t s, T *e) {
        const float4 *p = static_cast<const float4 *>(E);
        float4 a = p[(mu * 2) * V + s], b = p[(mu * 2 + 1) * V + s];
        e[0] = a.x; e[1] = a.y; e[2] = a.z; e[3] = a.w;
        e[4] = b.x; e[5] = b.y; e[6] = b.z; e[7] = b.w;
    }
    static TCYM_HD void store_e(void *E, int64_t V, int mu, int64_t s, const T *e) {
        float4 *p = static_cast<float4 *>(E);
        p[(mu * 2) * V + s] = make_float4(e[0], e[1], e[2], e[3]);
        p[(mu * 2 + 1) * V + s] = make_float4(e[4], e[5], e[6], e[7]);
    }
};

template <> struct Fmt<FMT_SU3_F64> {
    using T = double;
    using G = SU3<double>;
    using Mat = G::Mat;
    static constexpr int NA = 8, U_REALS = 18, E_REALS = 8;
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
