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

// Periodic neighbourhood of one site: wrapped coordinates x-1, x, x+1 (etc.).
struct Nbhd {
    int xs[3], ys[3], zs[3];
    int nx, ny;
    TCYM_HD Nbhd(const Geom &g, int64_t s) {
        nx = g.nx; ny = g.ny;
        int x = (int)(s % g.nx);
        int64_t r = s / g.nx;
        int y = (int)(r % g.ny);
        int z = (int)(r / g.ny);
        xs[0] = x == 0 ? g.nx - 1 : x - 1; xs[1] = x; xs[2] = x == g.nx - 1 ? 0 : x + 1;
        ys[0] = y == 0 ? g.ny - 1 : y - 1; ys[1] = y; ys[2] = y == g.ny - 1 ? 0 : y + 1;
        zs[0] = z == 0 ? g.nz - 1 : z - 1; zs[1] = z; zs[2] = z == g.nz - 1 ? 0 : z + 1;
    }
    // site at offset (dx,dy,dz), each in {-1,0,1}
    TCYM_HD int64_t at(int dx, int dy, int dz) const {
        return (int64_t)xs[dx + 1] + (int64_t)nx * ((int64_t)ys[dy + 1] + (int64_t)ny * zs[dz + 1]);
    }
    TCYM_HD int64_t off(const int *d) const { return at(d[0], d[1], d[2]); }
    TCYM_HD int parity() const { return (xs[1] + ys[1] + zs[1]) & 1; }
};

TCYM_HD void unit(int mu, int *d) { d[0] = mu == 0; d[1] = mu == 1; d[2] = mu == 2; }

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
