// Order of operations of a step whose state starts and ends in host memory
// (tcym_leapfrog_host): upload, step and download as one pipeline over chunks
// of the storage index (site pairs of the paired FP32 step, sites otherwise).
//
// The storage index i runs over N units in z-planes of P units (P = nx ny for
// sites and for the pairs of the paired layout alike); the stencil of unit i
// lies in the plane of i and the planes next to it, periodic in z (units of
// the first plane reach the last plane, units of the last the first).
// Chunks [jC, min(N, (j + 1) C)) are uploaded in order; chunk j is stepped
// (and then downloaded) as soon as the uploads cover every plane up to the
// one after the plane of its last unit; chunks holding a unit of the first
// plane wait for every upload.  Host-only code (the library and the host
// check build use it).
#pragma once
#include <cstdint>

namespace tcym {

enum PipeOp { PIPE_UPLOAD = 0, PIPE_STEP = 1 };

inline int64_t pipe_chunks(int64_t N, int64_t C) { return (N + C - 1) / C; }

// fn(PIPE_UPLOAD or PIPE_STEP, chunk) in issue order; every chunk once each
template <class Fn> void pipeline_schedule(int64_t N, int64_t P, int64_t C, Fn &&fn) {
    const int64_t n = pipe_chunks(N, C);
    auto hi = [&](int64_t j) { return (j + 1) * C < N ? (j + 1) * C : N; };
    int64_t first = 0;  // chunks [0, first) hold a unit of the first plane
    while (first < n && first * C < P) ++first;
    // uploads chunk j needs: through the plane after the plane of its last unit
    auto need = [&](int64_t j) {
        const int64_t end = ((hi(j) - 1) / P + 2) * P;
        return end < N ? end : N;
    };
    int64_t next = first;
    for (int64_t k = 0; k < n; ++k) {
        fn(PIPE_UPLOAD, k);
        const int64_t up = hi(k);
        while (next < n && up >= need(next)) fn(PIPE_STEP, next++);
    }
    for (int64_t j = 0; j < first; ++j) fn(PIPE_STEP, j);
}

}  // namespace tcym
