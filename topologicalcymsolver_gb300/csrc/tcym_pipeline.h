// Order of operations of a step whose state starts and ends in host memory
// (tcym_leapfrog_host): upload, step and download as one pipeline over chunks
// of the storage index (site pairs of the paired FP32 step, sites otherwise).
//
// The storage index i runs over N units in z-planes of P units (P = nx ny for
// sites and for the pairs of the paired layout alike); the stencil of unit i
// lies in the plane of i and the planes next to it, periodic in z (units of
// the first plane reach the last plane, units of the last the first).
// Chunks [b_j, b_{j+1}) are uploaded in order; chunk j is stepped (and then
// downloaded) as soon as the uploads cover every plane up to the one after
// the plane of its last unit; chunks holding a unit of the first plane wait
// for every upload.  Host-only code (the library and the host check build use
// it).
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

namespace tcym {

enum PipeOp { PIPE_UPLOAD = 0, PIPE_STEP = 1 };

// Chunk bounds b_0 = 0 < b_1 < ... = N, multiples of 128 but the last: chunks
// of about one plane at both ends, where only one transfer direction has work
// (before the first step can start, after the last upload), C in between.
inline std::vector<int64_t> pipeline_bounds(int64_t N, int64_t P, int64_t C) {
    const int64_t S = std::min(C, std::max<int64_t>(128, (P + 127) / 128 * 128));
    std::vector<int64_t> b{0};
    int64_t x = 0;
    auto push = [&](int64_t step) {
        x = x + step < N ? x + step : N;
        b.push_back(x);
    };
    for (int i = 0; i < 3 && x < N; ++i) push(S);  // the ramp up
    while (N - x > 3 * S + C) push(C);
    while (x < N) push(S);                          // the ramp down
    return b;
}

// fn(PIPE_UPLOAD or PIPE_STEP, chunk) in issue order; every chunk once each
template <class Fn> void pipeline_schedule(const std::vector<int64_t> &b, int64_t P, Fn &&fn) {
    const int64_t n = (int64_t)b.size() - 1, N = b.back();
    int64_t first = 0;  // chunks [0, first) hold a unit of the first plane
    while (first < n && b[first] < P) ++first;
    // uploads chunk j needs: through the plane after the plane of its last unit
    auto need = [&](int64_t j) {
        const int64_t end = ((b[j + 1] - 1) / P + 2) * P;
        return end < N ? end : N;
    };
    int64_t next = first;
    for (int64_t k = 0; k < n; ++k) {
        fn(PIPE_UPLOAD, k);
        while (next < n && b[k + 1] >= need(next)) fn(PIPE_STEP, next++);
    }
    for (int64_t j = 0; j < first; ++j) fn(PIPE_STEP, j);
}

}  // namespace tcym
