// Fixed-order final reduction of the per-block partial records and the
// Kahan-compensated N_CS accumulator (FP64, on the device).
#include "tcym_batch.cuh"

namespace tcym {

// One block: thread t sums partials t, t+256, ... in order, then a fixed
// shared-memory tree combines the 256 thread sums.  The order depends only on
// the number of partials, never on scheduling.  Thread 0 writes the result
// block and returns E.B and the N_CS sum through *edb / *ncs when given.
__device__ void finalize_block(const double *partial, int blocks, int na, int64_t V, double ncs_dt, double *res,
                               double *edb, double *ncs) {
    __shared__ double sh[kRedThreads][P_WIDTH];
    double v[P_WIDTH];
    for (int k = 0; k < P_WIDTH; ++k) v[k] = 0.0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x)
        for (int k = 0; k < P_WIDTH; ++k) {
            double x = partial[(int64_t)b * P_WIDTH + k];
            v[k] = k < P_GMAX ? v[k] + x : fmax(v[k], x);
        }
    for (int k = 0; k < P_WIDTH; ++k) sh[threadIdx.x][k] = v[k];
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < P_WIDTH; ++k) {
                double a = sh[threadIdx.x][k], b = sh[threadIdx.x + w][k];
                sh[threadIdx.x][k] = k < P_GMAX ? a + b : fmax(a, b);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double *t = sh[0];
        const double inv = 1.0 / (double)V;
        bool bad = false;
        for (int k = 0; k < P_WIDTH; ++k) bad |= !isfinite(t[k]);
        for (int m = 0; m < 3; ++m) { res[R_ESQ0 + m] = t[P_ESQ0 + m] * inv; res[R_BSQ0 + m] = t[P_BSQ0 + m] * inv; }
        res[R_GMAX] = t[P_GMAX];
        res[R_GRMS] = sqrt(t[P_GSQ] / ((double)na * (double)V));
        res[R_GABS] = t[P_GABS];
        res[R_UMAX] = t[P_UMAX];
        res[R_URMS] = sqrt(t[P_USQ] / (3.0 * (double)V));
        res[R_EDB] = t[P_EDB];
        res[R_NONFINITE] = bad ? 1.0 : res[R_NONFINITE];
        if (ncs_dt != 0.0) {
            // Kahan: sum += ncs_dt * E.B / (8 pi^2) with running compensation
            const double inv8pi2 = 0.125 / (3.14159265358979323846 * 3.14159265358979323846);
            double y = ncs_dt * t[P_EDB] * inv8pi2 - res[R_NCS_COMP];
            double s = res[R_NCS] + y;
            res[R_NCS_COMP] = (s - res[R_NCS]) - y;
            res[R_NCS] = s;
        }
        if (edb) *edb = res[R_EDB];
        if (ncs) *ncs = res[R_NCS];
    }
}

__global__ void __launch_bounds__(kRedThreads) k_finalize(const double *partial, int blocks, int na, int64_t V,
                                                          double ncs_dt, double *res) {
    finalize_block(partial, blocks, na, V, ncs_dt, res, nullptr, nullptr);
}

__global__ void __launch_bounds__(kRedThreads) k_finalize_restore(const double *partial, int blocks, int na,
                                                                  int64_t V, double *res, double *ctl, double tol,
                                                                  int it, int check) {
    if ((double)it >= ctl[0]) return;  // the same value for every thread
    finalize_block(partial, blocks, na, V, 0.0, res, nullptr, nullptr);
    if (threadIdx.x == 0) {
        const double gmax = res[R_GMAX];
        const bool bad = res[R_NONFINITE] != 0.0 || !(gmax == gmax);
        if (bad) ctl[1] = 1.0;
        if (bad || (check && gmax <= tol)) ctl[0] = fmin(ctl[0], (double)(it + 1));
    }
}

cudaError_t finalize_restore(const double *partial, int blocks, int na, int64_t V, double *result, double *ctl,
                             double tol, int it, bool check, cudaStream_t st) {
    k_finalize_restore<<<1, kRedThreads, 0, st>>>(partial, blocks, na, V, result, ctl, tol, it, check ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t preload_finalize() {
    cudaFuncAttributes fa;
    return cudaFuncGetAttributes(&fa, k_finalize);
}

cudaError_t finalize_obs(const double *partial, int blocks, int na, int64_t V, double ncs_dt, double *result,
                         cudaStream_t st) {
    k_finalize<<<1, kRedThreads, 0, st>>>(partial, blocks, na, V, ncs_dt, result);
    return cudaGetLastError();
}

// One block per member; out[2i] = E.B, out[2i+1] = N_CS of member i.
__global__ void __launch_bounds__(kRedThreads) k_finalize_members(const MemberReduce *items, double *out) {
    const MemberReduce it = items[blockIdx.x];
    finalize_block(it.partial + (int64_t)it.red_begin * P_WIDTH, it.red_blocks, it.na, it.V, it.ncs_dt, it.result,
                   out ? out + 2 * blockIdx.x : nullptr, out ? out + 2 * blockIdx.x + 1 : nullptr);
}

cudaError_t finalize_members(const MemberReduce *items, int n, double *out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_finalize_members<<<n, kRedThreads, 0, st>>>(items, out);
    return cudaGetLastError();
}

}  // namespace tcym
