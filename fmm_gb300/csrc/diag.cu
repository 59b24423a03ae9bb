// Diagnostics entry points: tree export, FMA-rate measurement, launch count.
#include <vector>

#include "internal.h"

namespace fmm {

thread_local int64_t g_launches = 0;

namespace {

__global__ void k_perm_leaf(int64_t n, const uint32_t* __restrict__ perm, const int32_t* __restrict__ leaf_sorted,
                            int32_t* __restrict__ leaf_orig) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) leaf_orig[perm[k]] = leaf_sorted[k];
}

__global__ void k_expand_pairs(int M, const int32_t* __restrict__ off, const int32_t* __restrict__ src,
                               int32_t* __restrict__ pairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    for (int q = off[i]; q < off[i + 1]; ++q) {
        pairs[2 * q] = i;
        pairs[2 * q + 1] = src[q];
    }
}

template <typename R>
__global__ void k_fma_rate(int iters, R seed, R* out) {
    R a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
      a7 = a0 + 7;
    const R b = (R)0.999999, c = (R)1e-7;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            a0 = a0 * b + c;
            a1 = a1 * b + c;
            a2 = a2 * b + c;
            a3 = a3 * b + c;
            a4 = a4 * b + c;
            a5 = a5 * b + c;
            a6 = a6 * b + c;
            a7 = a7 * b + c;
        }
    }
    const R s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == (R)-12345) out[0] = s;  // keeps the loop alive
}

}  // namespace

void count_launches(int k) { g_launches += k; }

}  // namespace fmm

using namespace fmm;

extern "C" {

int64_t fmm_launch_count(void) { return g_launches; }

int fmm_debug_tree(int64_t n, const double* X, int ncrit, double theta, int centroid_mode, int64_t* sizes,
                   double* center, double* r, double* rmax, int32_t* depth, int32_t* parent, int32_t* is_leaf,
                   int32_t* count, int32_t* leaf_of, int32_t* far_pairs, int32_t* near_pairs) {
    if (n < 2 || ncrit < 1 || !(theta > 0) || !X || !sizes) return FMM_EINVAL;
    Workspace& ws = thread_workspace();
    cudaStream_t st = nullptr;
    FMM_TRY(ws.in_coords.ensure(sizeof(double) * 3 * n));
    FMM_CUDA_TRY(cudaMemcpy(ws.in_coords.p, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
    TreeParams tp{ncrit, theta, centroid_mode, 0, {0, 0, 0}, 0, 0.0, 0};
    if (centroid_mode == 0) {
        host_centroid_sequential(X, n, tp.host_centroid);
        tp.have_host_centroid = 1;
    }
    TreeDev t;
    FMM_TRY(build_tree(ws, ws.in_coords.as<double>(), n, tp, t, st));
    FMM_TRY(build_lists(ws, t, tp, st));
    sizes[0] = t.num_nodes;
    sizes[1] = t.nfar;
    sizes[2] = t.nnear;
    sizes[3] = t.max_depth;
    if (!center) return FMM_OK;
    const int M = t.num_nodes;
    std::vector<double> cx(M), cy(M), cz(M);
    FMM_CUDA_TRY(cudaMemcpy(cx.data(), t.cx, sizeof(double) * M, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(cy.data(), t.cy, sizeof(double) * M, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(cz.data(), t.cz, sizeof(double) * M, cudaMemcpyDeviceToHost));
    for (int k = 0; k < M; ++k) {
        center[3 * k] = cx[k];
        center[3 * k + 1] = cy[k];
        center[3 * k + 2] = cz[k];
    }
    FMM_CUDA_TRY(cudaMemcpy(r, t.r, sizeof(double) * M, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(rmax, t.rmax, sizeof(double) * M, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(depth, t.depth, sizeof(int32_t) * M, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(parent, t.parent, sizeof(int32_t) * M, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(is_leaf, t.is_leaf, sizeof(int32_t) * M, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(count, t.count, sizeof(int32_t) * M, cudaMemcpyDeviceToHost));
    DevBuf tmp;
    const int64_t need = std::max<int64_t>(n, 2 * std::max(t.nfar, t.nnear));
    FMM_TRY(tmp.ensure(sizeof(int32_t) * (size_t)need));
    k_perm_leaf<<<(unsigned)((n + 255) / 256), 256>>>(n, t.perm, t.leaf_of, tmp.as<int32_t>());
    FMM_CUDA_TRY(cudaMemcpy(leaf_of, tmp.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    if (t.nfar > 0) {
        k_expand_pairs<<<(M + 255) / 256, 256>>>(M, t.far_off, t.far_src, tmp.as<int32_t>());
        FMM_CUDA_TRY(cudaMemcpy(far_pairs, tmp.p, sizeof(int32_t) * 2 * t.nfar, cudaMemcpyDeviceToHost));
    }
    if (t.nnear > 0) {
        k_expand_pairs<<<(M + 255) / 256, 256>>>(M, t.near_off, t.near_src, tmp.as<int32_t>());
        FMM_CUDA_TRY(cudaMemcpy(near_pairs, tmp.p, sizeof(int32_t) * 2 * t.nnear, cudaMemcpyDeviceToHost));
    }
    tmp.release();
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int fmm_measure_fma_peak(int precision, double* tflops) {
    if (!tflops || precision < 0 || precision > 1) return FMM_EINVAL;
    int dev = 0, sms = 0;
    FMM_CUDA_TRY(cudaGetDevice(&dev));
    FMM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DevBuf out;
    FMM_TRY(out.ensure(64));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = sms * 8;
    const int iters = precision == 0 ? 256 : 8192;
    double best = 0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (precision == 0)
            k_fma_rate<double><<<blocks, threads>>>(iters, 1.0, out.as<double>());
        else
            k_fma_rate<float><<<blocks, threads>>>(iters, 1.0f, out.as<float>());
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 64.0 * iters * (double)threads * blocks;
        if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    out.release();
    FMM_CUDA_TRY(cudaGetLastError());
    *tflops = best;
    return FMM_OK;
}

}  // extern "C"
