// Direct sum on sampled targets without any device allocation.
//
// Some callers cannot let the library call cudaMalloc: host codes whose
// memory manager has already reserved the whole device (a framework's caching
// allocator, or a QM/MM or MD program that sized its pools at start-up), and
// codes that must not trigger the device synchronisation that cudaMalloc and
// cudaFree may imply.  fmm_field_direct_targets_noalloc serves them: it takes
// the same device arrays as fmm_field_direct_targets_device and keeps its
// only scratch (the per-split partial sums and a status word) in a file-scope
// static device array of fixed size, so it allocates nothing.
//
// The array lives in every GPU that loads this library, until the process
// exits.  In host code its name is only a host-side stand-in, so its device
// address is looked up with cudaGetSymbolAddress once per device (on the first
// call made with that device current) and passed to the kernels.  All calls
// share the array: two calls whose work overlaps on the GPU (e.g. on two
// streams) race on it.
#include <algorithm>
#include <mutex>

#include "dispatch.cuh"
#include "internal.h"
#include "pair.cuh"

namespace fmm {

namespace {

// 4 MiB: 2^19 doubles.  The first 32 doubles hold the status word.
constexpr int64_t kStaticDoubles = int64_t(1) << 19;
constexpr int64_t kStatusDoubles = 32;
constexpr int64_t kPartialDoubles = kStaticDoubles - kStatusDoubles;

static __device__ __align__(256) double g_noalloc_scratch[kStaticDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mutex;
double* g_addr[kMaxDevices] = {};

// Device address of the static scratch for the current device (set-up on the
// first call on each device).
int scratch_address(double** out) {
    int dev = 0;
    FMM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return FMM_ENOTSUP;
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return FMM_ECUDA;
        }
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return FMM_OK;
}

int num_sms_noalloc() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// Same algorithm as the allocating direct sum, but the multipoles are scaled
// by the contraction coefficients while a tile is loaded, so no scaled copy
// of the multipoles is needed.
template <int M, int F>
__global__ void __launch_bounds__(128) k_direct_static(int64_t n, const int64_t* __restrict__ targets, int64_t ntgt,
                                                       const double* __restrict__ X, const double* __restrict__ mp,
                                                       const double* __restrict__ damp, int damp_type, int64_t chunk,
                                                       double* __restrict__ partial, unsigned long long* status) {
    constexpr int NF = nT(F), NM = nT(M);
    constexpr int TILE = 128;
    __shared__ double shx[TILE], shy[TILE], shz[TILE], shd[TILE], shm[NM][TILE];
    const int64_t ti = blockIdx.x * (int64_t)TILE + threadIdx.x;
    const int64_t i0 = ti < ntgt ? targets[ti] : 0;
    const bool in_range = i0 >= 0 && i0 < n;
    if (ti < ntgt && !in_range && blockIdx.y == 0) atomicOr(status, 2ull);
    const bool valid = ti < ntgt && in_range;
    const int64_t i = valid ? i0 : 0;
    const double xi = X[i], yi = X[n + i], zi = X[2 * n + i];
    const double di = damp ? damp[i] : 0.0;
    double acc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) acc[f] = 0.0;
    const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    for (int64_t jt = j0; jt < j1; jt += TILE) {
        const int64_t j = jt + threadIdx.x;
        if (j < j1) {
            shx[threadIdx.x] = X[j];
            shy[threadIdx.x] = X[n + j];
            shz[threadIdx.x] = X[2 * n + j];
            shd[threadIdx.x] = damp ? damp[j] : 0.0;
#pragma unroll
            for (int s = 0; s < NM; ++s) shm[s][threadIdx.x] = src_coef(s) * mp[(size_t)s * n + j];
        }
        __syncthreads();
        const int lim = (int)min((int64_t)TILE, j1 - jt);
        for (int k = 0; k < lim; ++k) {
            if (jt + k == i) continue;
            double m[NM];
#pragma unroll
            for (int s = 0; s < NM; ++s) m[s] = shm[s][k];
            pair_field<M, F, double>(xi - shx[k], yi - shy[k], zi - shz[k], di * shd[k], damp_type, m, acc);
        }
        __syncthreads();
    }
    if (valid) {
#pragma unroll
        for (int f = 0; f < NF; ++f) partial[((size_t)blockIdx.y * NF + f) * ntgt + ti] = acc[f];
    }
}

__global__ void k_reduce_static(int64_t ntgt, int nf, int ks, const double* __restrict__ partial,
                                double* __restrict__ field) {
    const int64_t ti = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ti >= ntgt) return;
    for (int f = 0; f < nf; ++f) {
        double s = 0.0;
        for (int k = 0; k < ks; ++k) s += partial[((size_t)k * nf + f) * ntgt + ti];
        field[(size_t)f * ntgt + ti] = s;
    }
}

// Exclusion fix-up (see the allocating path): subtracts the listed partners
// again and, in reference mode, adds their contribution at R = (1e10,1e10,1e10)
// and the self term.  Indices outside 0..n set the status word and are skipped.
template <int M, int F>
__global__ void k_excl_static(int64_t n, int64_t ntgt, const int64_t* __restrict__ targets,
                              const double* __restrict__ X, const double* __restrict__ mp, int exw,
                              const int32_t* __restrict__ excl, const double* __restrict__ damp, int damp_type,
                              int excl_mode, double* __restrict__ field, unsigned long long* status) {
    constexpr int NF = nT(F), NM = nT(M);
    const int64_t ti = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ti >= ntgt) return;
    const int64_t i = targets[ti];
    if (i < 0 || i >= n) return;  // reported by the direct-sum kernel
    const double xi = X[i], yi = X[n + i], zi = X[2 * n + i];
    const double di = damp ? damp[i] : 0.0;
    double add[NF], sub[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) add[f] = sub[f] = 0.0;
    bool self_listed = false;
    for (int w = 0; w < exw; ++w) {
        const int e = excl[(size_t)w * n + i];
        if (e == 0) continue;
        if (e < 0 || e > n) {
            atomicOr(status, 1ull);
            continue;
        }
        bool dup = false;
        for (int w2 = 0; w2 < w; ++w2)
            if (excl[(size_t)w2 * n + i] == e) dup = true;
        if (dup) continue;
        const int64_t j = e - 1;
        if (j == i) {
            self_listed = true;
            continue;
        }
        double m[NM];
#pragma unroll
        for (int s = 0; s < NM; ++s) m[s] = src_coef(s) * mp[(size_t)s * n + j];
        const double a = di * (damp ? damp[j] : 0.0);
        pair_field_cold<M, F, double>(xi - X[j], yi - X[n + j], zi - X[2 * n + j], a, damp_type, m, sub);
        if (excl_mode == 0) pair_field_cold<M, F, double>(1e10, 1e10, 1e10, a, damp_type, m, add);
    }
    if (excl_mode == 0) {
        double m[NM];
#pragma unroll
        for (int s = 0; s < NM; ++s) m[s] = src_coef(s) * mp[(size_t)s * n + i];
        if (self_listed)
            pair_field_cold<M, F, double>(1e10, 1e10, 1e10, di * di, damp_type, m, add);
        else
            pair_field_cold<M, F, double>(0.0, 0.0, 0.0, di * di, damp_type, m, add);
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) field[(size_t)f * ntgt + ti] += add[f] - sub[f];
}

// Every exclusion entry of every particle (not only the targets' rows) must be
// 0 or a 1-based particle index, as the allocating entry points require; a bad
// entry sets status bit 1 and the call returns FMM_EINVAL.
__global__ void k_check_excl_static(int64_t n, int exw, const int32_t* __restrict__ excl,
                                    unsigned long long* status) {
    const int64_t total = n * (int64_t)exw;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int e = excl[q];
        if (e < 0 || e > n) {
            atomicOr(status, 1ull);
            return;
        }
    }
}

int parse_damp_noalloc(const char* s, int len, int* out) {
    int l = (s && len > 0) ? len : 0;
    while (l > 0 && (s[l - 1] == ' ' || s[l - 1] == '\0')) --l;
    auto is = [&](const char* w) {
        int k = 0;
        while (w[k]) ++k;
        if (k != l) return false;
        for (int q = 0; q < k; ++q)
            if (s[q] != w[q]) return false;
        return true;
    };
    if (l == 0) *out = DAMP_NONE;
    else if (is("AMOEBA")) *out = DAMP_AMOEBA;
    else if (is("THOLE")) *out = DAMP_THOLE;
    else if (is("ERF")) *out = DAMP_ERF;
    else return FMM_EINVAL;
    return FMM_OK;
}

}  // namespace

}  // namespace fmm

using namespace fmm;

extern "C" int fmm_field_direct_targets_noalloc(int64_t n, const double* d_X, int mdim, const double* d_mp, int exw,
                                                const int32_t* d_ex, int64_t ntgt, const int64_t* d_targets,
                                                int field_order, double* d_field, const char* damp, int damp_len,
                                                const double* d_damp, const fmm_opts* opts) {
    int dt = 0;
    FMM_TRY(parse_damp_noalloc(damp, damp_len, &dt));
    const int m = dim_to_order(mdim);
    // the same argument checks as the allocating entry points
    if (n < 1 || n > (int64_t)INT32_MAX - 1 || m < 0 || exw < 0 || field_order < 0 || ntgt < 1 || !d_targets ||
        !d_X || !d_mp || !d_field)
        return FMM_EINVAL;
    if (m > 3 || field_order > 3) return FMM_ENOTSUP;
    if (dt != DAMP_NONE && !d_damp) return FMM_EINVAL;
    if (exw > 0 && !d_ex) return FMM_EINVAL;
    int excl_mode = 0;
    cudaStream_t st = nullptr;
    if (opts) {
        if (opts->version != 0 && opts->version != 1) return FMM_EINVAL;
        if (opts->excl_mode < 0 || opts->excl_mode > 1) return FMM_EINVAL;
        excl_mode = opts->excl_mode;
        st = (cudaStream_t)opts->stream;
    }
    const int nf = nT(field_order);
    if (ntgt * nf > kPartialDoubles) return FMM_EINVAL;  // beyond the static scratch
    double* scratch = nullptr;
    FMM_TRY(scratch_address(&scratch));
    unsigned long long* status = reinterpret_cast<unsigned long long*>(scratch);
    double* partial = scratch + kStatusDoubles;
    // split the sources so that the grid covers the GPU, within the scratch
    const int64_t tblocks = (ntgt + 127) / 128;
    int64_t ks = std::max<int64_t>(1, (8LL * num_sms_noalloc() + tblocks - 1) / tblocks);
    ks = std::min<int64_t>(ks, std::max<int64_t>(1, n / 256));
    ks = std::min<int64_t>(ks, kPartialDoubles / (ntgt * nf));
    ks = std::max<int64_t>(1, std::min<int64_t>(ks, 65535));
    const int64_t chunk = (n + ks - 1) / ks;
    const double* dd = dt != DAMP_NONE ? d_damp : nullptr;
    FMM_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned long long), st));
    if (exw > 0) {
        const int64_t total = n * (int64_t)exw;
        const unsigned cb = (unsigned)std::min<int64_t>((total + 255) / 256, 4LL * num_sms_noalloc());
        count_launches(1);
        k_check_excl_static<<<cb, 256, 0, st>>>(n, exw, d_ex, status);
    }
    dim3 grid((unsigned)tblocks, (unsigned)ks);
    FMM_MF_SWITCH_F64(m, field_order,
                  (k_direct_static<MM, FF><<<grid, 128, 0, st>>>(n, d_targets, ntgt, d_X, d_mp, dd, dt, chunk,
                                                                 partial, status)));
    count_launches(1);
    k_reduce_static<<<grid_for(ntgt, 256), 256, 0, st>>>(ntgt, nf, (int)ks, partial, d_field);
    if (exw > 0 || excl_mode == 0) {
        FMM_MF_SWITCH_F64(m, field_order,
                      (k_excl_static<MM, FF><<<grid_for(ntgt, 128), 128, 0, st>>>(
                          n, ntgt, d_targets, d_X, d_mp, exw, d_ex, dd, dt, excl_mode, d_field, status)));
    }
    FMM_CUDA_TRY(cudaGetLastError());
    unsigned long long h = 0;
    FMM_CUDA_TRY(cudaMemcpyAsync(&h, status, sizeof(h), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    return h ? FMM_EINVAL : FMM_OK;
}
