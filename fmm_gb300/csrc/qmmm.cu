// QM/MM helpers of the reference (src/fmm.F90:1134-1336) on the GPU.
//
// get_boxes / get_multipoles split the particles of an octree into a near
// field (the particles of leaves close to any QM target point) and a far
// field (the boxes whose multipoles stand in for their particles), with the
// reference's recursive test classify_box (fmm.F90:1134-1171): a node with a
// target point within rmax / theta of its centre is refined, a leaf that is
// still too close contributes its particles, any other node its box.
// interpolate_electron_fields carries local expansions given at boxes down the
// tree (L2L) and evaluates them at the particles (L2P).
//
// The octree is the reference's (sequential centroid, the same node order),
// so box indices are the reference's 1-based node numbers.  Near-field
// particles are listed leaf by leaf in node order; within a leaf in ascending
// particle index (the reference lists them in its insertion order, which
// depends on when the leaf's ancestors split).
#include <algorithm>
#include <vector>

#include <cub/cub.cuh>

#include "internal.h"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// too_close[node]: a target point within rmax / theta of the node centre
// (r * theta <= rmax, fmm.F90:1151-1157); one warp per node.
__global__ void k_too_close(const TreeDev t, const double* __restrict__ T, int64_t ntgt, double theta,
                            int32_t* __restrict__ too_close) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= t.num_nodes) return;
    const double cx = t.cx[w], cy = t.cy[w], cz = t.cz[w], rm = t.rmax[w];
    bool close = false;
    for (int64_t i = lane; i < ntgt; i += 32) {
        const double r = norm2_3(__dsub_rn(T[i], cx), __dsub_rn(T[ntgt + i], cy), __dsub_rn(T[2 * ntgt + i], cz));
        close |= __dmul_rn(r, theta) <= rm;
    }
    close = __any_sync(0xffffffffu, close);
    if (lane == 0) too_close[w] = close ? 1 : 0;
}

// Classification: a node is reached when every ancestor was too close; a
// reached node that is too close is refined (type 0) or, as a leaf, gives its
// particles (type 2); a reached node that is not too close gives its box
// (type 1).  Also the per-node counts for the output offsets.
__global__ void k_classify(const TreeDev t, const int32_t* __restrict__ too_close, int32_t* __restrict__ type,
                           int32_t* __restrict__ near_cnt, int32_t* __restrict__ box_cnt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t.num_nodes) return;
    bool reached = true;
    for (int a = t.parent[k]; a >= 0; a = t.parent[a]) reached &= too_close[a] != 0;
    int ty = 0;
    if (reached) ty = too_close[k] ? (t.is_leaf[k] ? 2 : 0) : 1;
    type[k] = ty;
    near_cnt[k] = ty == 2 ? t.count[k] : 0;
    box_cnt[k] = ty == 1 ? 1 : 0;
}

// Outputs in node order: near-field particles (1-based original indices,
// ascending within a leaf) and the boxes (centres, 1-based node numbers).
__global__ void k_box_outputs(const TreeDev t, const int32_t* __restrict__ type, const int32_t* __restrict__ near_off,
                              const int32_t* __restrict__ box_off, int64_t nbox, int32_t* __restrict__ idx_near,
                              double* __restrict__ box_c, int32_t* __restrict__ box_idx) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t.num_nodes) return;
    if (type[k] == 2 && idx_near) {
        int32_t* o = idx_near + near_off[k];
        const int s = t.start[k], c = t.count[k];
        for (int q = 0; q < c; ++q) {  // insertion sort of a leaf's (< 64) indices
            const int32_t v = (int32_t)t.perm[s + q] + 1;
            int z = q;
            while (z > 0 && o[z - 1] > v) {
                o[z] = o[z - 1];
                --z;
            }
            o[z] = v;
        }
    }
    if (type[k] == 1) {
        const int b = box_off[k];
        if (box_c) {
            box_c[b] = t.cx[k];
            box_c[nbox + b] = t.cy[k];
            box_c[2 * nbox + b] = t.cz[k];
        }
        if (box_idx) box_idx[b] = k + 1;
    }
}

// Raw Cartesian multipoles of the boxes (M_t = t! M'_t) for one density.
__global__ void k_box_moments(const TreeDev t, const int32_t* __restrict__ type, const int32_t* __restrict__ box_off,
                              int64_t nbox, int nq, const double* __restrict__ mom, double* __restrict__ out) {
    const int k = blockIdx.x;
    if (k >= t.num_nodes || type[k] != 1) return;
    const int b = box_off[k];
    for (int q = threadIdx.x; q < nq; q += blockDim.x)
        out[(size_t)q * nbox + b] = mom[(size_t)k * nq + q] * cfact(comp_x(q)) * cfact(comp_y(q)) * cfact(comp_z(q));
}

// The given local expansions into the nodes' rows (box_idx 1-based).
__global__ void k_set_locals(int64_t nbox, int nq, const double* __restrict__ local, const int32_t* __restrict__ box_idx,
                             double* __restrict__ loc) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nbox * nq) return;
    const int64_t b = e % nbox;
    const int q = (int)(e / nbox);
    loc[(size_t)(box_idx[b] - 1) * nq + q] = local[(size_t)q * nbox + b];
}

struct Classified {
    int64_t nnear = 0, nbox = 0;
};

// Tree of the reference and the classification; node-indexed scratch in
// ws.lattice (type, too_close, two counts and their offsets).
int build_and_classify(Workspace& ws, int64_t n, const double* X, int64_t ntgt, const double* T, double theta,
                       int ncrit, TreeDev& t, Classified& c, int32_t** type_out, int32_t** near_off, int32_t** box_off,
                       cudaStream_t st) {
    FMM_TRY(ws.in_coords.ensure(sizeof(double) * 3 * n));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_coords.p, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    TreeParams tp{ncrit, theta, 0, 1, {0, 0, 0}, 0, 0.0, 0};
    host_centroid_sequential(X, n, tp.host_centroid);
    FMM_TRY(build_tree(ws, ws.in_coords.as<double>(), n, tp, t, st));
    const int M = t.num_nodes;
    FMM_TRY(ws.lattice.ensure(sizeof(int32_t) * 6 * ((size_t)M + 1) + sizeof(double) * 3 * std::max<int64_t>(ntgt, 1)));
    int32_t* too_close = ws.lattice.as<int32_t>();
    int32_t* type = too_close + (M + 1);
    int32_t* ncnt = type + (M + 1);
    int32_t* bcnt = ncnt + (M + 1);
    int32_t* noff = bcnt + (M + 1);
    int32_t* boff = noff + (M + 1);
    double* dT = reinterpret_cast<double*>(ws.lattice.as<int32_t>() + 6 * ((size_t)M + 1));
    FMM_CUDA_TRY(cudaMemcpyAsync(dT, T, sizeof(double) * 3 * ntgt, cudaMemcpyHostToDevice, st));
    count_launches(1);
    k_too_close<<<grid_for((int64_t)M * 32, 128), 128, 0, st>>>(t, dT, ntgt, theta, too_close);
    count_launches(1);
    k_classify<<<grid_for(M, 256), 256, 0, st>>>(t, too_close, type, ncnt, bcnt);
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, ncnt, noff, M + 1, st);
    FMM_TRY(ws.cub_tmp.ensure(std::max<size_t>(tb, 1)));
    FMM_CUDA_TRY(cudaMemsetAsync(ncnt + M, 0, sizeof(int32_t), st));
    FMM_CUDA_TRY(cudaMemsetAsync(bcnt + M, 0, sizeof(int32_t), st));
    FMM_CUDA_TRY(cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tb, ncnt, noff, M + 1, st));
    FMM_CUDA_TRY(cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tb, bcnt, boff, M + 1, st));
    int32_t tot[2] = {0, 0};
    FMM_CUDA_TRY(cudaMemcpyAsync(&tot[0], noff + M, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaMemcpyAsync(&tot[1], boff + M, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    c.nnear = tot[0];
    c.nbox = tot[1];
    *type_out = type;
    *near_off = noff;
    *box_off = boff;
    return FMM_OK;
}

int parse_stream(const fmm_opts* o, cudaStream_t* st) {
    *st = nullptr;
    if (!o) return FMM_OK;
    if (o->version != 0 && o->version != 1) return FMM_EINVAL;
    *st = (cudaStream_t)o->stream;
    return FMM_OK;
}

// Outputs of the classification into host arrays (any may be NULL).
int box_outputs(const TreeDev& t, const Classified& c, const int32_t* type, const int32_t* noff, const int32_t* boff,
                int32_t* idx_near, double* box_c, int32_t* box_idx, cudaStream_t st) {
    if (!idx_near && !box_c && !box_idx) return FMM_OK;
    DevBuf out;
    const size_t bytes = sizeof(int32_t) * (size_t)(c.nnear + c.nbox) + sizeof(double) * 3 * (size_t)c.nbox + 64;
    FMM_TRY(out.ensure(bytes));
    double* d_bc = out.as<double>();
    int32_t* d_in = reinterpret_cast<int32_t*>(d_bc + 3 * c.nbox);
    int32_t* d_bi = d_in + c.nnear;
    count_launches(1);
    k_box_outputs<<<grid_for(t.num_nodes, 128), 128, 0, st>>>(t, type, noff, boff, c.nbox, d_in, d_bc, d_bi);
    int rc = cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ECUDA;
    if (rc == FMM_OK && idx_near && c.nnear > 0 &&
        cudaMemcpyAsync(idx_near, d_in, sizeof(int32_t) * c.nnear, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = FMM_ECUDA;
    if (rc == FMM_OK && box_c && c.nbox > 0 &&
        cudaMemcpyAsync(box_c, d_bc, sizeof(double) * 3 * c.nbox, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = FMM_ECUDA;
    if (rc == FMM_OK && box_idx && c.nbox > 0 &&
        cudaMemcpyAsync(box_idx, d_bi, sizeof(int32_t) * c.nbox, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = FMM_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) rc = FMM_ECUDA;
    out.release();
    return rc;
}

}  // namespace

}  // namespace fmm

using namespace fmm;

extern "C" {

int fmm_get_boxes(int64_t n, const double* X, int64_t ntgt, const double* T, double theta, int ncrit,
                  int expansion_order, int64_t* sizes, int32_t* idx_near, double* box_c, int32_t* box_idx,
                  const fmm_opts* opts) {
    if (n < 1 || n > (int64_t)INT32_MAX - 1 || ntgt < 1 || !X || !T || !sizes || ncrit < 1 || !(theta > 0.0) ||
        expansion_order < 0)
        return FMM_EINVAL;
    cudaStream_t st;
    FMM_TRY(parse_stream(opts, &st));
    Workspace& ws = thread_workspace();
    TreeDev t;
    Classified c;
    int32_t *type, *noff, *boff;
    FMM_TRY(build_and_classify(ws, n, X, ntgt, T, theta, ncrit, t, c, &type, &noff, &boff, st));
    sizes[0] = c.nnear;
    sizes[1] = c.nbox;
    return box_outputs(t, c, type, noff, boff, idx_near, box_c, box_idx, st);
}

int fmm_get_multipoles(int comm, int64_t n, const double* X, int mdim, int ndens, const double* mp, int64_t ntgt,
                       const double* T, double theta, int ncrit, int p, int64_t* sizes, int32_t* idx_near,
                       double* box_c, double* box_mp, const fmm_opts* opts) {
    (void)comm;
    if (n < 1 || n > (int64_t)INT32_MAX - 1 || ntgt < 1 || !X || !T || !mp || !sizes || ncrit < 1 ||
        !(theta > 0.0) || p < 0 || ndens < 1)
        return FMM_EINVAL;
    const int m = dim_to_order(mdim);
    if (m < 0) return FMM_EINVAL;
    if (m > 3 || p > kMaxP) return FMM_ENOTSUP;
    cudaStream_t st;
    FMM_TRY(parse_stream(opts, &st));
    Workspace& ws = thread_workspace();
    TreeDev t;
    Classified c;
    int32_t *type, *noff, *boff;
    FMM_TRY(build_and_classify(ws, n, X, ntgt, T, theta, ncrit, t, c, &type, &noff, &boff, st));
    sizes[0] = c.nnear;
    sizes[1] = c.nbox;
    FMM_TRY(box_outputs(t, c, type, noff, boff, idx_near, box_c, nullptr, st));
    if (!box_mp || c.nbox == 0) return FMM_OK;
    const int nq = nT(p);
    FMM_TRY(ws.in_mp.ensure(sizeof(double) * (size_t)mdim * n));
    DevBuf out;
    FMM_TRY(out.ensure(sizeof(double) * (size_t)c.nbox * nq));
    int rc = FMM_OK;
    for (int k = 0; k < ndens && rc == FMM_OK; ++k) {
        if (cudaMemcpyAsync(ws.in_mp.p, mp + (size_t)k * n * mdim, sizeof(double) * (size_t)mdim * n,
                            cudaMemcpyHostToDevice, st) != cudaSuccess) {
            rc = FMM_ECUDA;
            break;
        }
        Particles P{n, ws.in_coords.as<double>(), mdim, ws.in_mp.as<double>(), 0, nullptr, nullptr, DAMP_NONE};
        if ((rc = gather_sorted(ws, P, t, st)) != FMM_OK) break;
        if ((rc = launch_p2m_m2m(ws, P, t, p, st)) != FMM_OK) break;
        count_launches(1);
        k_box_moments<<<(unsigned)t.num_nodes, 128, 0, st>>>(t, type, boff, c.nbox, nq, ws.mom.as<double>(),
                                                             out.as<double>());
        if (cudaMemcpyAsync(box_mp + (size_t)k * c.nbox * nq, out.p, sizeof(double) * (size_t)c.nbox * nq,
                            cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = FMM_ECUDA;
    }
    out.release();
    return rc;
}

int fmm_interpolate_electron_fields(int comm, int64_t n, const double* X, int64_t nbox, int ndens,
                                    const double* local, const int32_t* box_idx, double theta, int ncrit, int p,
                                    int field_order, double* field, const fmm_opts* opts) {
    (void)comm;
    if (n < 1 || n > (int64_t)INT32_MAX - 1 || nbox < 0 || ndens < 1 || !X || (nbox > 0 && (!local || !box_idx)) ||
        !field || ncrit < 1 || !(theta > 0.0) || p < 0 || field_order < 0)
        return FMM_EINVAL;
    if (p > kMaxP || field_order > p) return FMM_ENOTSUP;
    cudaStream_t st;
    FMM_TRY(parse_stream(opts, &st));
    Workspace& ws = thread_workspace();
    FMM_TRY(ws.in_coords.ensure(sizeof(double) * 3 * n));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_coords.p, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    TreeParams tp{ncrit, theta, 0, 1, {0, 0, 0}, 0, 0.0, 0};
    host_centroid_sequential(X, n, tp.host_centroid);
    TreeDev t;
    FMM_TRY(build_tree(ws, ws.in_coords.as<double>(), n, tp, t, st));
    const int M = t.num_nodes, nq = nT(p), nf = nT(field_order);
    for (int64_t b = 0; b < nbox; ++b)
        if (box_idx[b] < 1 || box_idx[b] > M) return FMM_EINVAL;
    // sorted coordinates (a zero multipole stands in for the unused charges)
    FMM_TRY(ws.in_mp.ensure(sizeof(double) * n));
    FMM_CUDA_TRY(cudaMemsetAsync(ws.in_mp.p, 0, sizeof(double) * n, st));
    Particles P{n, ws.in_coords.as<double>(), 1, ws.in_mp.as<double>(), 0, nullptr, nullptr, DAMP_NONE};
    FMM_TRY(gather_sorted(ws, P, t, st));
    FMM_TRY(ws.loc.ensure(sizeof(double) * (size_t)M * nq));
    FMM_TRY(ws.fsorted.ensure(sizeof(double) * (size_t)n * nf));
    FMM_TRY(ws.out_field.ensure(sizeof(double) * (size_t)n * nf));
    DevBuf dl;
    FMM_TRY(dl.ensure(sizeof(double) * std::max<size_t>(1, (size_t)nbox * nq) + sizeof(int32_t) * (nbox + 1)));
    double* d_local = dl.as<double>();
    int32_t* d_idx = reinterpret_cast<int32_t*>(d_local + std::max<size_t>(1, (size_t)nbox * nq));
    int rc = FMM_OK;
    if (nbox > 0 && cudaMemcpyAsync(d_idx, box_idx, sizeof(int32_t) * nbox, cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = FMM_ECUDA;
    for (int k = 0; k < ndens && rc == FMM_OK; ++k) {
        if (cudaMemsetAsync(ws.loc.p, 0, sizeof(double) * (size_t)M * nq, st) != cudaSuccess ||
            cudaMemsetAsync(ws.fsorted.p, 0, sizeof(double) * (size_t)n * nf, st) != cudaSuccess) {
            rc = FMM_ECUDA;
            break;
        }
        if (nbox > 0) {
            if (cudaMemcpyAsync(d_local, local + (size_t)k * nbox * nq, sizeof(double) * (size_t)nbox * nq,
                                cudaMemcpyHostToDevice, st) != cudaSuccess) {
                rc = FMM_ECUDA;
                break;
            }
            count_launches(1);
            k_set_locals<<<grid_for(nbox * nq, 256), 256, 0, st>>>(nbox, nq, d_local, d_idx, ws.loc.as<double>());
        }
        if ((rc = launch_l2l_l2p(ws, P, t, p, field_order, false, st)) != FMM_OK) break;
        if ((rc = scatter_field(ws, t, n, nf, ws.out_field.as<double>(), st)) != FMM_OK) break;
        if (cudaMemcpyAsync(field + (size_t)k * n * nf, ws.out_field.p, sizeof(double) * (size_t)n * nf,
                            cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = FMM_ECUDA;
    }
    dl.release();
    return rc;
}

}  // extern "C"
