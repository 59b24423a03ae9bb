// C ABI (include/fmm_gpu.h): argument checking, device workspaces and the
// field_fmm / field_direct pipelines.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

#include "internal.h"
#include "mlp.cuh"

namespace fmm {

int DevBuf::ensure(size_t bytes) {
    if (bytes <= cap && p) return FMM_OK;
    release();
    if (bytes == 0) return FMM_OK;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        cap = 0;
        return FMM_ENOMEM;
    }
    cap = bytes;
    return FMM_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

void Workspace::release_buffers(bool keep_selector) {
    DevBuf* all[] = {&in_coords, &in_mp,     &in_excl,     &in_damp,    &out_field,  &keys_a,     &keys_b,
                     &vals_a,    &vals_b,    &cub_tmp,     &perm,       &pos_of,     &leaf_of,    &node_d,
                     &node_i,    &child,     &level_nodes, &leaves,     &node_key,   &node_val,   &node_key2,
                     &node_val2, &counters,  &scalars,     &front_a,    &front_b,    &far_pairs,  &near_pairs,
                     &far_sorted, &near_sorted, &node_dfs, &far_src,    &near_src,   &sx,         &sy,
                     &sz,        &smc,       &sd,          &fsorted,    &mom,        &loc,        &partial,
                     &term_off,  &term_abc,  &term_c, &f32buf, &wred, &far_ord, &sel_norms, &sel_params, &sel_scratch, &sysbuf,
                     &m2l_tgt, &m2l_keys, &m2l_keys2, &m2l_vals, &m2l_vals2, &m2l_ukeys, &m2l_cnt, &m2l_gstart,
                     &m2l_tcnt, &m2l_toff, &m2l_tasks, &m2l_T, &m2l_gq, &m2l_gab, &m2l_wsc, &m2l_out, &m2l_wsplit, &m2l_gop, &m2l_gopoff, &m2l_rowbase, &xlate, &l2pt, &dsmc, &f32node, &lattice, &p2p_order, &p2p_pad, &f32x2, &sel_budget, &corr_pairs, &corr_sorted, &corr_src, &leaf_ext};
    for (DevBuf* b : all)
        if (!(keep_selector && b == &sel_params)) b->release();
    if (!keep_selector) sel_ready = false;
    wred_p = term_order = xlate_p = l2pt_p = l2pt_f = -1;
    node_cap = 0;        // node_d / node_i are gone
    f32node_ok = false;
}

Workspace::~Workspace() {
    release_buffers(false);
    if (events_ready)
        for (auto& e : ev) cudaEventDestroy(e);
    if (aux) cudaStreamDestroy(aux);
    if (copy) cudaStreamDestroy(copy);
    if (copy_ev) cudaEventDestroy(copy_ev);
}

Workspace& thread_workspace() {
    thread_local Workspace ws;
    int dev = 0;
    cudaGetDevice(&dev);
    if (ws.device != dev) {
        ws.~Workspace();
        new (&ws) Workspace();
        ws.device = dev;
    }
    return ws;
}

namespace {

constexpr int kNumStats = 16 + kMaxP + 1 + 6 + 5 + 2;
constexpr int kTuneStats = 16 + kMaxP + 1 + 6;  // ncrit used, near-field shape (3), tuned by this call
struct Stats {
    double v[kNumStats] = {0};
};
thread_local Stats g_stats;

int parse_damp(const char* s, int len, int* out) {
    std::string d = (s && len > 0) ? std::string(s, (size_t)len) : std::string();
    size_t z = d.find('\0');
    if (z != std::string::npos) d.resize(z);
    while (!d.empty() && d.back() == ' ') d.pop_back();
    if (d.empty()) *out = DAMP_NONE;
    else if (d == "AMOEBA") *out = DAMP_AMOEBA;
    else if (d == "THOLE") *out = DAMP_THOLE;
    else if (d == "ERF") *out = DAMP_ERF;
    else return FMM_EINVAL;
    return FMM_OK;
}

struct Opts {
    int coef_mode = 0, excl_mode = 0, precision = 0, centroid_mode = 0, mac_mode = 0, selector = 0, autotune = 0;
    double target = 1e-6;
    cudaStream_t stream = nullptr;
};

int parse_opts(const fmm_opts* o, Opts* out) {
    if (!o) return FMM_OK;
    if (o->version != 0 && o->version != 1) return FMM_EINVAL;
    if (o->coef_mode < 0 || o->coef_mode > 1 || o->excl_mode < 0 || o->excl_mode > 1 || o->precision < 0 ||
        o->precision > 3 || o->centroid_mode < 0 || o->centroid_mode > 1 || o->mac_mode < 0 || o->mac_mode > 1 ||
        o->selector < 0 || o->selector > 1 || o->autotune < 0 || o->autotune > 1)
        return FMM_EINVAL;
    out->coef_mode = o->coef_mode;
    out->excl_mode = o->excl_mode;
    out->precision = o->precision;
    out->centroid_mode = o->centroid_mode;
    out->mac_mode = o->mac_mode;
    out->selector = o->selector;
    out->autotune = o->autotune;
    out->target = o->target_rel_err > 0 ? o->target_rel_err : 1e-6;
    out->stream = (cudaStream_t)o->stream;
    return FMM_OK;
}

int check_common(int64_t n, int mdim, int exw, int field_order, int damp, const double* damping) {
    if (n < 1 || n > (int64_t)INT32_MAX - 1) return FMM_EINVAL;
    const int m = dim_to_order(mdim);
    if (m < 0 || exw < 0 || field_order < 0) return FMM_EINVAL;
    if (m > 3 || field_order > 3) return FMM_ENOTSUP;
    if (damp != DAMP_NONE && !damping) return FMM_EINVAL;
    return FMM_OK;
}

// Exclusion indices must lie in 0..n (0 = unused slot): a branch-free
// minimum / maximum over the array (vectorisable), then one comparison.
int check_exclusions_host(int64_t n, int exw, const int32_t* ex) {
    if (exw > 0 && !ex) return FMM_EINVAL;
    const int64_t total = n * (int64_t)exw;
    int32_t lo = 0, hi = 0;
    for (int64_t q = 0; q < total; ++q) {
        lo = std::min(lo, ex[q]);
        hi = std::max(hi, ex[q]);
    }
    return (lo < 0 || (int64_t)hi > n) ? FMM_EINVAL : FMM_OK;
}

// Populates the pages of a host output buffer from a helper thread while
// the device works, so that the final device-to-host copy does not take the
// first-touch faults of freshly allocated memory (each byte is rewritten with
// its own value).  Joined before the copy, or when leaving the call.
class OutputPrefault {
  public:
    OutputPrefault(void* p, size_t bytes) {
        if (!p || bytes == 0) return;
        try {
            th_ = std::thread([p, bytes] {
                const long pg = sysconf(_SC_PAGESIZE);
                const size_t step = pg > 0 ? (size_t)pg : 4096;
                volatile char* c = static_cast<volatile char*>(p);
                for (size_t k = 0; k < bytes; k += step) c[k] = c[k];
                c[bytes - 1] = c[bytes - 1];
            });
        } catch (...) {
        }
    }
    void join() {
        if (th_.joinable()) th_.join();
    }
    ~OutputPrefault() { join(); }

  private:
    std::thread th_;
};

// Copies the multipoles and exclusions of a host call on the workspace's
// copy stream from a helper thread, so that the transfer overlaps the tree
// build; run_fmm joins it (ws.copy_join) and makes its stream wait for the
// copies before it first reads them.  Without a thread the copies are made
// here.
class DeferredInputCopy {
  public:
    DeferredInputCopy(Workspace& ws, void* d_mp, const void* mp, size_t mp_bytes, void* d_ex, const void* ex,
                      size_t ex_bytes)
        : ws_(ws) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            (!ws.copy && cudaStreamCreateWithFlags(&ws.copy, cudaStreamNonBlocking) != cudaSuccess) ||
            (!ws.copy_ev && cudaEventCreateWithFlags(&ws.copy_ev, cudaEventDisableTiming) != cudaSuccess)) {
            status_ = FMM_ECUDA;
            return;
        }
        auto copy = [this, dev, d_mp, mp, mp_bytes, d_ex, ex, ex_bytes] {
            cudaError_t e = cudaSetDevice(dev);
            if (e == cudaSuccess) e = cudaMemcpyAsync(d_mp, mp, mp_bytes, cudaMemcpyHostToDevice, ws_.copy);
            if (e == cudaSuccess && ex_bytes) e = cudaMemcpyAsync(d_ex, ex, ex_bytes, cudaMemcpyHostToDevice, ws_.copy);
            if (e == cudaSuccess) e = cudaEventRecord(ws_.copy_ev, ws_.copy);
            status_ = e == cudaSuccess ? FMM_OK : FMM_ECUDA;
        };
        started_ = true;
        try {
            th_ = std::thread(copy);
        } catch (...) {
            copy();
        }
        ws_.copy_join = [this] { return join(); };
    }
    bool started() const { return started_; }
    int join() {
        if (th_.joinable()) th_.join();
        return status_;
    }
    ~DeferredInputCopy() {
        join();
        ws_.copy_join = nullptr;
        if (started_ && status_ == FMM_OK) cudaEventSynchronize(ws_.copy_ev);  // no copy outlives the call
    }

  private:
    Workspace& ws_;
    std::thread th_;
    int status_ = FMM_OK;
    bool started_ = false;
};

__global__ void k_check_excl(int64_t total, int64_t n, const int32_t* __restrict__ ex, int* bad) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x)
        if (ex[q] < 0 || ex[q] > n) atomicExch(bad, 1);
}

__global__ void k_check_targets(int64_t ntgt, int64_t n, const int64_t* __restrict__ tg, int* bad) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ntgt; q += (int64_t)gridDim.x * blockDim.x)
        if (tg[q] < 0 || tg[q] >= n) atomicExch(bad, 1);
}

// Validates device-resident target indices (0..n-1).
int check_targets_device(Workspace& ws, int64_t n, int64_t ntgt, const int64_t* d_t, cudaStream_t st) {
    FMM_TRY(ws.counters.ensure(sizeof(unsigned long long) * 16));
    int* flag = reinterpret_cast<int*>(ws.counters.as<unsigned long long>() + 13);
    FMM_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
    count_launches(1);
    k_check_targets<<<(unsigned)std::min<int64_t>(4096, (ntgt + 255) / 256), 256, 0, st>>>(ntgt, n, d_t, flag);
    int h = 0;
    FMM_CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    return h ? FMM_EINVAL : FMM_OK;
}

// Validates device-resident exclusion indices (0 or 1..n) before any kernel uses them.
int check_exclusions_device(Workspace& ws, int64_t n, int exw, const int32_t* d_ex, cudaStream_t st) {
    if (exw == 0) return FMM_OK;
    if (!d_ex) return FMM_EINVAL;
    FMM_TRY(ws.counters.ensure(sizeof(unsigned long long) * 16));
    int* flag = reinterpret_cast<int*>(ws.counters.as<unsigned long long>() + 12);
    FMM_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
    const int64_t total = n * (int64_t)exw;
    count_launches(1);
    k_check_excl<<<(unsigned)std::min<int64_t>(4096, (total + 255) / 256), 256, 0, st>>>(total, n, d_ex, flag);
    int h = 0;
    FMM_CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    return h ? FMM_EINVAL : FMM_OK;
}

void ensure_events(Workspace& ws) {
    if (!ws.events_ready) {
        for (auto& e : ws.ev) cudaEventCreate(&e);
        ws.events_ready = true;
    }
}

// Copies host inputs into the workspace's device buffers (with defer, the
// multipoles and exclusions are left to a DeferredInputCopy).
int upload(Workspace& ws, int64_t n, const double* X, int mdim, const double* mp, int exw, const int32_t* ex,
           const double* damp, int nf, Particles* P, cudaStream_t st, bool defer = false) {
    FMM_TRY(ws.in_coords.ensure(sizeof(double) * 3 * n));
    FMM_TRY(ws.in_mp.ensure(sizeof(double) * (size_t)mdim * n));
    FMM_TRY(ws.in_excl.ensure(sizeof(int32_t) * (size_t)std::max(exw, 1) * n));
    FMM_TRY(ws.in_damp.ensure(sizeof(double) * n));
    FMM_TRY(ws.out_field.ensure(sizeof(double) * (size_t)nf * n));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_coords.p, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (!defer) {
        FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_mp.p, mp, sizeof(double) * (size_t)mdim * n, cudaMemcpyHostToDevice, st));
        if (exw > 0)
            FMM_CUDA_TRY(
                cudaMemcpyAsync(ws.in_excl.p, ex, sizeof(int32_t) * (size_t)exw * n, cudaMemcpyHostToDevice, st));
    }
    if (damp) FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_damp.p, damp, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    P->n = n;
    P->x = ws.in_coords.as<double>();
    P->dim = mdim;
    P->mp = ws.in_mp.as<double>();
    P->exw = exw;
    P->excl = ws.in_excl.as<int32_t>();
    P->damp = damp ? ws.in_damp.as<double>() : nullptr;
    return FMM_OK;
}

__global__ void k_gather_rows(int64_t n, int nf, const double* __restrict__ field, const int64_t* __restrict__ rows,
                              int nr, double* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nr * nf) return;
    const int r = q % nr, f = q / nr;
    out[(size_t)f * nr + r] = field[(size_t)f * n + rows[r]];
}

// Far pairs per expansion order (0..15) into hist.
__global__ void k_order_hist(int64_t m, const uint8_t* __restrict__ ord, unsigned long long* __restrict__ hist) {
    __shared__ unsigned int h[16];
    if (threadIdx.x < 16) h[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[ord[q] & 15], 1u);
    __syncthreads();
    if (threadIdx.x < 16 && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], (unsigned long long)h[threadIdx.x]);
}

constexpr int kCheckTargets = 16;  // sampled particles of the learned-selector check
constexpr double kSelThetaLoose = 0.6;  // default loose acceptance test of the learned selector

// Loose acceptance test of the learned selector: FMM_GB300_SEL_THETA
// overrides the default (tuning; values outside (0, 1) are ignored).
double sel_theta_loose() {
    static const double v = [] {
        const char* e = std::getenv("FMM_GB300_SEL_THETA");
        const double x = e ? std::atof(e) : 0.0;
        return (x > 0.0 && x < 1.0) ? x : kSelThetaLoose;
    }();
    return v;
}
constexpr double kSelPairsPerTarget = 150.0;
constexpr double kSelMargin = 0.6;  // default log10 margin of the per-pair budget

// log10 margin between a pair's predicted error and its budget:
// FMM_GB300_SEL_MARGIN overrides the default (tuning; values outside [0, 3]
// are ignored).
double sel_margin() {
    static const double v = [] {
        const char* e = std::getenv("FMM_GB300_SEL_MARGIN");
        const double x = e ? std::atof(e) : -1.0;
        return (x >= 0.0 && x <= 3.0) ? x : kSelMargin;
    }();
    return v;
}

// Relative RMS error (field columns of order >= 1) of F against R, both
// (ntgt x nf) column-major on the host.
double sampled_rms(const std::vector<double>& F, const std::vector<double>& R, int ntgt, int nf) {
    double acc = 0.0;
    for (int t = 0; t < ntgt; ++t) {
        double d = 0.0, g = 0.0;
        for (int f = 1; f < nf; ++f) {
            const double a = F[(size_t)f * ntgt + t], b = R[(size_t)f * ntgt + t];
            d += (a - b) * (a - b);
            g += b * b;
        }
        acc += g > 0 ? d / g : 0.0;
    }
    return std::sqrt(acc / ntgt);
}

// Periodic boxes (box != null): the 27 images of src/fmm.F90:156-175 in the
// reference's order (a_x outer, a_z inner), each with its own interaction
// lists built from (root, root + H a) (fmm.F90:337-343), its near field with
// the exclusions applied only in the central image (fmm.F90:660-736) and its
// M2L (fmm.F90:861-878); then the lattice sum beyond the images and the
// surface term (fmm.F90:884-979), before L2L and L2P.  FP64 and the fixed
// acceptance rule only.
int run_periodic(Workspace& ws, const Particles& P, int p, int f, const Modes& md, const TreeParams& tpl, TreeDev& t,
                 const Box9& box, cudaStream_t st, int* levels, unsigned long long* d_hist) {
    const int64_t n = P.n;
    const int nf = nT(f), nq = nT(p);
    FMM_TRY(ws.fsorted.ensure(sizeof(double) * (size_t)n * nf));
    FMM_TRY(ws.loc.ensure(sizeof(double) * (size_t)t.num_nodes * nq));
    FMM_CUDA_TRY(cudaMemsetAsync(ws.fsorted.p, 0, sizeof(double) * (size_t)n * nf, st));
    FMM_CUDA_TRY(cudaMemsetAsync(ws.loc.p, 0, sizeof(double) * (size_t)t.num_nodes * nq, st));
    int64_t nfar = 0, nnear = 0, npp = 0;
    for (int ai = -1; ai <= 1; ++ai)
        for (int aj = -1; aj <= 1; ++aj)
            for (int ak = -1; ak <= 1; ++ak) {
                // displacement = matmul(box_matrix, a) (fmm.F90:355, 662)
                for (int c = 0; c < 3; ++c)
                    t.shift[c] = (box.h[c] * ai + box.h[3 + c] * aj) + box.h[6 + c] * ak;
                t.central = (ai == 0 && aj == 0 && ak == 0) ? 1 : 0;
                FMM_TRY(build_lists(ws, t, tpl, st));
                if (t.nfar > 0 && t.far_ord) {  // far pairs per order, summed over the images
                    count_launches(1);
                    k_order_hist<<<(unsigned)std::min<int64_t>(1024, (t.nfar + 255) / 256), 256, 0, st>>>(
                        t.nfar, t.far_ord, d_hist);
                }
                FMM_TRY(launch_p2p_f64(ws, P, t, f, md, st, true));
                if (t.central) FMM_TRY(launch_excl_correction(ws, P, &t, f, md, ws.fsorted.as<double>(), st));
                FMM_TRY(launch_m2l_pairwise(ws, t, p, md, true, st));
                nfar += t.nfar;
                nnear += t.nnear;
                npp += t.near_particle_pairs;
            }
    t.shift[0] = t.shift[1] = t.shift[2] = 0.0;
    t.central = 1;
    int* d_levels = reinterpret_cast<int*>(ws.counters.as<unsigned long long>() + 15);
    FMM_TRY(launch_periodic_lattice(ws, t, p, f, md, box, ws.fsorted.as<double>(), d_levels, st));
    FMM_TRY(launch_l2l_l2p(ws, P, t, p, f, false, st));
    FMM_CUDA_TRY(cudaMemcpyAsync(levels, d_levels, sizeof(int), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    t.nfar = nfar;
    t.nnear = nnear;
    t.near_particle_pairs = npp;
    return FMM_OK;
}

int run_fmm(Workspace& ws, const Particles& P, double theta, int ncrit, int p, int f, const Opts& o,
            const TreeParams& tp, double* d_field, cudaStream_t st, const Box9* box = nullptr) {
    ensure_events(ws);
    ws.product_timed = false;
    ws.m2l_groups = 0;
    const bool learned = o.selector == 1;
    if (learned && !ws.sel_ready) return FMM_ENOTSUP;  // no selector weights loaded
    Modes md{o.coef_mode, o.excl_mode, o.precision};
    if (md.precision != 0 || learned) {
        // the mixed and learned paths mask exclusions and use exact tensors
        md.excl_mode = 1;
        md.coef_mode = 1;
    }
    if (learned && (p < 10 || dim_to_order(P.dim) > 2 || f < 1)) return FMM_ENOTSUP;
    // the FP32 near field and the double-float translations take orders <= 2
    if (md.precision != 0 && (dim_to_order(P.dim) > 2 || f > 2)) return FMM_ENOTSUP;
    TreeParams tpl = tp;
    if (o.mac_mode == 1 && P.damp_type != DAMP_NONE && P.damp) {
        const double dmin = min_damping_factor(ws, P.damp, P.n, st);
        tpl.rdamp = damping_range(P.damp_type, dmin * dmin, dim_to_order(P.dim) + f, 0.1 * o.target);
        // learned lists with the packed FP32 near field, AMOEBA: leaf pairs
        // inside the damping range may be far pairs, their particle pairs
        // inside the range corrected in the near field (FMM_GB300_DAMP_CORR=0:
        // demote them)
        const char* ce = std::getenv("FMM_GB300_DAMP_CORR");
        if (learned && (md.precision == 1 || md.precision == 2) && tpl.rdamp > 0.0 && P.damp_type == DAMP_AMOEBA &&
            p2p_packed_enabled(ws.p2p_shape.valid() ? ws.p2p_shape : P2pShape{}, f, P.damp_type) && !(ce && ce[0] == '0')) {
            tpl.corr_mode = 1;
            // AMOEBA depends on a r only: the range at a = 1 is the cutoff of a r
            const double xc = damping_range(P.damp_type, 1.0, dim_to_order(P.dim) + f, 0.1 * o.target);
            ws.corr_xcut2 = (float)(xc * xc);
        }
    }
    TreeDev t;
    const int nf = nT(f);
    ws.product_err = nullptr;  // set by the tensor-core M2L product, read at the end of the call
    // device counters: flags and counts of the phases (0..15), far pairs per
    // expansion order (16..31)
    FMM_TRY(ws.counters.ensure(sizeof(unsigned long long) * 32));
    unsigned long long* d_hist = ws.counters.as<unsigned long long>() + 16;
    FMM_CUDA_TRY(cudaMemsetAsync(d_hist, 0, sizeof(unsigned long long) * 16, st));
    cudaEventRecord(ws.ev[0], st);
    FMM_TRY(build_tree(ws, P.x, P.n, tp, t, st));
    cudaEventRecord(ws.ev[1], st);
    std::vector<double> ref_rows;
    std::vector<int64_t> rows;
    const int nt = learned ? (int)std::min<int64_t>(kCheckTargets, P.n) : 0;
    if (learned) {
        for (int k = 0; k < nt; ++k) rows.push_back((int64_t)(((uint64_t)k * 2654435761ull + 12345ull) % (uint64_t)P.n));
        FMM_TRY(ws.sel_scratch.ensure(sizeof(double) * (size_t)nt * nf * 2 + sizeof(int64_t) * nt));
        int64_t* d_rows = reinterpret_cast<int64_t*>(ws.sel_scratch.as<double>() + (size_t)nt * nf * 2);
        FMM_CUDA_TRY(cudaMemcpyAsync(d_rows, rows.data(), sizeof(int64_t) * nt, cudaMemcpyHostToDevice, st));
    }
    if (ws.copy_join) {  // multipoles and exclusions copied beside the tree build
        const int cst = ws.copy_join();
        ws.copy_join = nullptr;
        FMM_TRY(cst);
        FMM_CUDA_TRY(cudaStreamWaitEvent(st, ws.copy_ev, 0));
    }
    FMM_TRY(gather_sorted(ws, P, t, st));
    const bool f32_near = md.precision == 1 || md.precision == 2;
    if (f32_near || learned) FMM_TRY(prepare_f32_records(ws, P, t, st));
    FMM_TRY(launch_p2m_m2m(ws, P, t, p, st, md.precision != 0));
    if (learned) {
        FMM_TRY(launch_reduce_moments(ws, t, p, st));
        FMM_TRY(selector_node_norms(ws, t, p, P.damp ? ws.sd.as<double>() : nullptr, st));
        tpl.sel_params = ws.sel_params.as<float>();
        tpl.sel_lnorm = ws.sel_norms.as<float>();
        tpl.sel_dmin = ws.sel_norms.as<float>() + (size_t)t.num_nodes * (p + 1);
        tpl.sel_P = p;
        tpl.sel_chi = ws.f32node.as<float4>();  // prepare_f32_records
        tpl.sel_clo = tpl.sel_chi + t.num_nodes;
        // per-pair error budgets by target node: the truncation share of the
        // target error times half the node's typical local field (geometric
        // mean over its particles), spread over the far pairs a particle sees
        const double floor_fp32 = md.precision == 0 ? 0.0 : 9e-7;
        const double trunc = std::sqrt(std::max(o.target * o.target - floor_fp32 * floor_fp32, 0.04 * o.target * o.target));
        const float base = (float)(std::log10(trunc / std::sqrt(kSelPairsPerTarget)) - sel_margin());
        FMM_TRY(selector_node_budgets(ws, P, t, base, st));
        tpl.sel_budget = ws.sel_budget.as<float>();
        tpl.sel_theta = sel_theta_loose();
        if (tpl.corr_mode) {
            FMM_TRY(launch_leaf_extent(ws, P, t, st));
            tpl.corr_ext = ws.leaf_ext.as<float2>();
            tpl.corr_xcut2 = ws.corr_xcut2;
        }
    }
    cudaEventRecord(ws.ev[2], st);
    bool fallback = false;
    double check_rms = -1.0;
    int lattice_levels = 0;
    if (box) {
        FMM_TRY(run_periodic(ws, P, p, f, md, tpl, t, *box, st, &lattice_levels, d_hist));
        for (int k = 3; k <= 5; ++k) cudaEventRecord(ws.ev[k], st);
        cudaEventRecord(ws.ev[7], st);
        FMM_TRY(scatter_field(ws, t, P.n, nf, d_field, st));
    }
    for (int attempt = 0; attempt < 2 && !box; ++attempt) {
        FMM_TRY(build_lists(ws, t, tpl, st));
        if (learned && attempt == 0) {
            // FP64 direct sums at the sampled particles (the check of the
            // result) on a second stream of higher priority, so its blocks are
            // scheduled first and it runs beside the FP32-bound near field
            // rather than later beside the M2L product
            if (!ws.aux) {
                int lo = 0, hi = 0;
                FMM_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
                FMM_CUDA_TRY(cudaStreamCreateWithPriority(&ws.aux, cudaStreamNonBlocking, hi));
            }
            int64_t* d_rows = reinterpret_cast<int64_t*>(ws.sel_scratch.as<double>() + (size_t)nt * nf * 2);
            cudaEventRecord(ws.ev[10], st);
            FMM_CUDA_TRY(cudaStreamWaitEvent(ws.aux, ws.ev[10], 0));
            Modes mdir{1, 1, 0};
            FMM_TRY(launch_direct_f64(ws, P, f, mdir, ws.sel_scratch.as<double>(), ws.aux, nt, d_rows, 16));
            cudaEventRecord(ws.ev[11], ws.aux);
        }
        cudaEventRecord(ws.ev[3], st);
        if (f32_near)
            FMM_TRY(launch_p2p_f32(ws, P, t, f, st));
        else
            FMM_TRY(launch_p2p_f64(ws, P, t, f, md, st));
        cudaEventRecord(ws.ev[7], st);  // end of the near-field kernel proper
        FMM_TRY(launch_excl_correction(ws, P, &t, f, md, ws.fsorted.as<double>(), st));
        cudaEventRecord(ws.ev[4], st);
        FMM_TRY(launch_m2l(ws, t, p, md, st));
        cudaEventRecord(ws.ev[5], st);
        FMM_TRY(launch_l2l_l2p(ws, P, t, p, f, md.precision == 1 || md.precision == 3, st));
        FMM_TRY(scatter_field(ws, t, P.n, nf, d_field, st));
        if (!learned || attempt == 1) break;
        // check at the sampled particles; fall back to the fixed rule if the
        // measured error is above the target
        const int nt = (int)rows.size();
        double* d_got = ws.sel_scratch.as<double>() + (size_t)nt * nf;
        const int64_t* d_rows = reinterpret_cast<const int64_t*>(ws.sel_scratch.as<double>() + (size_t)nt * nf * 2);
        count_launches(1);
        k_gather_rows<<<(nt * nf + 127) / 128, 128, 0, st>>>(P.n, nf, d_field, d_rows, nt, d_got);
        std::vector<double> got((size_t)nt * nf);
        FMM_CUDA_TRY(cudaMemcpyAsync(got.data(), d_got, sizeof(double) * nt * nf, cudaMemcpyDeviceToHost, st));
        FMM_CUDA_TRY(cudaStreamSynchronize(st));
        if (ref_rows.empty()) {
            // the FP64 reference sums (second stream)
            FMM_CUDA_TRY(cudaEventSynchronize(ws.ev[11]));
            ref_rows.resize((size_t)nt * nf);
            FMM_CUDA_TRY(cudaMemcpy(ref_rows.data(), ws.sel_scratch.as<double>(), sizeof(double) * nt * nf,
                                    cudaMemcpyDeviceToHost));
        }
        check_rms = sampled_rms(got, ref_rows, nt, nf);
        if (check_rms <= o.target) break;
        fallback = true;
        tpl.sel_params = nullptr;  // fixed rule (theta, expansion order of the call)
    }
    cudaEventRecord(ws.ev[6], st);
    // far pairs per expansion order (outside the timed phases)
    unsigned long long hist[16] = {0};
    // (periodic boxes: summed image by image; t.nfar is then the total over
    // the images while t.far_ord holds only the last image's pairs)
    if (!box && t.nfar > 0 && t.far_ord) {
        count_launches(1);
        k_order_hist<<<(unsigned)std::min<int64_t>(1024, (t.nfar + 255) / 256), 256, 0, st>>>(t.nfar, t.far_ord,
                                                                                                    d_hist);
    }
    FMM_CUDA_TRY(cudaMemcpyAsync(hist, d_hist, sizeof(hist), cudaMemcpyDeviceToHost, st));
    // particle pairs the near field's damping correction evaluated (counter 9)
    unsigned long long corr_evals = 0;
    if (t.ncorr > 0)
        FMM_CUDA_TRY(cudaMemcpyAsync(&corr_evals, ws.counters.as<unsigned long long>() + 9, sizeof(corr_evals),
                                     cudaMemcpyDeviceToHost, st));
    int product_err = 0;
    if (ws.product_err)
        FMM_CUDA_TRY(cudaMemcpyAsync(&product_err, ws.product_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    FMM_CUDA_TRY(cudaGetLastError());
    if (product_err) return FMM_ETIMEOUT;  // a bounded wait of the M2L product gave up
    Stats s;
    s.v[0] = t.num_nodes;
    s.v[1] = t.num_leaves;
    s.v[2] = t.max_depth;
    s.v[3] = (double)t.nfar;
    s.v[4] = (double)t.nnear;
    s.v[5] = (double)t.near_particle_pairs;
    float ms = 0;
    for (int k = 0; k < 6; ++k) {
        cudaEventElapsedTime(&ms, ws.ev[k], ws.ev[k + 1]);
        s.v[6 + k] = ms;
    }
    cudaEventElapsedTime(&ms, ws.ev[0], ws.ev[6]);
    s.v[12] = ms;
    s.v[13] = fallback ? 1.0 : 0.0;
    s.v[14] = check_rms;
    double osum = 0.0;
    for (int q = 0; q <= kMaxP; ++q) {
        s.v[16 + q] = (double)hist[q];
        osum += (double)q * (double)hist[q];
    }
    s.v[15] = t.nfar > 0 ? osum / (double)t.nfar : 0.0;
    cudaEventElapsedTime(&ms, ws.ev[3], ws.ev[7]);
    s.v[16 + kMaxP + 1] = ms;
    ms = -1.0f;
    if (ws.product_timed) cudaEventElapsedTime(&ms, ws.ev[8], ws.ev[9]);
    s.v[16 + kMaxP + 2] = ms;
    s.v[16 + kMaxP + 3] = (double)ws.m2l_groups;
    s.v[16 + kMaxP + 4] = (double)ws.list_candidates;
    s.v[16 + kMaxP + 5] = (double)ws.list_evals;
    s.v[16 + kMaxP + 6] = (double)lattice_levels;
    s.v[kTuneStats + 0] = tp.ncrit;
    s.v[kTuneStats + 1] = ws.p2p_shape.threads;
    s.v[kTuneStats + 2] = ws.p2p_shape.stage;
    s.v[kTuneStats + 3] = ws.p2p_shape.queue;
    s.v[kTuneStats + 4] = 0.0;
    s.v[kTuneStats + 5] = (double)t.ncorr;
    s.v[kTuneStats + 6] = (double)corr_evals;
    g_stats = s;
    return FMM_OK;
}

// ---------------------------------------------------------------- batched packing
// Independent systems packed into one box: a G^3 grid (G a power of two) of
// cells of side S, one system centred in each, so that cell boundaries are
// octree node boundaries; exclusions become global indices.  Every system
// must hold more than ncrit particles (a tree of its own).
struct Packed {
    std::vector<double> Xp;
    std::vector<int32_t> exg, sys;
    double root_r = 0.0;
    int64_t min_size = 0;
};

int pack_systems(int nsys, const int64_t* offsets, const double* X, int exw, const int32_t* ex, int ncrit,
                 Packed* out) {
    const int64_t n = offsets[nsys];
    std::vector<double> cen(3 * (size_t)nsys);
    double hmax = 0.0;
    int64_t min_size = n;
    for (int k = 0; k < nsys; ++k) {
        const int64_t a = offsets[k], b = offsets[k + 1];
        if (b - a <= ncrit) return FMM_EINVAL;  // every system must need a tree of its own
        min_size = std::min(min_size, b - a);
        for (int64_t i = a; i < b; ++i)
            for (int w = 0; w < exw; ++w) {
                const int32_t e = ex[(size_t)w * n + i];
                if (e < 0 || e > b - a) return FMM_EINVAL;
            }
        double h = 0.0;
        for (int d = 0; d < 3; ++d) {
            double lo = X[d * n + a], hi = lo;
            for (int64_t i = a; i < b; ++i) {
                lo = std::min(lo, X[d * n + i]);
                hi = std::max(hi, X[d * n + i]);
            }
            cen[3 * (size_t)k + d] = 0.5 * (lo + hi);
            h = std::max(h, 0.5 * (hi - lo));
        }
        hmax = std::max(hmax, h);
    }
    int G = 1;
    while ((int64_t)G * G * G < nsys) G *= 2;
    const double S = 2.0 * hmax * 1.05 + 1e-6;
    out->Xp.assign((size_t)3 * n, 0.0);
    out->exg.assign((size_t)std::max(exw, 0) * n, 0);
    out->sys.assign((size_t)n, 0);
    for (int k = 0; k < nsys; ++k) {
        const int ix = k % G, iy = (k / G) % G, iz = k / (G * G);
        const double cc[3] = {(ix - 0.5 * (G - 1)) * S, (iy - 0.5 * (G - 1)) * S, (iz - 0.5 * (G - 1)) * S};
        for (int64_t i = offsets[k]; i < offsets[k + 1]; ++i) {
            for (int d = 0; d < 3; ++d) out->Xp[d * n + i] = (X[d * n + i] - cen[3 * (size_t)k + d]) + cc[d];
            out->sys[i] = k;
            for (int w = 0; w < exw; ++w) {
                const int32_t e = ex[(size_t)w * n + i];
                out->exg[(size_t)w * n + i] = e == 0 ? 0 : (int32_t)(e + offsets[k]);
            }
        }
    }
    out->root_r = 0.5 * G * S;
    out->min_size = min_size;
    return FMM_OK;
}

// ---------------------------------------------------------------- autotuner
// For a class of calls (particle count and density in half-octaves, orders,
// settings) the first call with opts->autotune times candidate values of
// ncrit with whole evaluations of its own input, then, at the best ncrit,
// launch shapes of the FP32 near field (threads per block, staging size,
// per-leaf grid or cost-ordered work queue) by that kernel's own time; the
// choice is kept for the process and, when the environment variable
// FMM_GB300_TUNE_CACHE names a file, in that file (one line per class).
struct TuneCfg {
    int ncrit = 0;
    P2pShape shape;
};

std::mutex g_tune_mu;
std::map<std::string, TuneCfg> g_tune;
bool g_tune_loaded = false;

const char* tune_cache_path() {
    const char* e = std::getenv("FMM_GB300_TUNE_CACHE");
    return (e && *e) ? e : nullptr;
}

void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = tune_cache_path();
    if (!path) return;
    FILE* fp = std::fopen(path, "r");
    if (!fp) return;
    char key[256];
    TuneCfg c;
    while (std::fscanf(fp, "%255s %d %d %d %d", key, &c.ncrit, &c.shape.threads, &c.shape.stage, &c.shape.queue) == 5)
        if (c.ncrit > 0 && c.shape.valid()) g_tune[key] = c;
    std::fclose(fp);
}

// The density is that of the bounding box of (at most 16384) evenly strided
// particles, or of the packing box of batched systems (half-width root_r).
std::string tune_key(int64_t n, const double* X, int mdim, int f, int p, const Opts& o, int dt, double theta,
                     bool batched, double root_r = 0.0) {
    double vol = 1.0;
    if (root_r > 0.0) {
        vol = 8.0 * root_r * root_r * root_r;
    } else {
        const int64_t step = std::max<int64_t>(1, n / 16384);
        double lo[3] = {X[0], X[n], X[2 * n]}, hi[3] = {X[0], X[n], X[2 * n]};
        for (int d = 0; d < 3; ++d)
            for (int64_t k = 0; k < n; k += step) {
                lo[d] = std::min(lo[d], X[d * n + k]);
                hi[d] = std::max(hi[d], X[d * n + k]);
            }
        for (int d = 0; d < 3; ++d) vol *= std::max(hi[d] - lo[d], 1e-3);
    }
    char b[256];
    std::snprintf(b, sizeof(b), "n%d:d%d:m%d:f%d:p%d:x%d:s%d:c%d:e%d:a%d:k%d:t%d:b%d",
                  (int)std::lround(2.0 * std::log2((double)n)), (int)std::lround(2.0 * std::log2((double)n / vol)),
                  mdim, f, p, o.precision, o.selector, o.coef_mode, o.excl_mode, o.mac_mode, dt,
                  (int)std::lround(theta * 1000.0), batched ? 1 : 0);
    return b;
}

// Runs the call with the tuned configuration of its class (tuning first if
// the class is new).  tp carries the call's tree parameters; ncrit is
// replaced by the chosen value, a candidate below ncrit_limit.
int run_fmm_tuned(Workspace& ws, const Particles& P, double theta, int ncrit, int p, int f, const Opts& o,
                  TreeParams tp, double* d_field, cudaStream_t st, const std::string& key, int64_t ncrit_limit) {
    TuneCfg cfg;
    bool have = false;
    const P2pShape user_shape = ws.p2p_shape;  // restored after the call
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        tune_load_locked();
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            cfg = it->second;
            have = true;
        }
    }
    bool tuned_now = false;
    if (!have) {
        double best = 1e300;
        int bestc = ncrit;
        std::vector<int> cands = {32, 48, 64, 96, 128};
        if (std::find(cands.begin(), cands.end(), ncrit) == cands.end()) cands.push_back(ncrit);
        ws.p2p_shape = P2pShape{};
        for (int c : cands) {
            if (c >= ncrit_limit) continue;  // batched: every system needs more than ncrit particles
            tp.ncrit = c;
            const int rc = run_fmm(ws, P, theta, c, p, f, o, tp, d_field, st);
            if (rc != FMM_OK) {
                ws.p2p_shape = user_shape;
                return rc;
            }
            const double t = g_stats.v[12];  // device time of the whole evaluation
            if (t < best) {
                best = t;
                bestc = c;
            }
        }
        cfg.ncrit = bestc;
        cfg.shape = P2pShape{};
        const bool f32_near = o.precision == 1 || o.precision == 2 || o.selector == 1;
        if (f32_near) {
            const P2pShape shapes[] = {{128, 320, 1}, {256, 320, 1}, {64, 320, 1}, {128, 160, 1},
                                       {256, 160, 1}, {128, 480, 1}, {128, 320, 0}, {256, 320, 0}};
            double bt = 1e300;
            tp.ncrit = bestc;
            for (const P2pShape& sh : shapes) {
                ws.p2p_shape = sh;
                const int rc = run_fmm(ws, P, theta, bestc, p, f, o, tp, d_field, st);
                if (rc != FMM_OK) {
                    ws.p2p_shape = user_shape;
                    return rc;
                }
                const double t = g_stats.v[16 + kMaxP + 1];  // near-field kernel
                if (t > 0 && t < bt) {
                    bt = t;
                    cfg.shape = sh;
                }
            }
        }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = cfg;
        if (const char* path = tune_cache_path()) {
            if (FILE* fp = std::fopen(path, "a")) {
                std::fprintf(fp, "%s %d %d %d %d\n", key.c_str(), cfg.ncrit, cfg.shape.threads, cfg.shape.stage,
                             cfg.shape.queue);
                std::fclose(fp);
            }
        }
        tuned_now = true;
    }
    ws.p2p_shape = cfg.shape;
    tp.ncrit = cfg.ncrit;
    const int rc = run_fmm(ws, P, theta, cfg.ncrit, p, f, o, tp, d_field, st);
    ws.p2p_shape = user_shape;
    FMM_TRY(rc);
    g_stats.v[kTuneStats + 0] = cfg.ncrit;
    g_stats.v[kTuneStats + 1] = cfg.shape.threads;
    g_stats.v[kTuneStats + 2] = cfg.shape.stage;
    g_stats.v[kTuneStats + 3] = cfg.shape.queue;
    g_stats.v[kTuneStats + 4] = tuned_now ? 1.0 : 0.0;
    return FMM_OK;
}

// ---------------------------------------------------------------- plans
// A plan keeps, for fixed coordinates, exclusions, damping factors and
// settings, the octree, the interaction lists and the M2L grouping in a
// workspace of its own, and evaluates multipole sets by replaying one CUDA
// graph of the kernels that read the multipoles (gather, P2M/M2M, near
// field, exclusion fix-up, M2L, L2L/L2P, scatter): no host synchronisation
// and no per-kernel launch cost per set.  Polarisation solvers evaluate the
// field of many induced-dipole sets at fixed coordinates this way.
struct PlanImpl {
    Workspace ws;
    DevBuf sys;  // packed systems: system id per particle
    TreeDev t;
    Particles P{};
    Modes md{0, 0, 0};
    int p = 0, f = 0, nf = 0;
    bool f32_near = false;
    bool direct = false;  // n <= ncrit: the direct sum, as field_fmm does
    cudaStream_t st = nullptr;
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;  // kernel nodes of the graph
    ~PlanImpl() {
        if (exec) cudaGraphExecDestroy(exec);
        if (st) cudaStreamDestroy(st);
    }
};

// The kernels of one evaluation (multipoles in ws.in_mp, field to
// ws.out_field), on the plan's structure.
int plan_numeric(PlanImpl& pl) {
    Workspace& ws = pl.ws;
    const Particles& P = pl.P;
    TreeDev& t = pl.t;
    cudaStream_t st = pl.st;
    if (pl.direct) return launch_direct_f64(ws, P, pl.f, pl.md, ws.out_field.as<double>(), st);
    ws.product_err = nullptr;
    FMM_TRY(gather_sorted(ws, P, t, st));
    if (pl.f32_near) FMM_TRY(prepare_f32_records(ws, P, t, st));
    FMM_TRY(launch_p2m_m2m(ws, P, t, pl.p, st, pl.md.precision != 0));
    if (pl.f32_near)
        FMM_TRY(launch_p2p_f32(ws, P, t, pl.f, st));
    else
        FMM_TRY(launch_p2p_f64(ws, P, t, pl.f, pl.md, st));
    FMM_TRY(launch_excl_correction(ws, P, &t, pl.f, pl.md, ws.fsorted.as<double>(), st));
    FMM_TRY(launch_m2l(ws, t, pl.p, pl.md, st));
    FMM_TRY(launch_l2l_l2p(ws, P, t, pl.p, pl.f, pl.md.precision == 1 || pl.md.precision == 3, st));
    FMM_TRY(scatter_field(ws, t, P.n, pl.nf, ws.out_field.as<double>(), st));
    return FMM_OK;
}

int count_kernel_nodes(cudaGraph_t g, int* out) {
    size_t nn = 0;
    FMM_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) FMM_CUDA_TRY(cudaGraphGetNodes(g, nodes.data(), &nn));
    int k = 0;
    for (size_t i = 0; i < nn; ++i) {
        cudaGraphNodeType ty;
        FMM_CUDA_TRY(cudaGraphNodeGetType(nodes[i], &ty));
        if (ty == cudaGraphNodeTypeKernel) ++k;
    }
    *out = k;
    return FMM_OK;
}

int plan_build(PlanImpl& pl, int64_t n, const double* X, int mdim, int exw, const int32_t* ex, double theta,
               int ncrit, int p, int f, int dt, const double* dampf, const Opts& o, const int32_t* sys = nullptr,
               double root_r = 0.0) {
    Workspace& ws = pl.ws;
    FMM_CUDA_TRY(cudaGetDevice(&ws.device));
    FMM_CUDA_TRY(cudaStreamCreateWithFlags(&pl.st, cudaStreamNonBlocking));
    cudaStream_t st = pl.st;
    pl.p = p;
    pl.f = f;
    pl.nf = nT(f);
    pl.md = Modes{o.coef_mode, o.excl_mode, o.precision};
    if (o.precision != 0) {  // as run_fmm: masked exclusions, exact tensors
        pl.md.excl_mode = 1;
        pl.md.coef_mode = 1;
    }
    pl.f32_near = o.precision == 1 || o.precision == 2;
    FMM_TRY(ws.in_coords.ensure(sizeof(double) * 3 * n));
    FMM_TRY(ws.in_mp.ensure(sizeof(double) * (size_t)mdim * n));
    FMM_TRY(ws.in_excl.ensure(sizeof(int32_t) * (size_t)std::max(exw, 1) * n));
    FMM_TRY(ws.in_damp.ensure(sizeof(double) * n));
    FMM_TRY(ws.out_field.ensure(sizeof(double) * (size_t)pl.nf * n));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_coords.p, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    FMM_CUDA_TRY(cudaMemsetAsync(ws.in_mp.p, 0, sizeof(double) * (size_t)mdim * n, st));
    if (exw > 0)
        FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_excl.p, ex, sizeof(int32_t) * (size_t)exw * n, cudaMemcpyHostToDevice, st));
    const double* damp = dt != DAMP_NONE ? dampf : nullptr;
    if (damp) FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_damp.p, damp, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    pl.P = Particles{n, ws.in_coords.as<double>(), mdim, ws.in_mp.as<double>(), exw, ws.in_excl.as<int32_t>(),
                     damp ? ws.in_damp.as<double>() : nullptr, dt};
    pl.direct = n <= ncrit;
    if (!pl.direct) {
        TreeParams tp{ncrit, theta, o.centroid_mode, 0, {0, 0, 0}, o.mac_mode, 0.0, p};
        if (sys) {  // packed systems (as fmm_field_fmm_batched): root given, system-aware lists
            FMM_TRY(pl.sys.ensure(sizeof(int32_t) * (size_t)n));
            FMM_CUDA_TRY(cudaMemcpyAsync(pl.sys.p, sys, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
            tp.centroid_mode = 1;
            tp.have_host_centroid = 1;
            tp.root_r = root_r;
            tp.d_sys = pl.sys.as<int32_t>();
        } else if (o.centroid_mode == 0) {
            host_centroid_sequential(X, n, tp.host_centroid);
            tp.have_host_centroid = 1;
        }
        if (o.mac_mode == 1 && dt != DAMP_NONE && damp) {
            const double dmin = min_damping_factor(ws, pl.P.damp, n, st);
            tp.rdamp = damping_range(dt, dmin * dmin, dim_to_order(mdim) + f, 0.1 * o.target);
        }
        FMM_TRY(build_tree(ws, pl.P.x, n, tp, pl.t, st));
        FMM_TRY(build_lists(ws, pl.t, tp, st));
    }
    // one evaluation builds the M2L structure and the cached tables ...
    FMM_TRY(plan_numeric(pl));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    // ... then the numeric kernels are captured
    ws.reuse_structure = true;
    cudaGraph_t g = nullptr;
    FMM_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    const int rc = plan_numeric(pl);
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (rc != FMM_OK || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc != FMM_OK ? rc : FMM_ECUDA;
    }
    const int kst = count_kernel_nodes(g, &pl.kernels);
    const cudaError_t ie = cudaGraphInstantiate(&pl.exec, g, 0);
    cudaGraphDestroy(g);
    FMM_TRY(kst);
    if (ie != cudaSuccess) {
        cudaGetLastError();
        pl.exec = nullptr;
        return FMM_ECUDA;
    }
    return FMM_OK;
}

int plan_launch(PlanImpl& pl) {
    Workspace& ws = pl.ws;
    FMM_CUDA_TRY(cudaGraphLaunch(pl.exec, pl.st));
    int err = 0;
    if (ws.product_err)
        FMM_CUDA_TRY(cudaMemcpyAsync(&err, ws.product_err, sizeof(int), cudaMemcpyDeviceToHost, pl.st));
    FMM_CUDA_TRY(cudaStreamSynchronize(pl.st));
    FMM_CUDA_TRY(cudaGetLastError());
    return err ? FMM_ETIMEOUT : FMM_OK;
}

}  // namespace
}  // namespace fmm

using namespace fmm;

extern "C" {

const char* fmm_version(void) { return "fmm_gb300 0.1 (sm_103a)"; }

const char* fmm_strerror(int s) {
    switch (s) {
        case FMM_OK: return "ok";
        case FMM_EINVAL: return "invalid argument";
        case FMM_ENOTSUP: return "unsupported mode or order";
        case FMM_ENOMEM: return "out of memory";
        case FMM_ECUDA: return "CUDA runtime error";
        case FMM_EDEPTH: return "octree deeper than 21 levels (near-coincident particles)";
        case FMM_EORDER: return "damped interaction order not supported";
        case FMM_ETIMEOUT: return "bounded device wait timed out";
        default: return "unknown status";
    }
}

int fmm_selector_load(const float* params, int64_t count) {
    if (!params || count != fmm_selector_param_count()) return FMM_EINVAL;
    Workspace& ws = thread_workspace();
    FMM_TRY(ws.sel_params.ensure(sizeof(float) * (size_t)kMlpBufFloats));
    FMM_CUDA_TRY(cudaMemcpy(ws.sel_params.p, params, sizeof(float) * (size_t)count, cudaMemcpyHostToDevice));
    count_launches(1);
    k_mlp_stage_global<<<1, 256>>>(ws.sel_params.as<float>());  // inference layout after the blob
    FMM_CUDA_TRY(cudaDeviceSynchronize());
    ws.sel_ready = true;
    return FMM_OK;
}

int fmm_release_workspace(void) {
    Workspace& ws = thread_workspace();
    // cudaFree waits for the device, so no enqueued work still uses the buffers
    ws.release_buffers(true);
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ECUDA;
}

int fmm_last_stats(double* out, int len) {
    int k = 0;
    for (; k < len && k < kNumStats; ++k) out[k] = g_stats.v[k];
    return k;
}

int fmm_field_direct_device(int64_t n, const double* d_X, int mdim, const double* d_mp, int exw,
                            const int32_t* d_ex, int field_order, double* d_field, const char* damp, int damp_len,
                            const double* d_damp, const fmm_opts* opts) {
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, d_damp));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    Workspace& ws = thread_workspace();
    FMM_TRY(check_exclusions_device(ws, n, exw, d_ex, o.stream));
    Particles P{n, d_X, mdim, d_mp, exw, d_ex, dt != DAMP_NONE ? d_damp : nullptr, dt};
    Modes md{o.coef_mode, o.excl_mode, o.precision};
    return launch_direct_f64(ws, P, field_order, md, d_field, o.stream);
}

int fmm_field_direct(int comm, int64_t n, const double* X, int mdim, const double* mp, int exw, const int32_t* ex,
                     int field_order, double* field, const char* damp, int damp_len, const double* dampf,
                     const fmm_opts* opts) {
    (void)comm;
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, dampf));
    FMM_TRY(check_exclusions_host(n, exw, ex));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    Workspace& ws = thread_workspace();
    cudaStream_t st = o.stream;
    const int nf = nT(field_order);
    Particles P;
    FMM_TRY(upload(ws, n, X, mdim, mp, exw, ex, dt != DAMP_NONE ? dampf : nullptr, nf, &P, st));
    OutputPrefault pf(field, sizeof(double) * (size_t)nf * n);
    P.damp_type = dt;
    Modes md{o.coef_mode, o.excl_mode, o.precision};
    FMM_TRY(launch_direct_f64(ws, P, field_order, md, ws.out_field.as<double>(), st));
    pf.join();
    FMM_CUDA_TRY(cudaMemcpyAsync(field, ws.out_field.p, sizeof(double) * (size_t)nf * n, cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    return FMM_OK;
}

int fmm_field_direct_targets_device(int64_t n, const double* d_X, int mdim, const double* d_mp, int exw,
                                    const int32_t* d_ex, int64_t ntgt, const int64_t* d_targets, int field_order,
                                    double* d_field, const char* damp, int damp_len, const double* d_damp,
                                    const fmm_opts* opts) {
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, d_damp));
    if (ntgt < 1 || !d_targets) return FMM_EINVAL;
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    Workspace& ws = thread_workspace();
    FMM_TRY(check_exclusions_device(ws, n, exw, d_ex, o.stream));
    FMM_TRY(check_targets_device(ws, n, ntgt, d_targets, o.stream));
    Particles P{n, d_X, mdim, d_mp, exw, d_ex, dt != DAMP_NONE ? d_damp : nullptr, dt};
    Modes md{o.coef_mode, o.excl_mode, o.precision};
    return launch_direct_f64(ws, P, field_order, md, d_field, o.stream, ntgt, d_targets);
}

int fmm_field_fmm_device(int64_t n, const double* d_X, int mdim, const double* d_mp, int exw, const int32_t* d_ex,
                         double theta, int ncrit, int p, int field_order, double* d_field, const char* damp,
                         int damp_len, const double* d_damp, const fmm_opts* opts) {
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, d_damp));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    if (o.autotune) return FMM_ENOTSUP;  // host entry points only
    if (ncrit < 1 || p < 0 || !(theta > 0.0)) return FMM_EINVAL;
    if (p > kMaxP) return FMM_ENOTSUP;
    Workspace& ws = thread_workspace();
    FMM_TRY(check_exclusions_device(ws, n, exw, d_ex, o.stream));
    Particles P{n, d_X, mdim, d_mp, exw, d_ex, dt != DAMP_NONE ? d_damp : nullptr, dt};
    if (n <= ncrit) {
        Modes md{o.coef_mode, o.excl_mode, o.precision};
        return launch_direct_f64(ws, P, field_order, md, d_field, o.stream);
    }
    TreeParams tp{ncrit, theta, o.centroid_mode, 0, {0, 0, 0}, o.mac_mode, 0.0, p};
    return run_fmm(ws, P, theta, ncrit, p, field_order, o, tp, d_field, o.stream);
}

int fmm_field_fmm(int comm, int64_t n, const double* X, int mdim, const double* mp, int exw, const int32_t* ex,
                  double theta, int ncrit, int p, int field_order, double* field, const char* damp, int damp_len,
                  const double* dampf, int is_periodic, const double* box, const fmm_opts* opts) {
    (void)comm;
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, dampf));
    FMM_TRY(check_exclusions_host(n, exw, ex));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    if (ncrit < 1 || p < 0 || !(theta > 0.0)) return FMM_EINVAL;
    Box9 hbox{};
    if (is_periodic) {
        // periodic boxes: FP64, fixed rule; the reference stops when N <= ncrit (fmm.F90:1382)
        if (!box || n <= ncrit) return FMM_EINVAL;
        if (o.precision != 0 || o.selector != 0 || o.autotune != 0) return FMM_ENOTSUP;
        for (int k = 0; k < 9; ++k) hbox.h[k] = box[k];
    }
    if (n <= ncrit) return fmm_field_direct(comm, n, X, mdim, mp, exw, ex, field_order, field, damp, damp_len, dampf, opts);
    if (p > kMaxP) return FMM_ENOTSUP;
    Workspace& ws = thread_workspace();
    cudaStream_t st = o.stream;
    const int nf = nT(field_order);
    Particles P;
    FMM_TRY(upload(ws, n, X, mdim, mp, exw, ex, dt != DAMP_NONE ? dampf : nullptr, nf, &P, st, true));
    DeferredInputCopy dc(ws, ws.in_mp.p, mp, sizeof(double) * (size_t)mdim * n, ws.in_excl.p, ex,
                         exw > 0 ? sizeof(int32_t) * (size_t)exw * n : 0);
    if (!dc.started()) return FMM_ECUDA;
    OutputPrefault pf(field, sizeof(double) * (size_t)nf * n);
    P.damp_type = dt;
    TreeParams tp{ncrit, theta, o.centroid_mode, 0, {0, 0, 0}, o.mac_mode, 0.0, p};
    if (o.centroid_mode == 0) {
        host_centroid_sequential(X, n, tp.host_centroid);
        tp.have_host_centroid = 1;
    }
    if (o.autotune)
        FMM_TRY(run_fmm_tuned(ws, P, theta, ncrit, p, field_order, o, tp, ws.out_field.as<double>(), st,
                              tune_key(n, X, mdim, field_order, p, o, dt, theta, false), n));
    else
        FMM_TRY(run_fmm(ws, P, theta, ncrit, p, field_order, o, tp, ws.out_field.as<double>(), st,
                        is_periodic ? &hbox : nullptr));
    pf.join();
    FMM_CUDA_TRY(cudaMemcpyAsync(field, ws.out_field.p, sizeof(double) * (size_t)nf * n, cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    return FMM_OK;
}

// Many independent systems in one call (see include/fmm_gpu.h).
int fmm_field_fmm_batched(int nsys, const int64_t* offsets, const double* X, int mdim, const double* mp, int exw,
                          const int32_t* ex, double theta, int ncrit, int p, int field_order, double* field,
                          const char* damp, int damp_len, const double* dampf, const fmm_opts* opts) {
    if (nsys < 1 || !offsets || offsets[0] != 0) return FMM_EINVAL;
    const int64_t n = offsets[nsys];
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, dampf));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    if (ncrit < 1 || p < 0 || !(theta > 0.0)) return FMM_EINVAL;
    if (p > kMaxP) return FMM_ENOTSUP;
    if (exw > 0 && !ex) return FMM_EINVAL;
    Packed pk;
    FMM_TRY(pack_systems(nsys, offsets, X, exw, ex, ncrit, &pk));
    const std::vector<double>& Xp = pk.Xp;
    const std::vector<int32_t>& exg = pk.exg;
    const std::vector<int32_t>& sys = pk.sys;
    const int64_t min_size = pk.min_size;
    Workspace& ws = thread_workspace();
    cudaStream_t st = o.stream;
    const int nf = nT(field_order);
    Particles P;
    FMM_TRY(upload(ws, n, Xp.data(), mdim, mp, exw, exg.data(), dt != DAMP_NONE ? dampf : nullptr, nf, &P, st));
    P.damp_type = dt;
    FMM_TRY(ws.sysbuf.ensure(sizeof(int32_t) * (size_t)n));
    // the node system ids reuse sysbuf after the tree is built, so keep the
    // per-particle ids in the scalars-independent buffer below
    DevBuf dsys;
    FMM_TRY(dsys.ensure(sizeof(int32_t) * (size_t)n));
    FMM_CUDA_TRY(cudaMemcpyAsync(dsys.p, sys.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    TreeParams tp{ncrit, theta, 1, 1, {0, 0, 0}, o.mac_mode, 0.0, p};
    tp.root_r = pk.root_r;
    tp.d_sys = dsys.as<int32_t>();
    int rc = o.autotune ? run_fmm_tuned(ws, P, theta, ncrit, p, field_order, o, tp, ws.out_field.as<double>(), st,
                                        tune_key(n, Xp.data(), mdim, field_order, p, o, dt, theta, true, pk.root_r),
                                        min_size)
                        : run_fmm(ws, P, theta, ncrit, p, field_order, o, tp, ws.out_field.as<double>(), st);
    if (rc == FMM_OK) {
        if (cudaMemcpyAsync(field, ws.out_field.p, sizeof(double) * (size_t)nf * n, cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = FMM_ECUDA;
    }
    cudaStreamSynchronize(st);
    dsys.release();
    return rc;
}

// FP32 near-field launch shape of the calling thread (see include/fmm_gpu.h).
int fmm_set_p2p_shape(int threads, int stage, int queue) {
    P2pShape sh{threads, stage, queue};
    if (threads == 0 && stage == 0 && queue == 0) sh = P2pShape{};
    if (!sh.valid()) return FMM_EINVAL;
    thread_workspace().p2p_shape = sh;
    return FMM_OK;
}

// Plans (see include/fmm_gpu.h).
struct fmm_plan {
    fmm::PlanImpl impl;
};

int fmm_plan_create(int64_t n, const double* X, int mdim, int exw, const int32_t* ex, double theta, int ncrit, int p,
                    int field_order, const char* damp, int damp_len, const double* dampf, const fmm_opts* opts,
                    fmm_plan** plan) {
    if (!plan) return FMM_EINVAL;
    *plan = nullptr;
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, dampf));
    FMM_TRY(check_exclusions_host(n, exw, ex));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    if (!X || ncrit < 1 || p < 0 || !(theta > 0.0)) return FMM_EINVAL;
    if (p > kMaxP || o.selector != 0 || o.autotune != 0) return FMM_ENOTSUP;  // fixed acceptance rule only
    if (o.precision != 0 && (dim_to_order(mdim) > 2 || field_order > 2)) return FMM_ENOTSUP;
    fmm_plan* h = new (std::nothrow) fmm_plan;
    if (!h) return FMM_ENOMEM;
    const int st = plan_build(h->impl, n, X, mdim, exw, ex, theta, ncrit, p, field_order, dt, dampf, o);
    if (st != FMM_OK) {
        delete h;
        return st;
    }
    *plan = h;
    return FMM_OK;
}

int fmm_plan_create_batched(int nsys, const int64_t* offsets, const double* X, int mdim, int exw, const int32_t* ex,
                            double theta, int ncrit, int p, int field_order, const char* damp, int damp_len,
                            const double* dampf, const fmm_opts* opts, fmm_plan** plan) {
    if (!plan) return FMM_EINVAL;
    *plan = nullptr;
    if (nsys < 1 || !offsets || offsets[0] != 0 || !X) return FMM_EINVAL;
    const int64_t n = offsets[nsys];
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, dampf));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    if (ncrit < 1 || p < 0 || !(theta > 0.0)) return FMM_EINVAL;
    if (exw > 0 && !ex) return FMM_EINVAL;
    if (p > kMaxP || o.selector != 0 || o.autotune != 0) return FMM_ENOTSUP;
    if (o.precision != 0 && (dim_to_order(mdim) > 2 || field_order > 2)) return FMM_ENOTSUP;
    Packed pk;
    FMM_TRY(pack_systems(nsys, offsets, X, exw, ex, ncrit, &pk));
    fmm_plan* h = new (std::nothrow) fmm_plan;
    if (!h) return FMM_ENOMEM;
    const int st = plan_build(h->impl, n, pk.Xp.data(), mdim, exw, pk.exg.data(), theta, ncrit, p, field_order, dt,
                              dampf, o, pk.sys.data(), pk.root_r);
    if (st != FMM_OK) {
        delete h;
        return st;
    }
    *plan = h;
    return FMM_OK;
}

int fmm_plan_execute(fmm_plan* plan, const double* mp, double* field) {
    if (!plan || !mp || !field) return FMM_EINVAL;
    PlanImpl& pl = plan->impl;
    const Particles& P = pl.P;
    FMM_CUDA_TRY(cudaMemcpyAsync(pl.ws.in_mp.p, mp, sizeof(double) * (size_t)P.dim * P.n, cudaMemcpyHostToDevice,
                                 pl.st));
    FMM_TRY(plan_launch(pl));
    FMM_CUDA_TRY(cudaMemcpyAsync(field, pl.ws.out_field.p, sizeof(double) * (size_t)pl.nf * P.n,
                                 cudaMemcpyDeviceToHost, pl.st));
    FMM_CUDA_TRY(cudaStreamSynchronize(pl.st));
    return FMM_OK;
}

int fmm_plan_execute_device(fmm_plan* plan, const double* d_mp, double* d_field) {
    if (!plan || !d_mp || !d_field) return FMM_EINVAL;
    PlanImpl& pl = plan->impl;
    const Particles& P = pl.P;
    FMM_CUDA_TRY(cudaMemcpyAsync(pl.ws.in_mp.p, d_mp, sizeof(double) * (size_t)P.dim * P.n, cudaMemcpyDeviceToDevice,
                                 pl.st));
    FMM_TRY(plan_launch(pl));
    FMM_CUDA_TRY(cudaMemcpyAsync(d_field, pl.ws.out_field.p, sizeof(double) * (size_t)pl.nf * P.n,
                                 cudaMemcpyDeviceToDevice, pl.st));
    FMM_CUDA_TRY(cudaStreamSynchronize(pl.st));
    return FMM_OK;
}

int fmm_plan_kernels(const fmm_plan* plan) { return plan ? plan->impl.kernels : -1; }

void fmm_plan_destroy(fmm_plan* plan) { delete plan; }

}  // extern "C"
