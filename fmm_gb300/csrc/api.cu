// C ABI (include/fmm_gpu.h): argument checking, device workspaces and the
// field_fmm / field_direct pipelines.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

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

Workspace::~Workspace() {
    DevBuf* all[] = {&in_coords, &in_mp,     &in_excl,     &in_damp,    &out_field,  &keys_a,     &keys_b,
                     &vals_a,    &vals_b,    &cub_tmp,     &perm,       &pos_of,     &leaf_of,    &node_d,
                     &node_i,    &child,     &level_nodes, &leaves,     &node_key,   &node_val,   &node_key2,
                     &node_val2, &counters,  &scalars,     &front_a,    &front_b,    &far_pairs,  &near_pairs,
                     &far_sorted, &near_sorted, &node_dfs, &far_src,    &near_src,   &sx,         &sy,
                     &sz,        &smc,       &sd,          &fsorted,    &mom,        &loc,        &partial,
                     &term_off,  &term_abc,  &term_c, &f32buf, &wred, &far_ord, &sel_norms, &sel_params, &sel_scratch};
    for (DevBuf* b : all) b->release();
    if (events_ready)
        for (auto& e : ev) cudaEventDestroy(e);
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

struct Stats {
    double v[13] = {0};
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
    int coef_mode = 0, excl_mode = 0, precision = 0, centroid_mode = 0, mac_mode = 0, selector = 0;
    double target = 1e-6;
    cudaStream_t stream = nullptr;
};

int parse_opts(const fmm_opts* o, Opts* out) {
    if (!o) return FMM_OK;
    if (o->version != 0 && o->version != 1) return FMM_EINVAL;
    if (o->coef_mode < 0 || o->coef_mode > 1 || o->excl_mode < 0 || o->excl_mode > 1 || o->precision < 0 ||
        o->precision > 3 || o->centroid_mode < 0 || o->centroid_mode > 1 || o->mac_mode < 0 || o->mac_mode > 1 ||
        o->selector < 0 || o->selector > 1)
        return FMM_EINVAL;
    out->coef_mode = o->coef_mode;
    out->excl_mode = o->excl_mode;
    out->precision = o->precision;
    out->centroid_mode = o->centroid_mode;
    out->mac_mode = o->mac_mode;
    out->selector = o->selector;
    out->target = o->target_rel_err > 0 ? o->target_rel_err : 1e-6;
    out->stream = (cudaStream_t)o->stream;
    return FMM_OK;
}

int check_common(int64_t n, int mdim, int exw, int field_order, int damp, const double* damping) {
    if (n < 1 || n > (int64_t)INT32_MAX - 1) return FMM_EINVAL;
    const int m = dim_to_order(mdim);
    if (m < 0 || exw < 0 || field_order < 0) return FMM_EINVAL;
    if (m > 2 || field_order > 2) return FMM_ENOTSUP;
    if (damp != DAMP_NONE && !damping) return FMM_EINVAL;
    return FMM_OK;
}

int check_exclusions_host(int64_t n, int exw, const int32_t* ex) {
    if (exw > 0 && !ex) return FMM_EINVAL;
    for (int64_t q = 0; q < n * (int64_t)exw; ++q)
        if (ex[q] < 0 || ex[q] > n) return FMM_EINVAL;
    return FMM_OK;
}

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

// Copies host inputs into the workspace's device buffers.
int upload(Workspace& ws, int64_t n, const double* X, int mdim, const double* mp, int exw, const int32_t* ex,
           const double* damp, int nf, Particles* P, cudaStream_t st) {
    FMM_TRY(ws.in_coords.ensure(sizeof(double) * 3 * n));
    FMM_TRY(ws.in_mp.ensure(sizeof(double) * (size_t)mdim * n));
    FMM_TRY(ws.in_excl.ensure(sizeof(int32_t) * (size_t)std::max(exw, 1) * n));
    FMM_TRY(ws.in_damp.ensure(sizeof(double) * n));
    FMM_TRY(ws.out_field.ensure(sizeof(double) * (size_t)nf * n));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_coords.p, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_mp.p, mp, sizeof(double) * (size_t)mdim * n, cudaMemcpyHostToDevice, st));
    if (exw > 0)
        FMM_CUDA_TRY(cudaMemcpyAsync(ws.in_excl.p, ex, sizeof(int32_t) * (size_t)exw * n, cudaMemcpyHostToDevice, st));
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

int run_fmm(Workspace& ws, const Particles& P, double theta, int ncrit, int p, int f, const Opts& o,
            const TreeParams& tp, double* d_field, cudaStream_t st) {
    ensure_events(ws);
    if (o.selector == 1) return FMM_ENOTSUP;  // learned selector: not built yet
    Modes md{o.coef_mode, o.excl_mode, o.precision};
    if (md.precision != 0) {
        // the mixed paths mask exclusions in the FP32 loop and use exact tensors
        md.excl_mode = 1;
        md.coef_mode = 1;
    }
    TreeParams tpl = tp;
    if (o.mac_mode == 1 && P.damp_type != DAMP_NONE && P.damp) {
        const double dmin = min_damping_factor(ws, P.damp, P.n, st);
        tpl.rdamp = damping_range(P.damp_type, dmin * dmin, dim_to_order(P.dim) + f, 0.1 * o.target);
    }
    TreeDev t;
    const int nf = nT(f);
    cudaEventRecord(ws.ev[0], st);
    FMM_TRY(build_tree(ws, P.x, P.n, tp, t, st));
    cudaEventRecord(ws.ev[1], st);
    FMM_TRY(build_lists(ws, t, tpl, st));
    cudaEventRecord(ws.ev[2], st);
    FMM_TRY(gather_sorted(ws, P, t, st));
    FMM_TRY(launch_p2m_m2m(ws, P, t, p, st));
    cudaEventRecord(ws.ev[3], st);
    if (md.precision == 1 || md.precision == 2)
        FMM_TRY(launch_p2p_f32(ws, P, t, f, st));
    else
        FMM_TRY(launch_p2p_f64(ws, P, t, f, md, st));
    FMM_TRY(launch_excl_correction(ws, P, &t, f, md, ws.fsorted.as<double>(), st));
    cudaEventRecord(ws.ev[4], st);
    FMM_TRY(launch_m2l(ws, t, p, md, st));
    cudaEventRecord(ws.ev[5], st);
    FMM_TRY(launch_l2l_l2p(ws, P, t, p, f, st));
    FMM_TRY(scatter_field(ws, t, P.n, nf, d_field, st));
    cudaEventRecord(ws.ev[6], st);
    FMM_CUDA_TRY(cudaEventSynchronize(ws.ev[6]));
    FMM_CUDA_TRY(cudaGetLastError());
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
    g_stats = s;
    return FMM_OK;
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

int fmm_last_stats(double* out, int len) {
    int k = 0;
    for (; k < len && k < 13; ++k) out[k] = g_stats.v[k];
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
    P.damp_type = dt;
    Modes md{o.coef_mode, o.excl_mode, o.precision};
    FMM_TRY(launch_direct_f64(ws, P, field_order, md, ws.out_field.as<double>(), st));
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
    (void)box;
    int dt = 0;
    FMM_TRY(parse_damp(damp, damp_len, &dt));
    FMM_TRY(check_common(n, mdim, exw, field_order, dt, dampf));
    FMM_TRY(check_exclusions_host(n, exw, ex));
    Opts o;
    FMM_TRY(parse_opts(opts, &o));
    if (is_periodic) return FMM_ENOTSUP;
    if (ncrit < 1 || p < 0 || !(theta > 0.0)) return FMM_EINVAL;
    if (n <= ncrit) return fmm_field_direct(comm, n, X, mdim, mp, exw, ex, field_order, field, damp, damp_len, dampf, opts);
    if (p > kMaxP) return FMM_ENOTSUP;
    Workspace& ws = thread_workspace();
    cudaStream_t st = o.stream;
    const int nf = nT(field_order);
    Particles P;
    FMM_TRY(upload(ws, n, X, mdim, mp, exw, ex, dt != DAMP_NONE ? dampf : nullptr, nf, &P, st));
    P.damp_type = dt;
    TreeParams tp{ncrit, theta, o.centroid_mode, 0, {0, 0, 0}, o.mac_mode, 0.0, p};
    if (o.centroid_mode == 0) {
        host_centroid_sequential(X, n, tp.host_centroid);
        tp.have_host_centroid = 1;
    }
    FMM_TRY(run_fmm(ws, P, theta, ncrit, p, field_order, o, tp, ws.out_field.as<double>(), st));
    FMM_CUDA_TRY(cudaMemcpyAsync(field, ws.out_field.p, sizeof(double) * (size_t)nf * n, cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    return FMM_OK;
}

}  // extern "C"
