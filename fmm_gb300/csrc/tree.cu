// Octree build and interaction lists on the GPU.
//
// The reference inserts particles one at a time into a pointer octree and
// splits a leaf when it reaches ncrit (src/fmm.F90:137-273).  The resulting
// tree depends only on the point set: a node is internal exactly when its
// subtree holds >= ncrit particles, its children are its non-empty octants,
// and each child's centre is the parent centre +- half the parent's
// half-width (src/fmm.F90:221-245).  This file builds the same tree from
// sorted keys:
//   1. root centre = mean of the coordinates (sequential order like the
//      reference's SUM, or a fixed blocked order), half-width = 1.0001 x the
//      largest |x - c| (src/fmm.F90:184-189);
//   2. every particle descends 21 levels with the reference's strict
//      comparisons (x > c -> octant bit) against the same double-precision
//      centres, giving a 63-bit key of octant digits (root digit first);
//   3. a stable radix sort of the keys (ties keep the input order);
//   4. nodes level by level: a node's children are the runs of equal next
//      digit inside its key range, found by binary search; a child is a leaf
//      when it holds fewer than ncrit particles;
//   5. node ids in depth-first preorder over octants 0..7, obtained by
//      sorting the nodes by (first particle, depth) (src/fmm.F90:286-299).
// Interaction lists (src/fmm.F90:325-385) come from a level-synchronous
// expansion of (target, source) node pairs starting at (root, root), with the
// reference's acceptance test r*theta > rmax_i + rmax_j and descent rule;
// the norm is the scaled sum of squares of gfortran's NORM2, evaluated with
// round-to-nearest IEEE operations and no contraction, so that the frequent
// exact ties of the acceptance test resolve as in a CPU run.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.h"
#include "mlp.cuh"
#include "pair.cuh"

namespace fmm {

namespace {

constexpr int kLanes = 1024;


// scalars layout: [0..2] centre, [3] r, [4] rmax, [5] max |x - c| (as bits)
__global__ void k_centroid_lanes(const double* __restrict__ X, int64_t n, double* __restrict__ lanes) {
    const int d = blockIdx.x / (kLanes / 256);
    const int l = (blockIdx.x % (kLanes / 256)) * 256 + threadIdx.x;
    const double* v = X + (size_t)d * n;
    double s = 0.0;
    for (int64_t i = l; i < n; i += kLanes) s = __dadd_rn(s, v[i]);
    lanes[d * kLanes + l] = s;
}

__global__ void k_centroid_finish(const double* __restrict__ lanes, int64_t n, double* __restrict__ scalars) {
    const int d = threadIdx.x;
    if (d < 3) {
        double s = 0.0;
        for (int l = 0; l < kLanes; ++l) s = __dadd_rn(s, lanes[d * kLanes + l]);
        scalars[d] = __ddiv_rn(s, (double)n);
    }
}

// One block per coordinate; chunks staged in shared memory, summed by one
// thread in index order while the block loads the next chunk.
__global__ void k_centroid_seq(const double* __restrict__ X, int64_t n, double* __restrict__ scalars) {
    constexpr int kChunk = 2048;
    __shared__ double buf[2][kChunk];
    const double* v = X + (size_t)blockIdx.x * n;
    double s = 0.0;
    int cur = 0;
    for (int k = threadIdx.x; k < kChunk; k += blockDim.x) buf[0][k] = (k < n) ? v[k] : 0.0;
    __syncthreads();
    for (int64_t base = 0; base < n; base += kChunk) {
        const int64_t nb = base + kChunk;
        for (int k = threadIdx.x; k < kChunk; k += blockDim.x) buf[cur ^ 1][k] = (nb + k < n) ? v[nb + k] : 0.0;
        if (threadIdx.x == 0) {
            const int lim = (int)min((int64_t)kChunk, n - base);
            for (int k = 0; k < lim; ++k) s = __dadd_rn(s, buf[cur][k]);
        }
        __syncthreads();
        cur ^= 1;
    }
    if (threadIdx.x == 0) scalars[blockIdx.x] = __ddiv_rn(s, (double)n);
}

__global__ void k_min_damp(const double* __restrict__ d, int64_t n, double* out) {
    double m = 1e300;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmin(m, d[i]);
    typedef cub::BlockReduce<double, 256> BR;
    __shared__ typename BR::TempStorage tmp;
    double bm = BR(tmp).Reduce(m, [](double a, double b) { return fmin(a, b); });
    if (threadIdx.x == 0 && bm >= 0.0) atomicMin(reinterpret_cast<unsigned long long*>(out), __double_as_longlong(bm));
}

__global__ void k_set_centroid(double* scalars, double c0, double c1, double c2) {
    scalars[0] = c0;
    scalars[1] = c1;
    scalars[2] = c2;
    scalars[5] = 0.0;
}

__global__ void k_radius(const double* __restrict__ X, int64_t n, double* __restrict__ scalars) {
    const double c0 = scalars[0], c1 = scalars[1], c2 = scalars[2];
    double m = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        m = fmax(m, fabs(__dsub_rn(X[i], c0)));
        m = fmax(m, fabs(__dsub_rn(X[n + i], c1)));
        m = fmax(m, fabs(__dsub_rn(X[2 * n + i], c2)));
    }
    typedef cub::BlockReduce<double, 256> BR;
    __shared__ typename BR::TempStorage tmp;
    double bm = BR(tmp).Reduce(m, [](double a, double b) { return fmax(a, b); });
    if (threadIdx.x == 0) atomicMax(reinterpret_cast<unsigned long long*>(scalars + 5), __double_as_longlong(bm));
}

__global__ void k_root(double* scalars, int64_t n, int ncrit, double* bd, int32_t* bi, int64_t cap, double root_r) {
    const double r = root_r > 0.0 ? root_r : __dmul_rn(scalars[5], 1.0001);
    const double rmax = __dsqrt_rn(__dmul_rn(__dmul_rn(1.5, r), r));
    scalars[3] = r;
    scalars[4] = rmax;
    bd[0 * cap] = scalars[0];
    bd[1 * cap] = scalars[1];
    bd[2 * cap] = scalars[2];
    bd[3 * cap] = r;
    bd[4 * cap] = rmax;
    bi[0 * cap] = 0;               // start
    bi[1 * cap] = (int32_t)n;      // count
    bi[2 * cap] = 1;               // depth
    bi[3 * cap] = -1;              // parent
    bi[4 * cap] = 0;               // octant
    bi[5 * cap] = (n < ncrit) ? 1 : 0;  // leaf
}

__global__ void k_keys(const double* __restrict__ X, int64_t n, const double* __restrict__ scalars,
                       uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = X[i], y = X[n + i], z = X[2 * n + i];
    double cx = scalars[0], cy = scalars[1], cz = scalars[2], r = scalars[3];
    uint64_t key = 0;
#pragma unroll 1
    for (int l = 0; l < kMaxDepth; ++l) {
        const int o = (x > cx ? 1 : 0) | (y > cy ? 2 : 0) | (z > cz ? 4 : 0);
        key = (key << 3) | (uint64_t)o;
        r = __dmul_rn(r, 0.5);
        cx = __dadd_rn(cx, __dmul_rn(r, (o & 1) ? 1.0 : -1.0));
        cy = __dadd_rn(cy, __dmul_rn(r, (o & 2) ? 1.0 : -1.0));
        cz = __dadd_rn(cz, __dmul_rn(r, (o & 4) ? 1.0 : -1.0));
    }
    keys[i] = key;
    vals[i] = (uint32_t)i;
}

// counters: [0] num_nodes, [1] internal nodes created this level, [2] error flag
__global__ void k_build_level(int d, int p0, int p1, const uint64_t* __restrict__ keys, int ncrit, double* bd,
                              int32_t* bi, int64_t cap, int* counters) {
    // eight lanes per node: lane o (1..7) binary-searches the first particle
    // of octant >= o (the node's keys are sorted), lane 0 writes the children
    const int sub = threadIdx.x & 7, gbase = threadIdx.x & 24;
    const unsigned gmask = 0xffu << gbase;
    const int b = p0 + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 3);
    if (b >= p1) return;
    if (bi[5 * cap + b]) return;  // leaf (the node's eight lanes leave together)
    const int s = bi[0 * cap + b];
    const int e = s + bi[1 * cap + b];
    const int shift = 3 * (kMaxDepth - d);
    int a = s;
    if (sub > 0) {
        int h = e;
        while (a < h) {
            const int mid = (a + h) >> 1;
            if ((int)((keys[mid] >> shift) & 7ull) < sub)
                a = mid + 1;
            else
                h = mid;
        }
    }
    int lo[9];
#pragma unroll
    for (int o = 0; o < 8; ++o) lo[o] = __shfl_sync(gmask, a, gbase + o);
    lo[8] = e;
    if (sub != 0) return;
    int nc = 0, ni = 0;
    for (int o = 0; o < 8; ++o)
        if (lo[o + 1] > lo[o]) {
            ++nc;
            if (lo[o + 1] - lo[o] >= ncrit) ++ni;
        }
    const int base = atomicAdd(&counters[0], nc);
    if (ni) atomicAdd(&counters[1], ni);
    if (base + nc > cap) {
        atomicExch(&counters[2], 1);
        return;
    }
    const double pcx = bd[0 * cap + b], pcy = bd[1 * cap + b], pcz = bd[2 * cap + b];
    const double rc = __dmul_rn(bd[3 * cap + b], 0.5);
    const double rmax = __dsqrt_rn(__dmul_rn(__dmul_rn(1.5, rc), rc));
    int k = 0;
    for (int o = 0; o < 8; ++o) {
        const int cnt = lo[o + 1] - lo[o];
        if (cnt <= 0) continue;
        const int id = base + k++;
        bd[0 * cap + id] = __dadd_rn(pcx, __dmul_rn(rc, (o & 1) ? 1.0 : -1.0));
        bd[1 * cap + id] = __dadd_rn(pcy, __dmul_rn(rc, (o & 2) ? 1.0 : -1.0));
        bd[2 * cap + id] = __dadd_rn(pcz, __dmul_rn(rc, (o & 4) ? 1.0 : -1.0));
        bd[3 * cap + id] = rc;
        bd[4 * cap + id] = rmax;
        bi[0 * cap + id] = lo[o];
        bi[1 * cap + id] = cnt;
        bi[2 * cap + id] = d + 1;
        bi[3 * cap + id] = b;
        bi[4 * cap + id] = o;
        const int leaf = cnt < ncrit ? 1 : 0;
        bi[5 * cap + id] = leaf;
        if (!leaf && d + 1 > kMaxDepth) atomicExch(&counters[2], 2);
    }
}

__global__ void k_node_sort_keys(int M, const int32_t* bi, int64_t cap, uint64_t* keys, int32_t* vals) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= M) return;
    keys[b] = ((uint64_t)(uint32_t)bi[0 * cap + b] << 5) | (uint64_t)bi[2 * cap + b];
    vals[b] = b;
}

__global__ void k_inverse(int M, const int32_t* dfs2build, int32_t* build2dfs) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < M) build2dfs[dfs2build[k]] = k;
}

__global__ void k_remap(int M, const int32_t* __restrict__ dfs2build, const int32_t* __restrict__ build2dfs,
                        const double* __restrict__ bd, const int32_t* __restrict__ bi, int64_t cap, TreeDev t,
                        int32_t* __restrict__ leaf_flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    const int b = dfs2build[k];
    t.cx[k] = bd[0 * cap + b];
    t.cy[k] = bd[1 * cap + b];
    t.cz[k] = bd[2 * cap + b];
    t.r[k] = bd[3 * cap + b];
    t.rmax[k] = bd[4 * cap + b];
    t.start[k] = bi[0 * cap + b];
    t.count[k] = bi[1 * cap + b];
    t.depth[k] = bi[2 * cap + b];
    const int pb = bi[3 * cap + b];
    const int pk = pb >= 0 ? build2dfs[pb] : -1;
    t.parent[k] = pk;
    t.is_leaf[k] = bi[5 * cap + b];
    leaf_flag[k] = bi[5 * cap + b];
    if (pk >= 0) t.child[8 * pk + bi[4 * cap + b]] = k;
    t.level_nodes[b] = k;
}

__global__ void k_iota(int M, int32_t* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < M) out[k] = k;
}

__global__ void k_leaf_of(int nleaves, const int32_t* __restrict__ leaves, const int32_t* __restrict__ start,
                          const int32_t* __restrict__ count, int32_t* __restrict__ leaf_of) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (w >= nleaves) return;
    const int k = leaves[w];
    const int s = start[k], c = count[k];
    for (int q = lane; q < c; q += 32) leaf_of[s + q] = k;
}

// System of each node from its first and last particle (key-sorted order);
// -1 when they differ (the node spans several packed systems).
__global__ void k_node_sys(int M, const int32_t* __restrict__ start, const int32_t* __restrict__ count,
                           const uint32_t* __restrict__ perm, const int32_t* __restrict__ sys,
                           int32_t* __restrict__ sysid) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    const int a = sys[perm[start[k]]], b = sys[perm[start[k] + count[k] - 1]];
    sysid[k] = a == b ? a : -1;
}

__global__ void k_pos_of(int64_t n, const uint32_t* __restrict__ perm, int32_t* __restrict__ pos_of) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) pos_of[perm[k]] = (int32_t)k;
}

// counters: [0] next frontier size, [1] far count, [2] near count, [3] overflow flag
// Slots for this lane's `cnt` entries in a list shared by the whole grid: one
// atomic per warp (warp-wide inclusive scan of the counts); every lane of
// the warp must call it.  Returns the first slot of the lane's entries.
__device__ __forceinline__ unsigned long long warp_alloc(unsigned long long* ctr, unsigned cnt, int lane) {
    unsigned x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const unsigned total = __shfl_sync(0xffffffffu, x, 31);
    unsigned long long base = 0;
    if (lane == 31 && total) base = atomicAdd(ctr, (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + (x - cnt);
}

// Outcome of one candidate pair (i, j): far (at `order`), near (two leaves),
// or refined into the children of the larger node; entries are appended to
// the far list, the near list or the next frontier.  Called by every lane of
// the warp (skip: no candidate).
// With corr (two leaves inside the damping range, accepted as far), the pair
// is also appended to the damping-correction list corrp (counter 5).
template <typename RR>
__device__ __forceinline__ void emit_pair(bool skip, bool accept, int order, int i, int j, bool li, bool lj,
                                          bool mixed, RR ri, RR rj, const TreeDev& t, int2* __restrict__ out,
                                          int64_t cap_out, uint64_t* __restrict__ far, int64_t cap_far,
                                          uint64_t* __restrict__ nearp, int64_t cap_near,
                                          unsigned long long* counters, int lane, bool corr = false,
                                          uint64_t* __restrict__ corrp = nullptr, int64_t cap_corr = 0) {
    const bool isfar = !skip && accept;
    const bool isnear = !skip && !accept && li && lj && !mixed;
    const bool refine = !skip && !accept && !isnear;
    const bool iscorr = isfar && corr;
    int c[8], nc = 0;
    bool descend_i = false;
    if (refine) {
        descend_i = lj || ((ri > rj) && !li);
        const int* ch = t.child + 8 * (descend_i ? i : j);
#pragma unroll
        for (int o = 0; o < 8; ++o) {
            const int v = ch[o];
            if (v >= 0) c[nc++] = v;
        }
    }
    const unsigned long long kf = warp_alloc(&counters[1], isfar ? 1u : 0u, lane);
    const unsigned long long kn = warp_alloc(&counters[2], isnear ? 1u : 0u, lane);
    const unsigned long long kr = warp_alloc(&counters[0], (unsigned)nc, lane);
    const unsigned long long kc = warp_alloc(&counters[5], iscorr ? 1u : 0u, lane);
    if (iscorr) {
        if (kc < (unsigned long long)cap_corr)
            corrp[kc] = ((uint64_t)(uint32_t)i << 32) | (uint32_t)j;
        else
            counters[3] = 1;
    }
    if (isfar) {
        if (kf < (unsigned long long)cap_far)
            far[kf] = ((uint64_t)(uint32_t)i << 36) | ((uint64_t)(order & 15) << 32) | (uint32_t)j;
        else
            counters[3] = 1;
    }
    if (isnear) {
        if (kn < (unsigned long long)cap_near)
            nearp[kn] = ((uint64_t)(uint32_t)i << 32) | (uint32_t)j;
        else
            counters[3] = 1;
    }
    if (refine) {
        if (kr + nc > (unsigned long long)cap_out) {
            counters[3] = 1;
        } else {
            for (int o = 0; o < nc; ++o) out[kr + o] = descend_i ? make_int2(c[o], j) : make_int2(i, c[o]);
        }
    }
}

__global__ void k_list_iter(const int2* __restrict__ in, int nin, int2* __restrict__ out, int64_t cap_out,
                            uint64_t* __restrict__ far, int64_t cap_far, uint64_t* __restrict__ nearp,
                            int64_t cap_near, const TreeDev t, double theta, double rdamp, int order,
                            unsigned long long* counters) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool skip = q >= nin;
    int i = 0, j = 0;
    double ri = 0.0, rj = 0.0;
    bool li = false, lj = false, mixed = false, accept = false;
    if (!skip) {
        i = in[q].x;
        j = in[q].y;
        // delta = c_i - (c_j + displacement) (fmm.F90:357-358); the
        // displacement is that of the periodic image (0 without one)
        const double dx = __dsub_rn(t.cx[i], __dadd_rn(t.cx[j], t.shift[0]));
        const double dy = __dsub_rn(t.cy[i], __dadd_rn(t.cy[j], t.shift[1]));
        const double dz = __dsub_rn(t.cz[i], __dadd_rn(t.cz[j], t.shift[2]));
        const double r = norm2_3(dx, dy, dz);
        ri = t.rmax[i];
        rj = t.rmax[j];
        li = t.is_leaf[i] != 0;
        lj = t.is_leaf[j] != 0;
        // batched systems: no pairs across systems; nodes spanning several
        // systems are always refined
        if (t.sysid) {
            const int si = t.sysid[i], sj = t.sysid[j];
            if (si >= 0 && sj >= 0 && si != sj) skip = true;
            mixed = si < 0 || sj < 0;
        }
        accept = !mixed && __dmul_rn(r, theta) > __dadd_rn(ri, rj);
        if (accept && rdamp > 0.0) {
            // closest possible particle distance: centre distance minus the cube circumradii
            const double gap = __dsub_rn(r, __dmul_rn(1.7320508075688772, __dadd_rn(t.r[i], t.r[j])));
            accept = gap >= rdamp;
        }
    }
    emit_pair(skip, accept, order, i, j, li, lj, mixed, ri, rj, t, out, cap_out, far, cap_far, nearp, cap_near,
              counters, lane);
}

// Learned acceptance (selector): a pair that passes the loose geometric test
// (theta_loose) and the damping-range test is accepted at the lowest order q
// (2..qmax) whose predicted log10 truncation error is within the per-pair
// budget; otherwise it is refined exactly like a pair the test rejects.
// corr_mode: two leaves that pass the geometric test but lie inside the
// damping range go to the network as well, as undamped pairs (the damping
// feature at its far value: the M2L carries the undamped kernel); accepted,
// they are far pairs whose particle pairs inside the range are corrected by
// the near-field kernel (the difference of the damped and undamped
// kernels), and listed in corrp.
__global__ void __launch_bounds__(128) k_list_iter_learned(
    const int2* __restrict__ in, int nin, int2* __restrict__ out, int64_t cap_out, uint64_t* __restrict__ far,
    int64_t cap_far, uint64_t* __restrict__ nearp, int64_t cap_near, const TreeDev t, float theta_loose, float rdamp,
    int qmax, const float* __restrict__ params, const float* __restrict__ lnorm, const float* __restrict__ dmin,
    int P, const float* __restrict__ log_budget, const float4* __restrict__ chi, const float4* __restrict__ clo,
    unsigned long long* counters, int corr_mode, uint64_t* __restrict__ corrp, int64_t cap_corr,
    const float2* __restrict__ lext, float xcut2) {
    extern __shared__ __align__(16) float sm_sel[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* X = sm_sel + wib * kWarpTcFloats;  // this warp's network scratch
    float* Y = X + 32 * kMlpInP;
    const float* S = params + kMlpInfOff;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    bool skip = q >= nin;
    int i = 0, j = 0;
    float ri = 0.0f, rj = 0.0f;  // FP32 node data throughout: the FP64 pipe is the scarce one
    bool li = false, lj = false, mixed = false, accept = false, corr = false, ingap = false;
    float4 ci = make_float4(0.f, 0.f, 0.f, 0.f), cj = ci, oi = ci, oj = ci;
    if (!skip) {
        i = in[q].x;
        j = in[q].y;
        ci = chi[i];
        cj = chi[j];
        oi = clo[i];
        oj = clo[j];
        ri = ci.w;
        rj = cj.w;
        li = t.is_leaf[i] != 0;
        lj = t.is_leaf[j] != 0;
        // batched systems: no pairs across systems; nodes spanning several
        // systems are always refined
        if (t.sysid) {
            const int si = t.sysid[i], sj = t.sysid[j];
            if (si >= 0 && sj >= 0 && si != sj) skip = true;
            mixed = si < 0 || sj < 0;
        }
        // loose geometric gate in FP32 (the network decides; no parity with
        // the reference's rule is involved here)
        const float dx = (ci.x - cj.x) + (oi.x - oj.x), dy = (ci.y - cj.y) + (oi.y - oj.y),
                    dz = (ci.z - cj.z) + (oi.z - oj.z);
        const float r = sqrtf(dx * dx + dy * dy + dz * dz);
        accept = !skip && !mixed && r * theta_loose > ri + rj;
        if (accept && rdamp > 0.0f) {
            const float gap = r - 1.7320508f * (oi.w + oj.w);
            if (gap < rdamp) {
                if (corr_mode && li && lj) {
                    // listed for the correction unless no particle pair of the
                    // two leaves can have a r below the cutoff: a r >= dmin_i
                    // dmin_j (r - extent_i - extent_j)
                    ingap = true;
                    const float2 ea = lext[i], eb = lext[j];
                    const float xm = ea.y * eb.y * fmaxf(r - ea.x - eb.x - 1e-2f, 0.0f);
                    corr = xm * xm < xcut2;
                } else {
                    accept = false;
                }
            }
        }
    }
    // the network runs once per warp on the pairs that passed the loose test
    const unsigned need = __ballot_sync(0xffffffffu, accept);
    if (need && lane == 0) atomicAdd(&counters[4], (unsigned long long)__popc(need));
    int order = 0;
    if (need) {
        const int slot = __popc(need & ((1u << lane) - 1u));
        if (accept) {
            float x[kMlpIn];
            selector_features_f32(chi, clo, t.count, lnorm, dmin, P, i, j, x);
            if (ingap) x[16] = 1.0f;  // the M2L carries the undamped kernel; the damping is corrected pairwise
            mlp_input(S, x, X + slot * kMlpInP);
        }
        __syncwarp();
        warp_mlp_tc(params, X, Y, __popc(need), lane);
        if (accept) {
            const float b = log_budget[i];  // the target node's budget
            for (int o = kQmin; o <= qmax; ++o)
                if (Y[slot * kMlpOutP + (o - kQmin)] <= b) {
                    order = o;
                    break;
                }
            accept = order > 0;
        }
    }
    emit_pair(skip, accept, order, i, j, li, lj, mixed, ri, rj, t, out, cap_out, far, cap_far, nearp, cap_near,
              counters, lane, corr, corrp, cap_corr);
}

__global__ void k_split_pairs(int64_t m, const uint64_t* __restrict__ sorted, int32_t* __restrict__ src,
                              uint8_t* __restrict__ ord) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= m) return;
    src[k] = (int32_t)(sorted[k] & 0xffffffffull);
    if (ord) ord[k] = (uint8_t)((sorted[k] >> 32) & 15ull);
}

__global__ void k_csr_offsets(int M, int64_t m, const uint64_t* __restrict__ sorted, int32_t* __restrict__ off,
                              int shift) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > M) return;
    const uint64_t key = (uint64_t)(uint32_t)i << shift;
    int64_t a = 0, h = m;
    while (a < h) {
        const int64_t mid = (a + h) >> 1;
        if (sorted[mid] < key)
            a = mid + 1;
        else
            h = mid;
    }
    off[i] = (int32_t)a;
}

__global__ void k_near_pair_count(int64_t m, const uint64_t* __restrict__ sorted, const int32_t* __restrict__ count,
                                  unsigned long long* out) {
    unsigned long long s = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(sorted[k] >> 32), j = (int)(sorted[k] & 0xffffffffull);
        s += (unsigned long long)count[i] * (unsigned long long)count[j];
    }
    typedef cub::BlockReduce<unsigned long long, 256> BR;
    __shared__ typename BR::TempStorage tmp;
    unsigned long long b = BR(tmp).Sum(s);
    if (threadIdx.x == 0) atomicAdd(out, b);
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

int ensure_cub_tmp(Workspace& ws, size_t bytes) { return ws.cub_tmp.ensure(bytes); }

// (Re)allocate the build-order node arrays, preserving the first `keep` nodes.
int grow_nodes(Workspace& ws, int64_t new_cap, int keep, cudaStream_t st) {
    if (new_cap <= ws.node_cap) return FMM_OK;
    DevBuf nd, ni;
    if (nd.ensure(sizeof(double) * 5 * new_cap) || ni.ensure(sizeof(int32_t) * 6 * new_cap)) {
        nd.release();
        ni.release();
        return FMM_ENOMEM;
    }
    if (keep > 0) {
        for (int c = 0; c < 5; ++c)
            FMM_CUDA_TRY(cudaMemcpyAsync(nd.as<double>() + c * new_cap, ws.node_d.as<double>() + c * ws.node_cap,
                                         sizeof(double) * keep, cudaMemcpyDeviceToDevice, st));
        for (int c = 0; c < 6; ++c)
            FMM_CUDA_TRY(cudaMemcpyAsync(ni.as<int32_t>() + c * new_cap, ws.node_i.as<int32_t>() + c * ws.node_cap,
                                         sizeof(int32_t) * keep, cudaMemcpyDeviceToDevice, st));
        FMM_CUDA_TRY(cudaStreamSynchronize(st));
    }
    ws.node_d.release();
    ws.node_i.release();
    ws.node_d = nd;
    ws.node_i = ni;
    ws.node_cap = new_cap;
    return FMM_OK;
}

}  // namespace

double damping_range(int damp, double a, int nmax, double eps) {
    if (damp == DAMP_NONE || !(a > 0.0)) return 0.0;
    constexpr int NM = 6;
    nmax = std::min(nmax, NM);
    const int j0 = damp == DAMP_AMOEBA ? 1 : 0;
    double last_bad = 0.0;
    // log-spaced scan of r in [1e-3, 1e5]; the deviation decays monotonically at large r
    for (int k = 0; k <= 4000; ++k) {
        const double r = 1e-3 * std::pow(1e8, k / 4000.0);
        double g[NM + 1], g0[NM + 1];
        radial_g<NM, double>(damp, r * r, a, g);
        radial_g<NM, double>(DAMP_NONE, r * r, a, g0);
        double dev = 0.0;
        for (int j = j0; j <= nmax; ++j) dev = std::max(dev, std::fabs(g[j] - g0[j]) / std::fabs(g0[j]));
        if (dev > eps) last_bad = r;
    }
    return last_bad * std::pow(1e8, 1.0 / 4000.0);
}

void host_centroid_sequential(const double* X, int64_t n, double c[3]) {
    for (int d = 0; d < 3; ++d) {
        volatile double s = 0.0;  // keep the sequential order
        const double* v = X + (size_t)d * n;
        double acc = 0.0;
        for (int64_t i = 0; i < n; ++i) acc = acc + v[i];
        s = acc;
        c[d] = s / (double)n;
    }
}

int build_tree(Workspace& ws, const double* d_X, int64_t n, const TreeParams& tp, TreeDev& t, cudaStream_t st) {
    ws.f32node_ok = false;  // FP32 node data belong to the previous tree
    t.n = n;
    t.ncrit = tp.ncrit;
    FMM_TRY(ws.scalars.ensure(sizeof(double) * (8 + 3 * kLanes)));
    FMM_TRY(ws.counters.ensure(sizeof(unsigned long long) * 16));
    double* scal = ws.scalars.as<double>();
    // root centre
    if (tp.have_host_centroid) {
        count_launches(1);
        k_set_centroid<<<1, 1, 0, st>>>(scal, tp.host_centroid[0], tp.host_centroid[1], tp.host_centroid[2]);
    } else if (tp.centroid_mode == 0) {
        count_launches(1);
        k_centroid_seq<<<3, 256, 0, st>>>(d_X, n, scal);
        FMM_CUDA_TRY(cudaMemsetAsync(scal + 5, 0, sizeof(double), st));
    } else {
        count_launches(1);
        k_centroid_lanes<<<3 * (kLanes / 256), 256, 0, st>>>(d_X, n, scal + 8);
        count_launches(1);
        k_centroid_finish<<<1, 32, 0, st>>>(scal + 8, n, scal);
        FMM_CUDA_TRY(cudaMemsetAsync(scal + 5, 0, sizeof(double), st));
    }
    count_launches(1);
    k_radius<<<std::min<int64_t>(1024, grid_for(n, 256)), 256, 0, st>>>(d_X, n, scal);
    // node arrays
    int64_t want = std::max<int64_t>(1024, 4 * (n / std::max(1, tp.ncrit)) + 64);
    FMM_TRY(grow_nodes(ws, want, 0, st));
    count_launches(1);
    k_root<<<1, 1, 0, st>>>(scal, n, tp.ncrit, ws.node_d.as<double>(), ws.node_i.as<int32_t>(), ws.node_cap,
                            tp.root_r);
    // keys and sort
    FMM_TRY(ws.keys_a.ensure(sizeof(uint64_t) * n));
    FMM_TRY(ws.keys_b.ensure(sizeof(uint64_t) * n));
    FMM_TRY(ws.vals_a.ensure(sizeof(uint32_t) * n));
    FMM_TRY(ws.vals_b.ensure(sizeof(uint32_t) * n));
    count_launches(1);
    k_keys<<<grid_for(n, 256), 256, 0, st>>>(d_X, n, scal, ws.keys_a.as<uint64_t>(), ws.vals_a.as<uint32_t>());
    size_t tmp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, ws.keys_a.as<uint64_t>(), ws.keys_b.as<uint64_t>(),
                                    ws.vals_a.as<uint32_t>(), ws.vals_b.as<uint32_t>(), (int)n, 0, 3 * kMaxDepth, st);
    FMM_TRY(ensure_cub_tmp(ws, tmp_bytes));
    FMM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(ws.cub_tmp.p, tmp_bytes, ws.keys_a.as<uint64_t>(),
                                                 ws.keys_b.as<uint64_t>(), ws.vals_a.as<uint32_t>(),
                                                 ws.vals_b.as<uint32_t>(), (int)n, 0, 3 * kMaxDepth, st));
    const uint64_t* skeys = ws.keys_b.as<uint64_t>();
    // levels
    int* ctr = reinterpret_cast<int*>(ws.counters.p);
    int hc[3];
    int num = 1;
    int level_lo = 0, level_hi = 1;  // build ids of the current level
    int internal = (n >= tp.ncrit) ? 1 : 0;
    t.level_start[1] = 0;
    int d = 1;
    while (internal > 0) {
        const int64_t need = (int64_t)num + 8LL * internal;
        if (need > ws.node_cap) FMM_TRY(grow_nodes(ws, std::max<int64_t>(need, 2 * ws.node_cap), num, st));
        hc[0] = num;
        hc[1] = 0;
        hc[2] = 0;
        FMM_CUDA_TRY(cudaMemcpyAsync(ctr, hc, sizeof(hc), cudaMemcpyHostToDevice, st));
        count_launches(1);
        k_build_level<<<grid_for((int64_t)(level_hi - level_lo) * 8, 128), 128, 0, st>>>(
            d, level_lo, level_hi, skeys, tp.ncrit, ws.node_d.as<double>(), ws.node_i.as<int32_t>(), ws.node_cap, ctr);
        FMM_CUDA_TRY(cudaMemcpyAsync(hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, st));
        FMM_CUDA_TRY(cudaStreamSynchronize(st));
        if (hc[2] == 1) return FMM_ECUDA;  // capacity (cannot happen: checked above)
        if (hc[2] == 2) return FMM_EDEPTH;
        level_lo = level_hi;
        level_hi = hc[0];
        num = hc[0];
        internal = hc[1];
        ++d;
        t.level_start[d] = level_lo;
        if (d > kMaxDepth + 1) return FMM_EDEPTH;
    }
    const int M = num;
    t.num_nodes = M;
    t.max_depth = d;
    t.nlevels = d;
    t.level_start[d + 1] = M;
    // DFS order
    FMM_TRY(ws.node_key.ensure(sizeof(uint64_t) * M));
    FMM_TRY(ws.node_key2.ensure(sizeof(uint64_t) * M));
    FMM_TRY(ws.node_val.ensure(sizeof(int32_t) * M * 2));
    FMM_TRY(ws.node_val2.ensure(sizeof(int32_t) * M));
    count_launches(1);
    k_node_sort_keys<<<grid_for(M, 256), 256, 0, st>>>(M, ws.node_i.as<int32_t>(), ws.node_cap,
                                                        ws.node_key.as<uint64_t>(), ws.node_val.as<int32_t>());
    tmp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, ws.node_key.as<uint64_t>(), ws.node_key2.as<uint64_t>(),
                                    ws.node_val.as<int32_t>(), ws.node_val2.as<int32_t>(), M, 0, 64, st);
    FMM_TRY(ensure_cub_tmp(ws, tmp_bytes));
    FMM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(ws.cub_tmp.p, tmp_bytes, ws.node_key.as<uint64_t>(),
                                                 ws.node_key2.as<uint64_t>(), ws.node_val.as<int32_t>(),
                                                 ws.node_val2.as<int32_t>(), M, 0, 64, st));
    int32_t* dfs2build = ws.node_val2.as<int32_t>();
    int32_t* build2dfs = ws.node_val.as<int32_t>();
    count_launches(1);
    k_inverse<<<grid_for(M, 256), 256, 0, st>>>(M, dfs2build, build2dfs);
    // final node arrays (dfs order)
    FMM_TRY(ws.child.ensure(sizeof(int32_t) * 8 * (size_t)M));
    FMM_TRY(ws.level_nodes.ensure(sizeof(int32_t) * (size_t)M * 2));
    FMM_TRY(ws.leaves.ensure(sizeof(int32_t) * (size_t)M + 64));
    FMM_TRY(ws.node_dfs.ensure(sizeof(double) * 5 * (size_t)M + sizeof(int32_t) * 6 * (size_t)M));
    double* nd = ws.node_dfs.as<double>();
    int32_t* nint = reinterpret_cast<int32_t*>(nd + 5 * (size_t)M);
    t.cx = nd;
    t.cy = nd + M;
    t.cz = nd + 2 * (size_t)M;
    t.r = nd + 3 * (size_t)M;
    t.rmax = nd + 4 * (size_t)M;
    t.start = nint;
    t.count = nint + M;
    t.depth = nint + 2 * (size_t)M;
    t.parent = nint + 3 * (size_t)M;
    t.is_leaf = nint + 4 * (size_t)M;
    int32_t* leaf_flag = nint + 5 * (size_t)M;
    t.child = ws.child.as<int32_t>();
    t.level_nodes = ws.level_nodes.as<int32_t>();
    FMM_CUDA_TRY(cudaMemsetAsync(t.child, 0xff, sizeof(int32_t) * 8 * (size_t)M, st));
    count_launches(1);
    k_remap<<<grid_for(M, 256), 256, 0, st>>>(M, dfs2build, build2dfs, ws.node_d.as<double>(),
                                               ws.node_i.as<int32_t>(), ws.node_cap, t, leaf_flag);
    // leaves in dfs order
    int* d_nsel = reinterpret_cast<int*>(ws.counters.as<unsigned long long>() + 8);
    tmp_bytes = 0;
    int32_t* iota = ws.node_val.as<int32_t>() + M;
    count_launches(1);
    k_iota<<<grid_for(M, 256), 256, 0, st>>>(M, iota);
    cub::DeviceSelect::Flagged(nullptr, tmp_bytes, iota, leaf_flag, ws.leaves.as<int32_t>(), d_nsel, M, st);
    FMM_TRY(ensure_cub_tmp(ws, tmp_bytes));
    FMM_CUDA_TRY(cub::DeviceSelect::Flagged(ws.cub_tmp.p, tmp_bytes, iota, leaf_flag, ws.leaves.as<int32_t>(), d_nsel,
                                            M, st));
    int nl = 0;
    FMM_CUDA_TRY(cudaMemcpyAsync(&nl, d_nsel, sizeof(int), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    t.num_leaves = nl;
    t.leaves = ws.leaves.as<int32_t>();
    // particle maps
    FMM_TRY(ws.leaf_of.ensure(sizeof(int32_t) * n));
    FMM_TRY(ws.pos_of.ensure(sizeof(int32_t) * n));
    t.perm = ws.vals_b.as<uint32_t>();
    t.leaf_of = ws.leaf_of.as<int32_t>();
    t.pos_of = ws.pos_of.as<int32_t>();
    count_launches(1);
    k_leaf_of<<<grid_for((int64_t)nl * 32, 256), 256, 0, st>>>(nl, t.leaves, t.start, t.count, t.leaf_of);
    count_launches(1);
    k_pos_of<<<grid_for(n, 256), 256, 0, st>>>(n, t.perm, t.pos_of);
    t.sysid = nullptr;
    if (tp.d_sys) {
        FMM_TRY(ws.sysbuf.ensure(sizeof(int32_t) * (size_t)M));
        t.sysid = ws.sysbuf.as<int32_t>();
        count_launches(1);
        k_node_sys<<<grid_for(M, 256), 256, 0, st>>>(M, t.start, t.count, t.perm, tp.d_sys, t.sysid);
    }
    double sc[5];
    FMM_CUDA_TRY(cudaMemcpyAsync(sc, scal, sizeof(sc), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    t.root_c[0] = sc[0];
    t.root_c[1] = sc[1];
    t.root_c[2] = sc[2];
    t.root_r = sc[3];
    return FMM_OK;
}

double min_damping_factor(Workspace& ws, const double* d, int64_t n, cudaStream_t st) {
    if (ws.scalars.ensure(sizeof(double) * (8 + 3 * kLanes)) != FMM_OK) return 0.0;
    double* out = ws.scalars.as<double>() + 7;
    const double big = 1e300;
    if (cudaMemcpyAsync(out, &big, sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess) return 0.0;
    count_launches(1);
    k_min_damp<<<(unsigned)std::min<int64_t>(1024, grid_for(n, 256)), 256, 0, st>>>(d, n, out);
    double h = 0.0;
    if (cudaMemcpyAsync(&h, out, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return 0.0;
    if (cudaStreamSynchronize(st) != cudaSuccess) return 0.0;
    return h >= 1e299 ? 0.0 : h;
}

int build_lists(Workspace& ws, TreeDev& t, const TreeParams& tp, cudaStream_t st) {
    const int M = t.num_nodes;
    // capacities: pair counts grow like theta^-3; never below what the
    // workspace already holds (buffers only grow), so repeated calls on
    // similar systems do not retry
    const double th = std::max(0.05, std::min(tp.theta, tp.sel_params ? tp.sel_theta : tp.theta));
    const double per = std::min(4000.0, 25.0 / (th * th * th));
    int64_t cap_far = std::max<int64_t>({4096, (int64_t)(per * M), (int64_t)(ws.far_pairs.cap / sizeof(uint64_t))});
    int64_t cap_near = std::max<int64_t>(
        {4096, (int64_t)(0.4 * per * t.num_leaves), (int64_t)(ws.near_pairs.cap / sizeof(uint64_t))});
    int64_t cap_front = std::max<int64_t>({4096, cap_far, (int64_t)(ws.front_a.cap / sizeof(int2))});
    const bool corr = tp.sel_params && tp.corr_mode && tp.mac_mode == 1 && tp.rdamp > 0.0 && tp.corr_ext;
    int64_t cap_corr = corr ? std::max<int64_t>({4096, cap_near, (int64_t)(ws.corr_pairs.cap / sizeof(uint64_t))}) : 0;
    unsigned long long* ctr = ws.counters.as<unsigned long long>();
    for (int attempt = 0; attempt < 8; ++attempt) {
        FMM_TRY(ws.front_a.ensure(sizeof(int2) * cap_front));
        FMM_TRY(ws.front_b.ensure(sizeof(int2) * cap_front));
        FMM_TRY(ws.far_pairs.ensure(sizeof(uint64_t) * cap_far));
        FMM_TRY(ws.near_pairs.ensure(sizeof(uint64_t) * cap_near));
        if (corr) FMM_TRY(ws.corr_pairs.ensure(sizeof(uint64_t) * cap_corr));
        const int2 root = make_int2(0, 0);
        FMM_CUDA_TRY(cudaMemcpyAsync(ws.front_a.p, &root, sizeof(int2), cudaMemcpyHostToDevice, st));
        // frontier, far, near, overflow flag, network evaluations, correction pairs
        unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
        FMM_CUDA_TRY(cudaMemcpyAsync(ctr, h, sizeof(h), cudaMemcpyHostToDevice, st));
        int64_t nin = 1;
        int64_t candidates = 0;
        int2* fin = ws.front_a.as<int2>();
        int2* fout = ws.front_b.as<int2>();
        bool overflow = false;
        while (nin > 0) {
            candidates += nin;
            FMM_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st));
            count_launches(1);
            if (tp.sel_params) {
                const size_t smem = sizeof(float) * 4 * (size_t)kWarpTcFloats;
                FMM_CUDA_TRY(cudaFuncSetAttribute((const void*)k_list_iter_learned,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                k_list_iter_learned<<<grid_for(nin, 128), 128, smem, st>>>(
                    fin, (int)nin, fout, cap_front, ws.far_pairs.as<uint64_t>(), cap_far, ws.near_pairs.as<uint64_t>(),
                    cap_near, t, (float)tp.sel_theta, tp.mac_mode == 1 ? (float)tp.rdamp : 0.0f, tp.order,
                    tp.sel_params, tp.sel_lnorm, tp.sel_dmin, tp.sel_P, tp.sel_budget, tp.sel_chi, tp.sel_clo,
                    ctr, corr ? 1 : 0, corr ? ws.corr_pairs.as<uint64_t>() : nullptr, cap_corr, tp.corr_ext,
                    tp.corr_xcut2);
            } else
            k_list_iter<<<grid_for(nin, 256), 256, 0, st>>>(fin, (int)nin, fout, cap_front,
                                                             ws.far_pairs.as<uint64_t>(), cap_far,
                                                             ws.near_pairs.as<uint64_t>(), cap_near, t, tp.theta,
                                                             tp.mac_mode == 1 ? tp.rdamp : 0.0, tp.order, ctr);
            FMM_CUDA_TRY(cudaMemcpyAsync(h, ctr, sizeof(h), cudaMemcpyDeviceToHost, st));
            FMM_CUDA_TRY(cudaStreamSynchronize(st));
            if (h[3]) {
                overflow = true;
                break;
            }
            nin = (int64_t)h[0];
            std::swap(fin, fout);
        }
        if (overflow) {
            if ((int64_t)h[0] > cap_front) cap_front = 2 * (int64_t)h[0];
            if ((int64_t)h[1] > cap_far) cap_far = 2 * (int64_t)h[1];
            if ((int64_t)h[2] > cap_near) cap_near = 2 * (int64_t)h[2];
            if ((int64_t)h[5] > cap_corr) cap_corr = 2 * (int64_t)h[5];
            cap_front *= 2;
            continue;
        }
        t.nfar = (int64_t)h[1];
        t.nnear = (int64_t)h[2];
        t.ncorr = corr ? (int64_t)h[5] : 0;
        ws.list_candidates = candidates;
        ws.list_evals = (int64_t)h[4];
        // sort both lists by (target, source) and build CSR offsets; the keys
        // are target << 36 (far, with the order in bits 32-35) or << 32
        // (near), so only the bits up to the largest node index are sorted
        FMM_TRY(ws.far_sorted.ensure(sizeof(uint64_t) * std::max<int64_t>(1, t.nfar)));
        FMM_TRY(ws.near_sorted.ensure(sizeof(uint64_t) * std::max<int64_t>(1, t.nnear)));
        int nbits = 1;
        while (nbits < 31 && (1 << nbits) < M) ++nbits;
        const int far_bits = std::min(64, 36 + nbits), near_bits = std::min(64, 32 + nbits);
        size_t tb = 0, tb2 = 0;
        cub::DeviceRadixSort::SortKeys(nullptr, tb, ws.far_pairs.as<uint64_t>(), ws.far_sorted.as<uint64_t>(),
                                       (int)t.nfar, 0, far_bits, st);
        cub::DeviceRadixSort::SortKeys(nullptr, tb2, ws.near_pairs.as<uint64_t>(), ws.near_sorted.as<uint64_t>(),
                                       (int)t.nnear, 0, near_bits, st);
        FMM_TRY(ensure_cub_tmp(ws, std::max(tb, tb2)));
        if (t.nfar > 0)
            FMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(ws.cub_tmp.p, tb, ws.far_pairs.as<uint64_t>(),
                                                        ws.far_sorted.as<uint64_t>(), (int)t.nfar, 0, far_bits, st));
        if (t.nnear > 0)
            FMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(ws.cub_tmp.p, tb2, ws.near_pairs.as<uint64_t>(),
                                                        ws.near_sorted.as<uint64_t>(), (int)t.nnear, 0, near_bits,
                                                        st));
        FMM_TRY(ws.far_src.ensure(sizeof(int32_t) * (std::max<int64_t>(1, t.nfar) + (M + 1))));
        FMM_TRY(ws.near_src.ensure(sizeof(int32_t) * (std::max<int64_t>(1, t.nnear) + (M + 1))));
        t.far_src = ws.far_src.as<int32_t>();
        t.far_off = t.far_src + std::max<int64_t>(1, t.nfar);
        FMM_TRY(ws.far_ord.ensure(std::max<int64_t>(1, t.nfar)));
        t.far_ord = ws.far_ord.as<uint8_t>();
        t.near_src = ws.near_src.as<int32_t>();
        t.near_off = t.near_src + std::max<int64_t>(1, t.nnear);
        if (t.nfar > 0) {
            count_launches(1);
            k_split_pairs<<<grid_for(t.nfar, 256), 256, 0, st>>>(t.nfar, ws.far_sorted.as<uint64_t>(), t.far_src,
                                                                  t.far_ord);
        }
        if (t.nnear > 0) {
            count_launches(1);
            k_split_pairs<<<grid_for(t.nnear, 256), 256, 0, st>>>(t.nnear, ws.near_sorted.as<uint64_t>(), t.near_src,
                                                                   nullptr);
        }
        count_launches(1);
        k_csr_offsets<<<grid_for(M + 1, 256), 256, 0, st>>>(M, t.nfar, ws.far_sorted.as<uint64_t>(), t.far_off, 36);
        count_launches(1);
        k_csr_offsets<<<grid_for(M + 1, 256), 256, 0, st>>>(M, t.nnear, ws.near_sorted.as<uint64_t>(), t.near_off, 32);
        t.corr_off = t.corr_src = nullptr;
        if (corr) {
            // damping-correction list: sorted by (target, source), CSR by target
            FMM_TRY(ws.corr_sorted.ensure(sizeof(uint64_t) * std::max<int64_t>(1, t.ncorr)));
            FMM_TRY(ws.corr_src.ensure(sizeof(int32_t) * (std::max<int64_t>(1, t.ncorr) + (M + 1))));
            t.corr_src = ws.corr_src.as<int32_t>();
            t.corr_off = t.corr_src + std::max<int64_t>(1, t.ncorr);
            if (t.ncorr > 0) {
                size_t tb3 = 0;
                cub::DeviceRadixSort::SortKeys(nullptr, tb3, ws.corr_pairs.as<uint64_t>(),
                                               ws.corr_sorted.as<uint64_t>(), (int)t.ncorr, 0, near_bits, st);
                FMM_TRY(ensure_cub_tmp(ws, tb3));
                FMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(ws.cub_tmp.p, tb3, ws.corr_pairs.as<uint64_t>(),
                                                            ws.corr_sorted.as<uint64_t>(), (int)t.ncorr, 0,
                                                            near_bits, st));
                count_launches(1);
                k_split_pairs<<<grid_for(t.ncorr, 256), 256, 0, st>>>(t.ncorr, ws.corr_sorted.as<uint64_t>(),
                                                                       t.corr_src, nullptr);
            }
            count_launches(1);
            k_csr_offsets<<<grid_for(M + 1, 256), 256, 0, st>>>(M, t.ncorr, ws.corr_sorted.as<uint64_t>(),
                                                                t.corr_off, 32);
        }
        unsigned long long* pc = ctr + 4;
        FMM_CUDA_TRY(cudaMemsetAsync(pc, 0, sizeof(unsigned long long), st));
        if (t.nnear > 0) {
            count_launches(1);
            k_near_pair_count<<<std::min<int64_t>(1024, grid_for(t.nnear, 256)), 256, 0, st>>>(
                t.nnear, ws.near_sorted.as<uint64_t>(), t.count, pc);
        }
        unsigned long long npp = 0;
        FMM_CUDA_TRY(cudaMemcpyAsync(&npp, pc, sizeof(npp), cudaMemcpyDeviceToHost, st));
        FMM_CUDA_TRY(cudaStreamSynchronize(st));
        t.near_particle_pairs = (int64_t)npp;
        return FMM_OK;
    }
    return FMM_ENOMEM;
}

}  // namespace fmm
