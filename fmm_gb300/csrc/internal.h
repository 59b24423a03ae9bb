// Internal declarations shared by the translation units of the library.
#pragma once

#include <functional>

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace fmm {

// A growable device allocation (grows, never shrinks; freed with the context).
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// Octree in device memory.  Particles are kept in key-sorted order; nodes in
// depth-first preorder over octants 0..7 (the reference's numbering,
// src/fmm.F90:275-299), with the root at index 0.
struct TreeDev {
    int64_t n = 0;
    int ncrit = 0;
    int num_nodes = 0;
    int num_leaves = 0;
    int max_depth = 0;  // root has depth 1
    int nlevels = 0;
    int level_start[kMaxDepth + 3] = {0};  // ranges of level_nodes per depth (index = depth)
    double root_c[3] = {0, 0, 0};
    double root_r = 0;
    // per sorted particle
    uint32_t* perm = nullptr;    // sorted position -> original index
    int32_t* pos_of = nullptr;   // original index -> sorted position
    int32_t* leaf_of = nullptr;  // sorted position -> leaf node id
    // per node
    double *cx = nullptr, *cy = nullptr, *cz = nullptr, *r = nullptr, *rmax = nullptr;
    int32_t *depth = nullptr, *parent = nullptr, *start = nullptr, *count = nullptr, *is_leaf = nullptr;
    int32_t* child = nullptr;        // 8 per node, -1 where empty
    int32_t* level_nodes = nullptr;  // node ids grouped by depth
    int32_t* leaves = nullptr;       // ids of the leaves
    int32_t* sysid = nullptr;        // batched systems: system of each node (-1: spans several), or null
    // interaction lists, CSR by target node, sources ascending
    int64_t nfar = 0, nnear = 0;
    int64_t near_particle_pairs = 0;
    int32_t *far_off = nullptr, *far_src = nullptr;
    uint8_t* far_ord = nullptr;  // expansion order of each far pair
    int32_t *near_off = nullptr, *near_src = nullptr;
    // damping-correction list (corr_mode): far leaf pairs inside the damping
    // range, CSR by target leaf like the near list
    int64_t ncorr = 0;
    int32_t *corr_off = nullptr, *corr_src = nullptr;
    // periodic boxes: the lists in use are those of the image whose source
    // cells are displaced by `shift`; `central` is 0 for the 26 other images
    double shift[3] = {0.0, 0.0, 0.0};
    int central = 1;
};

// A 3x3 box matrix, column-major (the reference's box_matrix(3,3)).
struct Box9 {
    double h[9];
};

struct Workspace;

// Tree and list construction (tree.cu).
struct TreeParams {
    int ncrit;
    double theta;
    int centroid_mode;     // 0 sequential, 1 blocked
    int have_host_centroid;
    double host_centroid[3];
    int mac_mode;          // 0 reference MAC, 1 also demote pairs within the damping range
    double rdamp;          // damping range for mac_mode 1 (bohr)
    int order;             // expansion order stored with every far pair (fixed rule)
    // learned acceptance (selector); null params = fixed rule
    const float* sel_params = nullptr;  // MLP parameter blob (device)
    const float* sel_lnorm = nullptr;   // per node log10 norms of reduced weights by order
    const float* sel_dmin = nullptr;    // per node smallest damping factor
    int sel_P = 0;                      // order of the stored norms
    const float* sel_budget = nullptr;  // per target node: log10 of the per-pair error budget
    double sel_theta = 0.0;             // loose acceptance test applied before the network
    const float4* sel_chi = nullptr;    // FP32 node centres (hi, rmax in w) of the learned list build
    const float4* sel_clo = nullptr;    // and their low parts (half-width in w)
    double root_r = 0.0;                // > 0: root half-width given (batched packing box)
    int corr_mode = 0;                  // learned lists: leaf pairs inside the damping range may be far
                                        // (listed in the damping-correction list)
    const float2* corr_ext = nullptr;   // per leaf (particle extent, smallest damping factor)
    float corr_xcut2 = 0.0f;            // (a r)^2 beyond which a pair needs no damping correction
    const int32_t* d_sys = nullptr;     // batched systems: system id of each particle (input order)
};

// Distance beyond which the damped kernel's radial derivatives g_j (j <= nmax)
// differ from the undamped ones by at most eps (relative), for pair damping
// factor a (smallest a gives the longest range).
double damping_range(int damp, double a, int nmax, double eps);
int build_tree(Workspace& ws, const double* d_coords, int64_t n, const TreeParams& tp, TreeDev& t, cudaStream_t st);
int build_lists(Workspace& ws, TreeDev& t, const TreeParams& tp, cudaStream_t st);
// Smallest damping factor of n particles (device array), 0 if none is positive.
double min_damping_factor(Workspace& ws, const double* d_damp, int64_t n, cudaStream_t st);

// Host-side sequential centroid (the reference's SUM order).
void host_centroid_sequential(const double* coords, int64_t n, double c[3]);

// A batch of consecutive displacement groups of the grouped M2L whose
// operators are held at once: groups [g0, g1), their tasks [t0, t1), and the
// offset of their first operator.
struct M2lBatch {
    int g0, g1;
    int64_t gop_base;
    int t0, t1;
};

struct P2pShape {
    int threads = 128;
    int stage = 320;
    int queue = 1;
    int pack = 1;  // sources two at a time in packed FP32 (Blackwell f32x2 instructions)
    bool valid() const;
};
// Whether the FP32 near field runs the packed kernel for this shape, field
// order and damping kind.
bool p2p_packed_enabled(const P2pShape& sh, int field_order, int damp);

struct Workspace {
    // inputs on device (host entry points copy here)
    DevBuf in_coords, in_mp, in_excl, in_damp, out_field;
    // tree
    DevBuf keys_a, keys_b, vals_a, vals_b, cub_tmp;
    DevBuf perm, pos_of, leaf_of;
    DevBuf node_d, node_i, child, level_nodes, leaves, node_key, node_val, node_key2, node_val2;
    DevBuf counters, scalars;
    DevBuf front_a, front_b, far_pairs, near_pairs, far_sorted, near_sorted, corr_pairs, corr_sorted, corr_src;
    DevBuf node_dfs, far_src, near_src, far_ord, sysbuf;
    DevBuf sel_norms, sel_params, sel_scratch;
    DevBuf sel_budget;  // per node: log10 error budget of far pairs with that target, then its field scale
    // grouped M2L
    DevBuf m2l_tgt, m2l_keys, m2l_keys2, m2l_vals, m2l_vals2, m2l_ukeys, m2l_cnt, m2l_gstart, m2l_tcnt, m2l_toff,
        m2l_tasks, m2l_T, m2l_gq, m2l_gab, m2l_wsc, m2l_out, m2l_wsplit, m2l_gop, m2l_gopoff, m2l_rowbase;
    // sorted particle data
    DevBuf sx, sy, sz, smc, sd;
    DevBuf f32buf;   // FP32 particle records of the mixed-precision near field
    DevBuf f32node;  // node centres as FP32 hi/lo pairs
    DevBuf fsorted;
    // expansions
    DevBuf mom, loc, wred;
    DevBuf lattice;  // periodic boxes (level multipoles and contributions), QM/MM classification scratch
    int wred_p = -1;  // order of the reduced weights in wred computed from this call's moments (-1: none)
    // direct sum: scaled multipoles and partial sums
    DevBuf dsmc, partial;
    // second stream (the learned selector's sampled direct sum overlaps the tree phases)
    cudaStream_t aux = nullptr;
    // host entry points: the multipoles and exclusions are copied on `copy`
    // by a helper thread while the tree is built; run_fmm waits for
    // `copy_ev` (after `copy_join`) before it first reads them
    cudaStream_t copy = nullptr;
    cudaEvent_t copy_ev = nullptr;
    std::function<int()> copy_join;
    // ref-mode closed-form tensor tables
    DevBuf term_off, term_abc, term_c;
    int term_order = -1;
    // packed components of order <= xlate_p (P2M / M2M / L2L)
    DevBuf xlate;
    int xlate_p = -1;
    // L2P coefficient table at (l2pt_p, l2pt_f)
    DevBuf l2pt;
    int l2pt_p = -1, l2pt_f = -1;
    bool sel_ready = false;  // selector weights loaded
    // timing
    cudaEvent_t ev[16] = {};
    bool events_ready = false;
    bool product_timed = false;  // ev[8], ev[9] bracket the grouped M2L product kernel of the last call
    bool f32node_ok = false;     // f32node holds the FP32 node data of the current tree
    int* product_err = nullptr;  // device flag of the tensor-core M2L product, checked at the end of a call
    int64_t m2l_groups = 0;      // displacement groups of the last grouped M2L
    // replays (plans): the tree, lists and M2L structure of the previous
    // evaluation are kept and only the kernels that read multipoles run
    bool reuse_structure = false;
    P2pShape p2p_shape;  // FP32 near-field launch shape
    DevBuf p2p_order;    // target leaves by decreasing pair work (queue mode), and scratch
    float corr_xcut2 = 0.0f;  // damping correction: (a r)^2 beyond which a pair needs none
    DevBuf leaf_ext;          // damping correction: per leaf (particle extent, smallest damping factor)
    DevBuf p2p_pad;      // packed near field: padded leaf starts (node-indexed), odd-leaf flags and their scan
    DevBuf f32x2;        // packed near field: interleaved source records of padded leaves
    int m2l_ng = 0, m2l_ntasks = 0;  // grouped M2L structure of the last evaluation
    bool m2l_pairwise = false;       // the last structure chose the per-pair M2L kernel
    std::vector<M2lBatch> m2l_batches;  // operator batches of the last structure
    int64_t list_candidates = 0; // cell pairs examined by the last list build
    int64_t list_evals = 0;      // of which evaluated by the selector network
    int device = -1;
    int64_t node_cap = 0;
    ~Workspace();
    // Frees every device buffer (keep_selector: except the loaded selector
    // network) and forgets the tables cached in them.
    void release_buffers(bool keep_selector);
};

Workspace& thread_workspace();

// Adds k to the calling thread's count of this library's kernel launches.
void count_launches(int k);

// Kernels launchers (direct.cu, near.cu, expansions.cu).
struct Particles {
    int64_t n;
    const double* x;  // coordinates, column-major (n,3) in the caller's order
    int dim;
    const double* mp;  // (n, dim)
    int exw;
    const int32_t* excl;  // (n, exw)
    const double* damp;   // (n) or null
    int damp_type;
};

struct Modes {
    int coef_mode;
    int excl_mode;
    int precision;
};

// split_cap > 0 bounds the source splits per target (fewer, longer blocks:
// used when the sum runs beside other work on a second stream).
int launch_direct_f64(Workspace& ws, const Particles& P, int field_order, const Modes& md, double* d_field,
                      cudaStream_t st, int64_t ntgt = 0, const int64_t* d_targets = nullptr, int split_cap = 0);
// FP32 particle records and node centres of the mixed-precision near field
// (near_f32.cu; after gather_sorted).
int prepare_f32_records(Workspace& ws, const Particles& P, const TreeDev& t, cudaStream_t st);
// Per leaf: particle extent from the leaf centre and smallest damping factor
// (ws.leaf_ext, from the FP32 records), for the damping correction.
int launch_leaf_extent(Workspace& ws, const Particles& P, const TreeDev& t, cudaStream_t st);
// FP32 field estimate at a few targets (exclusions masked) from those
// records, into d_out (ntgt x nT(field_order), FP64, column-major).
int launch_direct_scale_f32(Workspace& ws, const Particles& P, const TreeDev& t, int field_order, double* d_out,
                            cudaStream_t st, int64_t ntgt, const int64_t* d_targets);

// FMM phases (near.cu / expansions.cu)
int gather_sorted(Workspace& ws, const Particles& P, const TreeDev& t, cudaStream_t st);
// image: the lists are a periodic image's (t.shift, t.central) and the near
// field is added to ws.fsorted instead of written.
int launch_p2p_f64(Workspace& ws, const Particles& P, const TreeDev& t, int field_order, const Modes& md,
                   cudaStream_t st, bool image = false);
// df: P2M sums in double-float (FP32 pipe) instead of FP64 (mixed path)
int launch_p2m_m2m(Workspace& ws, const Particles& P, const TreeDev& t, int p, cudaStream_t st, bool df = false);
int launch_m2l(Workspace& ws, const TreeDev& t, int p, const Modes& md, cudaStream_t st);
// M2L pair by pair on the CUDA cores (FP64), ref or exact tensors, honouring
// t.shift; accumulate adds into the local expansions instead of writing them.
int launch_m2l_pairwise(Workspace& ws, const TreeDev& t, int p, const Modes& md, bool accumulate, cudaStream_t st);
// Periodic boxes: lattice sum beyond the 27 images into the root's local
// expansion and the surface (dipole) term into the sorted field d_fs;
// *d_levels receives the number of lattice levels used.
int launch_periodic_lattice(Workspace& ws, const TreeDev& t, int p, int f, const Modes& md, const Box9& H,
                            double* d_fs, int* d_levels, cudaStream_t st);
int launch_m2l_reduced(Workspace& ws, const TreeDev& t, int p, bool fp32, cudaStream_t st);
int launch_m2l_grouped(Workspace& ws, const TreeDev& t, int p, bool fp32, cudaStream_t st);
int launch_reduce_moments(Workspace& ws, const TreeDev& t, int p, cudaStream_t st);
// selector.cu
int selector_node_norms(Workspace& ws, const TreeDev& t, int P, const double* d_sorted_damp, cudaStream_t st);
// Local field scale per leaf (near_f32.cu; after prepare_f32_records) and the
// per-node error budgets built from it (selector.cu).
int launch_leaf_field_scale(Workspace& ws, const Particles& P, const TreeDev& t, float* d_scale, cudaStream_t st);
int selector_node_budgets(Workspace& ws, const Particles& P, const TreeDev& t, float base, cudaStream_t st);
int selector_pair_data(Workspace& ws, const Particles& Pt, const TreeDev& t, int P, const int2* d_pairs, int npairs,
                       float* d_feats, float* d_labels, cudaStream_t st);
int selector_unpack_far(Workspace& ws, const TreeDev& t, int2* d_out, cudaStream_t st);
int launch_l2l_l2p(Workspace& ws, const Particles& P, const TreeDev& t, int p, int field_order, bool fp32,
                   cudaStream_t st);
// Launch shape of the FP32 near field (Workspace::p2p_shape; the autotuner
// sets it): threads per block (64, 128, 256), float4s per staging buffer
// (two per warp), and whether warps take target leaves from a queue ordered
// by decreasing pair work (persistent grid) instead of one leaf each.
int launch_p2p_f32(Workspace& ws, const Particles& P, const TreeDev& t, int field_order, cudaStream_t st);
int launch_excl_correction(Workspace& ws, const Particles& P, const TreeDev* t, int field_order, const Modes& md,
                           double* d_field_sorted_or_orig, cudaStream_t st);
int scatter_field(Workspace& ws, const TreeDev& t, int64_t n, int nf, double* d_field, cudaStream_t st);

}  // namespace fmm
