/*
 * fmm_gpu.h - C ABI of the GB300 (sm_103a) implementation of the fmm
 * field-evaluation path (peter-reinholdt/fmm).
 *
 * The two entry points replace the reference's Fortran module procedures
 *   field_direct  (src/fmm.F90:1338-1352)
 *   field_fmm     (src/fmm.F90:1354-1400)
 * with the same argument meaning.  Arrays are Fortran column-major and
 * owned by the caller:
 *   coordinates  n x 3            double  (x column, y column, z column)
 *   multipoles   n x mdim         double  packed alphabetical order
 *                                         (q; x,y,z; xx,xy,xz,yy,yz,zz; ...),
 *                                         mdim = (m+1)(m+2)(m+3)/6
 *   exclusions   n x exw          int32   1-based particle indices, 0-padded
 *   field        n x nT(f)        double  written (zeroed by the callee first:
 *                                         the reference only accumulates into
 *                                         it, src/fmm.F90:731,813,1113)
 *   damping      n                double  per-particle damping factors, or
 *                                         NULL when damp_type is empty
 * field(:,1) is minus the potential, field(:,2:4) the electric field, and
 * the order-k block minus the k-th derivative of the potential.
 * Orders: multipole order m <= 3 (mdim <= 20) and field order f <= 3 in FP64;
 * the mixed-precision and learned paths take m <= 2 and f <= 2 (otherwise
 * FMM_ENOTSUP).  Damped kernels stop at tensor order 6 (m + f <= 6 always
 * holds here), as the reference's damped tensors do.
 *
 * `damp` is the reference's damp_type: "AMOEBA", "THOLE", "ERF" or "" (any
 * trailing blanks are ignored, as Fortran's trim() does), with length
 * `damp_len` (no NUL terminator needed).  `comm` is accepted and ignored:
 * this build runs on one GPU and performs no MPI or collective calls.
 *
 * Every call returns FMM_OK (0) or a negative status; nothing aborts the
 * process (the reference uses `error stop`, src/fmm.F90:594,1376,1382).
 */
#ifndef FMM_GPU_H
#define FMM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FMM_OK 0
#define FMM_EINVAL (-1)    /* bad argument (unknown damp type, bad sizes, exclusion index out of range) */
#define FMM_ENOTSUP (-2)   /* unsupported mode (periodic boxes, orders outside the built kernels)      */
#define FMM_ENOMEM (-3)    /* device or host allocation failed                                         */
#define FMM_ECUDA (-4)     /* a CUDA runtime call failed                                               */
#define FMM_EDEPTH (-5)    /* the octree would need more than 21 levels (near-coincident particles)   */
#define FMM_EORDER (-6)    /* damped interaction above the supported tensor order                     */
#define FMM_ETIMEOUT (-7)  /* a bounded device wait gave up                                           */

/* Options that do not exist in the reference API.  A NULL pointer means the
 * defaults, which reproduce the reference's behaviour (all fields 0). */
typedef struct fmm_opts {
    int version;        /* must be 1 (or 0 for "defaults")                                      */
    int coef_mode;      /* 0 ref: M2L tensors from the reference's int32 Cnij closed form
                               (src/tensors_recursive.F90; wraps at tensor order >= 11)
                           1 exact: exact Cartesian tensors (Hermite recursion)               */
    int excl_mode;      /* 0 ref: excluded sources moved to R=(1e10,1e10,1e10), self pair only
                               skipped if listed (src/fmm.F90:714-720, 802-806)
                           1 mask: excluded pairs and the self pair skipped; excluded pairs
                               that the far field counted are subtracted again           */
    int precision;      /* 0 fp64; 1 mixed: FP32 near field and M2L with blocked FP64
                           accumulation, FP64 tree, M2M/L2L and final sums;
                           2 FP32 near field only; 3 FP32 M2L only                       */
    int centroid_mode;  /* 0 sequential sum (as the reference), 1 blocked (1024 lanes)       */
    int mac_mode;       /* 0 reference MAC (r*theta > rmax_i + rmax_j)
                           1 damping-aware: additionally demote cell pairs whose closest
                               particles are within the damping range to the near field  */
    int selector;       /* 0 fixed expansion order; 1 learned per-pair order (MLP)           */
    double target_rel_err; /* error target for mac_mode 1 / selector 1 (default 1e-6)       */
    void *stream;       /* cudaStream_t for the *_device entry points (NULL = legacy stream) */
    int autotune;       /* 1: ncrit and the FP32 near field's launch shape chosen by timing
                           candidates on the first call of each class of calls (size,
                           density, orders, settings; host entry points fmm_field_fmm and
                           fmm_field_fmm_batched, not periodic); the choice is kept for
                           the process and in the file $FMM_GB300_TUNE_CACHE if set.  The
                           ncrit argument is then only a candidate.                       */
    int reserved[7];
} fmm_opts;

/* Replaces fmm::field_direct (src/fmm.F90:1338-1352); O(N^2) direct sum.
 * Host pointers; blocks until `field` holds the result. */
int fmm_field_direct(int comm, int64_t n, const double *coordinates, int mdim, const double *multipoles, int exw,
                     const int32_t *exclusions, int field_order, double *field, const char *damp, int damp_len,
                     const double *damping_factors, const fmm_opts *opts);

/* Replaces fmm::field_fmm (src/fmm.F90:1354-1400).  Falls back to the direct
 * sum when n <= ncrit, as the reference does (src/fmm.F90:1381-1383).
 * is_periodic != 0 evaluates the periodic system of box_matrix (3x3,
 * column-major, the cell vectors as columns) as the reference does: the 27
 * images of the box with their own interaction lists, near fields (exclusions
 * only in the central image) and M2L, the lattice sum beyond them (levels of
 * 3x3x3 supercells until a level's local-expansion norm drops below 1e-8, at
 * most 50) and the surface (dipole) term (src/fmm.F90:156-175, 337-343,
 * 623-747, 826-979).  Periodic calls need box_matrix and n > ncrit
 * (otherwise FMM_EINVAL; the reference stops) and run in FP64 with the fixed
 * acceptance rule (opts->precision 0, opts->selector 0, else FMM_ENOTSUP).
 * Host pointers; blocks until `field` holds the result. */
int fmm_field_fmm(int comm, int64_t n, const double *coordinates, int mdim, const double *multipoles, int exw,
                  const int32_t *exclusions, double theta, int ncrit, int expansion_order, int field_order,
                  double *field, const char *damp, int damp_len, const double *damping_factors, int is_periodic,
                  const double *box_matrix, const fmm_opts *opts);

/* QM/MM helpers.  Replace fmm::get_boxes, fmm::get_multipoles and
 * fmm::interpolate_electron_fields (src/fmm.F90:1134-1336), which split the
 * particles into a near field and far-field boxes around a set of QM target
 * points (classify_box: a node with a target within rmax / theta of its
 * centre is refined, a leaf that is still that close gives its particles,
 * any other node its box) and evaluate local expansions given at boxes at the
 * particles.  The octree is the reference's (same node numbers, 1-based).
 * Call once with all output pointers NULL to get sizes[0] (near-field
 * particles) and sizes[1] (boxes), then with outputs of those sizes:
 *   idx_near_field   sizes[0]                   1-based particle indices,
 *                                               leaf by leaf in node order,
 *                                               ascending within a leaf (the
 *                                               reference uses its insertion
 *                                               order there)
 *   box_coordinates  sizes[1] x 3               box centres
 *   box_indices      sizes[1]                   1-based node numbers
 *   box_multipoles   sizes[1] x nT(p) x ndens   raw Cartesian moments of the
 *                                               boxes, one set per density
 *                                               (multipoles: n x mdim x ndens)
 * fmm_interpolate_electron_fields takes local expansions local_expansion
 * (nbox x nT(p) x ndens, the reference's local-expansion convention) at the
 * 1-based nodes box_indices and writes field (n x nT(field_order) x ndens;
 * zeroed first, the reference adds into it).  The reference's own helpers stop
 * in their final clean-up (fmm.F90:301-326 deallocates interaction lists
 * that they never build); these return their results.  Host pointers;
 * multipoles of order <= 3. */
int fmm_get_boxes(int64_t n, const double *coordinates, int64_t ntgt, const double *target_coordinates,
                  double theta, int ncrit, int expansion_order, int64_t *sizes, int32_t *idx_near_field,
                  double *box_coordinates, int32_t *box_indices, const fmm_opts *opts);
int fmm_get_multipoles(int comm, int64_t n, const double *coordinates, int mdim, int ndens, const double *multipoles,
                       int64_t ntgt, const double *target_coordinates, double theta, int ncrit, int expansion_order,
                       int64_t *sizes, int32_t *idx_near_field, double *box_coordinates, double *box_multipoles,
                       const fmm_opts *opts);
int fmm_interpolate_electron_fields(int comm, int64_t n, const double *coordinates, int64_t nbox, int ndens,
                                    const double *local_expansion, const int32_t *box_indices, double theta,
                                    int ncrit, int expansion_order, int field_order, double *field,
                                    const fmm_opts *opts);

/* Many independent systems in one call (no counterpart in the reference,
 * which handles one system per call).  System k owns particles
 * offsets[k] .. offsets[k+1]-1 of the concatenated arrays (same layouts as
 * fmm_field_fmm, n = offsets[nsys]); its exclusion indices are 1-based within
 * the system.  Systems do not interact.  They are packed into one octree
 * whose top levels form a grid with one system per cell; list generation
 * drops cross-system pairs, so every phase runs once for all systems.  Each
 * system must have more than ncrit particles.  The per-system trees differ
 * from those of separate calls (their root box is the grid cell), so results
 * agree with separate calls to within the FMM truncation error, not bitwise.
 * Host pointers; blocks until `field` holds the result. */
int fmm_field_fmm_batched(int nsys, const int64_t *offsets, const double *coordinates, int mdim,
                          const double *multipoles, int exw, const int32_t *exclusions, double theta, int ncrit,
                          int expansion_order, int field_order, double *field, const char *damp, int damp_len,
                          const double *damping_factors, const fmm_opts *opts);

/* Same computations on arrays already resident in device memory (same
 * layouts), enqueued on opts->stream.  No host<->device copies of particle
 * data; the call returns after enqueueing all work except where it must read
 * a size back (tree build), which it does with a stream synchronisation. */
int fmm_field_direct_device(int64_t n, const double *d_coordinates, int mdim, const double *d_multipoles, int exw,
                            const int32_t *d_exclusions, int field_order, double *d_field, const char *damp,
                            int damp_len, const double *d_damping_factors, const fmm_opts *opts);

int fmm_field_fmm_device(int64_t n, const double *d_coordinates, int mdim, const double *d_multipoles, int exw,
                         const int32_t *d_exclusions, double theta, int ncrit, int expansion_order, int field_order,
                         double *d_field, const char *damp, int damp_len, const double *d_damping_factors,
                         const fmm_opts *opts);

/* Direct sum evaluated at a subset of the particles only (every particle is
 * still a source): d_targets holds ntgt 0-based particle indices, d_field is
 * (ntgt x nT(field_order)) column-major.  No counterpart in the reference;
 * this is the FP64 error oracle used to measure the accuracy of the fast
 * paths on sampled targets. */
int fmm_field_direct_targets_device(int64_t n, const double *d_coordinates, int mdim, const double *d_multipoles,
                                    int exw, const int32_t *d_exclusions, int64_t ntgt, const int64_t *d_targets,
                                    int field_order, double *d_field, const char *damp, int damp_len,
                                    const double *d_damping_factors, const fmm_opts *opts);

/* Allocation-free variant of fmm_field_direct_targets_device (no counterpart
 * in the reference).  For callers that cannot let a library allocate device
 * memory: host programs whose memory manager already owns the device (a
 * framework's caching allocator, a simulation code that reserved its pools up
 * front) and code that must avoid the implicit synchronisation cudaMalloc and
 * cudaFree can cause.  The caller passes the same device inputs and the output
 * array; the only scratch is a fixed 4 MiB static device array inside this
 * library (present on every GPU that loads it, until the process exits), so
 * ntgt * nT(field_order) may be at most FMM_NOALLOC_MAX_VALUES, otherwise the
 * call returns FMM_EINVAL without doing any work.  The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress); make that
 * first call before any stream capture.  All calls share the array, so calls
 * whose work overlaps on the GPU (different streams or threads) race and must
 * be serialised by the caller.  The call blocks until its stream has finished
 * (it reads a status word back).  Arguments are validated as by
 * fmm_field_direct_targets_device: an out-of-range target or an exclusion
 * entry outside 0..n in any row returns FMM_EINVAL.
 * Supports opts->excl_mode and opts->stream; other options are ignored. */
#define FMM_NOALLOC_MAX_VALUES 524256
int fmm_field_direct_targets_noalloc(int64_t n, const double *d_coordinates, int mdim, const double *d_multipoles,
                                     int exw, const int32_t *d_exclusions, int64_t ntgt, const int64_t *d_targets,
                                     int field_order, double *d_field, const char *damp, int damp_len,
                                     const double *d_damping_factors, const fmm_opts *opts);

/* Frees the device memory this library holds for the calling host thread
 * (no counterpart in the reference, whose module-global tree is freed at the
 * end of every call by `finalize`, src/fmm.F90:301-309).  The entry points
 * keep their device buffers between calls, per host thread, growing them to
 * the largest problem seen (about 9 GB at N = 1M with the learned selector);
 * a long-running host calls this when it is done with the FMM for a while.
 * The loaded selector network is kept.  The next call allocates again.
 * Waits for the device to finish the thread's work first. */
int fmm_release_workspace(void);

/* Statistics of the last fmm_field_fmm* call on this thread: tree and list
 * sizes and per-phase device times in milliseconds.  `out` receives up to
 * `len` doubles in this order: num_nodes, num_leaves, max_depth, m2l_pairs,
 * p2p_leaf_pairs, p2p_particle_pairs, t_tree (with the learned selector's
 * sampled direct sum), t_p2m_m2m, t_lists, t_p2p, t_m2l, t_l2l_l2p (with the
 * selector's check), t_total, selector_fallback (1 if the learned selector's
 * sampled check failed and the fixed rule was used), sampled_rms_err (learned
 * selector only, else -1), mean expansion order of the far pairs, the
 * number of far pairs at each expansion order 0..12, the device time of the
 * near-field kernel alone and of the grouped M2L product kernel alone (-1 if
 * that kernel did not run), the number of displacement groups of the grouped
 * M2L, the cell pairs examined by the list build and how many of them the
 * learned selector's network evaluated, and the number of lattice levels the
 * periodic sum used (0 without a periodic box); then the ncrit the call used,
 * the FP32 near field's launch shape (threads per block, staging float4s,
 * work queue 0/1) and 1 if this call ran the autotuner; then the number of
 * far leaf pairs inside the damping range whose particle pairs the near
 * field corrected (learned lists with the packed FP32 near field, AMOEBA;
 * else 0) and the number of particle pairs of those leaf pairs whose
 * correction it evaluated.  Returns the number written (at most 42). */
int fmm_last_stats(double *out, int len);

/* Diagnostics (no counterpart in the reference): builds the octree and
 * interaction lists of `coordinates` exactly as fmm_field_fmm does and copies
 * them out.  sizes[0..3] receive num_nodes, far pairs, near pairs, max_depth;
 * call first with all array pointers NULL to get the sizes.  Per node (DFS
 * preorder ids): centre (3 per node), half-width r, rmax, depth, parent id
 * (-1 for the root), leaf flag, particle count; per particle (input order):
 * leaf id; far/near lists as (target, source) id pairs sorted ascending. */
int fmm_debug_tree(int64_t n, const double *coordinates, int ncrit, double theta, int centroid_mode, int64_t *sizes,
                   double *center, double *r, double *rmax, int32_t *depth, int32_t *parent, int32_t *is_leaf,
                   int32_t *count, int32_t *leaf_of, int32_t *far_pairs, int32_t *near_pairs);

/* Diagnostics: sustained CUDA-core FMA rate of this GPU, measured by a short
 * register-resident FMA loop over all SMs.  precision 0 = FP64, 1 = FP32.
 * Writes TFLOP/s (2 flops per FMA) to *tflops. */
int fmm_measure_fma_peak(int precision, double *tflops);

/* Number of kernels this library launched on the calling thread so far. */
int64_t fmm_launch_count(void);

/* Learned expansion-order selector (no counterpart in the reference): loads
 * the network parameters (count = fmm_selector_param_count() floats, the
 * layout written by fmm_gb300/selector_train.py) for the calling thread.
 * opts->selector = 1 then makes fmm_field_fmm* accept far pairs by the
 * network's predicted truncation error (orders 2..expansion_order, which must
 * be >= 10), check the result at sampled particles against an FP64 direct sum
 * and fall back to the fixed rule (theta, expansion_order) if the check
 * fails.  Without loaded weights opts->selector = 1 returns FMM_ENOTSUP. */
int fmm_selector_load(const float *params, int64_t count);
int fmm_selector_param_count(void);

/* Selector network kernels (training and checks): parameter count, batched
 * forward pass, gradient of the mean squared error, Adam training; and
 * training-data collection for one system (features and log10 errors at
 * orders 2..12 of sampled far pairs; the octree uses the blocked centroid;
 * `pairs`, if not NULL, receives each sampled pair's target and source node
 * ids, depth-first preorder, 2 per pair).  Host pointers. */
int fmm_mlp_param_count(void);
int fmm_mlp_forward(const float *params, const float *x, int64_t n, float *y);
int fmm_mlp_grad(const float *params, const float *x, const float *y, int64_t n, float *grad, float *loss);
int fmm_mlp_train(float *params, const float *x, const float *y, int64_t n, int epochs, int batch, float lr,
                  uint64_t seed, float *losses);
int fmm_selector_collect(int64_t n, const double *coordinates, int mdim, const double *multipoles,
                         const double *damping_factors, int ncrit, double theta, int max_pairs, uint64_t seed,
                         float *features, float *labels, int *npairs, int32_t *pairs);

/* Launch shape of the mixed-precision near field for the calling thread's
 * later calls (no counterpart in the reference): threads per block (64, 128
 * or 256), float4s per staging buffer (64..1024, a multiple of 16; two
 * buffers per warp) and queue = 1 for resident warps that take target leaves
 * in order of decreasing pair work, 0 for one warp per leaf.  (0, 0, 0)
 * restores the default (128, 320, 1).  Results do not depend on threads or
 * queue; the staging size changes the grouping of the compensated sums.  An
 * autotuned call uses its class's shape and leaves this one in place. */
int fmm_set_p2p_shape(int threads, int stage, int queue);

/* Plans (no counterpart in the reference): for fixed coordinates,
 * exclusions, damping factors and settings, fmm_plan_create builds the octree,
 * the interaction lists and the M2L grouping once (arguments as
 * fmm_field_fmm; fixed acceptance rule, opts->selector must be 0; no periodic
 * boxes) and captures the kernels that read the multipoles into a CUDA graph.
 * fmm_plan_execute then evaluates the field of one multipole set (n x mdim,
 * host arrays) by one graph launch, with the results fmm_field_fmm gives for
 * the same inputs; fmm_plan_execute_device takes device arrays.  A plan owns
 * its device memory and stream; calls on one plan must not overlap.  Made for
 * fields of many multipole sets at fixed coordinates (induced dipoles in a
 * polarisation solver).  fmm_plan_kernels: kernel launches per evaluation. */
typedef struct fmm_plan fmm_plan;
int fmm_plan_create(int64_t n, const double *coordinates, int mdim, int exw, const int32_t *exclusions, double theta,
                    int ncrit, int expansion_order, int field_order, const char *damp, int damp_len,
                    const double *damping_factors, const fmm_opts *opts, fmm_plan **plan);
/* The same for independent systems packed as fmm_field_fmm_batched packs
 * them (arguments as that call without the multipoles); execute then takes
 * and returns the concatenated arrays of all systems. */
int fmm_plan_create_batched(int nsys, const int64_t *offsets, const double *coordinates, int mdim, int exw,
                            const int32_t *exclusions, double theta, int ncrit, int expansion_order, int field_order,
                            const char *damp, int damp_len, const double *damping_factors, const fmm_opts *opts,
                            fmm_plan **plan);
int fmm_plan_execute(fmm_plan *plan, const double *multipoles, double *field);
int fmm_plan_execute_device(fmm_plan *plan, const double *d_multipoles, double *d_field);
int fmm_plan_kernels(const fmm_plan *plan);
void fmm_plan_destroy(fmm_plan *plan);

/* Human-readable text for a status code. */
const char *fmm_strerror(int status);

/* Library version string. */
const char *fmm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FMM_GPU_H */
