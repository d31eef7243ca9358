/*
 * skf.h — C ABI of the GB300 strong-recursive-skeletonization FMM.
 *
 * Every entry point returns an int status (SKF_OK = 0).  Device pointers are
 * borrowed for the duration of the call; a plan owns the device buffers it
 * allocates.  One plan must not be used from two host threads at once;
 * different plans may run concurrently on different streams.
 *
 * Reference interfaces each call replaces (annayesy/skelFMM, Python):
 *   skf_plan_create     SkelFMMBatched.build_from_copy   skelfmm/batched_fmm.py:92-174
 *   skf_plan_apply      SkelFMMBatched.matvec            skelfmm/batched_fmm.py:539-564
 *   skf_kernel_apply    KernelOperator.torch_apply       skelfmm/operators.py:69-89
 *                       (the kernel_apply seam, skelfmm/batched_fmm.py:21-44,180-217)
 *   skf_skel_boxes      util.skel_box_helper over a level skelfmm/util.py:381-437,
 *                       driven by RecursiveSkeletonization.skel_tree
 *                       skelfmm/recursive_skel.py:412-492
 *   skf_proxy_rows      proxy surface size, skelfmm/util.py:72-78 + 87-124
 */
#ifndef SKF_H
#define SKF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SKF_OK 0
#define SKF_ERR_ARG 1         /* bad argument / shape (ValueError in the reference) */
#define SKF_ERR_OOM 2         /* device allocation failed */
#define SKF_ERR_CUDA 3        /* a CUDA runtime call failed */
#define SKF_ERR_UNSUPPORTED 4 /* operator/precision combination not built */
#define SKF_ERR_ID 5          /* interpolative decomposition failed: a proxy matrix has a
                                 non-finite entry (a non-finite point or normal) */

/* operators (skelfmm/operators.py:159-216) */
#define SKF_LAPLACE_2D 0
#define SKF_LAPLACE_3D 1
#define SKF_HELMHOLTZ_2D 2
#define SKF_HELMHOLTZ_3D 3
#define SKF_LAPLACE_DOUBLE_LAYER_3D 4
#define SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D 5
#define SKF_HELMHOLTZ_DOUBLE_LAYER_3D 6
#define SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D 7
#define SKF_NUM_OPS 8

/* apply precision */
#define SKF_PREC_FP64 0  /* everything in FP64 */
#define SKF_PREC_MIXED 1     /* FP32 kernel evaluation (compensated FP32 sums), FP64 T/T^T */
#define SKF_PREC_MIXED_T32 2 /* as SKF_PREC_MIXED with FP32 T/T^T (half the T bytes) */

/* translation kinds in a target box's interaction list */
#define SKF_KIND_COLLEAGUE 0   /* u += K q ; uskel[:r_u] -= K[:r_u,:r_s] qskel[:r_s] */
#define SKF_KIND_COARSE_UP 1   /* u += K q ; uskel[:r_u] -= K[:r_u,:] q            */
#define SKF_KIND_COARSE_DOWN 2 /* u += K q - K[:, :r_s] qskel[:r_s]                */
#define SKF_KIND_ROOT 3        /* u += K q (dense root level)                       */

typedef struct skf_plan skf_plan;
typedef struct skf_tree skf_tree;

/*
 * A built skeletonization in ragged (CSR) form.  "Entries" are the points a
 * box holds at its own level (leaf points, or the union of its children's
 * skeletons), in the box's skeleton-first order.  All pointers are HOST
 * pointers; skf_plan_create copies what it needs to the device.
 */
typedef struct {
  int32_t op;          /* SKF_* operator id */
  int32_t ndim;        /* 2 or 3 */
  double kappa;        /* wavenumber (0 for Laplace) */
  int64_t npoints;     /* N, length of the apply's input/output vectors */
  int32_t nboxes;
  int32_t nlevels;
  int32_t root_level;
  const int32_t* box_level; /* [nboxes] */
  const int64_t* box_off;   /* [nboxes+1] entry offsets */
  const int32_t* box_rank;  /* [nboxes] skeleton size (0 = not compressed) */
  const double* entry_xyz;  /* [E*ndim] coordinates of every entry */
  const double* entry_geom; /* [E*3] normals of every entry, or NULL */
  const int64_t* entry_pslot; /* [E] entry index in the parent box of each skeleton
                                 entry of a box below the root level, else -1 */
  int64_t nperm;               /* number of (entry, point) pairs = N */
  const int64_t* perm_entry;   /* [nperm] leaf entries ...            */
  const int64_t* perm_point;   /* [nperm] ... and the point each holds */
  const int64_t* t_off;        /* [nboxes] element offset of box T, or -1 */
  const double* t_data;        /* T blocks, row-major rank x (bs-rank);
                                  complex operators: interleaved (re,im) */
  int64_t t_len;               /* number of scalars in t_data (complex: pairs) */
  const int64_t* list_off;     /* [nboxes+1] per-target interaction lists */
  const int32_t* list_src;     /* [L] source box */
  const int8_t* list_kind;     /* [L] SKF_KIND_* */
  int32_t t_on_device;         /* 1: t_data is a DEVICE pointer (copied device to
                                  device), 0: host pointer like the rest */
  int32_t entries_on_device;   /* 1: entry_xyz and entry_geom are DEVICE pointers,
                                  0: host pointers like the rest */
} skf_plan_desc;

typedef struct {
  int64_t nentries;
  int64_t npairs_fused;   /* kernel evaluations per apply (translations) */
  int64_t t_scalars;      /* scalars in all T blocks */
  int64_t device_bytes;   /* bytes the plan holds on the device */
  int32_t nwork;          /* translation work items */
  int32_t is_complex;
  int64_t npairs_evaluated_mixed; /* kernel evaluations the mixed apply performs
                                     (fewer than npairs_fused on the symmetric path) */
  int32_t launches_fp64;  /* kernel launches of one FP64 apply (memsets excluded) */
  int32_t launches_mixed; /* kernel launches of one mixed apply (memsets excluded) */
  double rows_256_over_64; /* target rows a per-direction translation evaluates with
                              256-row work items over those with 64-row items
                              (rows padded per item, weighted by source entries) */
} skf_plan_info;

int skf_plan_create(const skf_plan_desc* desc, skf_plan** out);
int skf_plan_destroy(skf_plan* plan);
int skf_plan_query(const skf_plan* plan, skf_plan_info* info);

/* y = A x with the built operator.  x, y: DEVICE pointers to npoints FP64
   (complex operators: interleaved complex128).  stream: cudaStream_t or NULL. */
int skf_plan_apply(skf_plan* plan, const void* x, void* y, int32_t precision, void* stream);

/* Same product with HOST buffers: copies x in, applies, copies y out, and
   synchronises the stream before returning. */
int skf_plan_apply_host(skf_plan* plan, const void* x_host, void* y_host, int32_t precision, void* stream);

/* Plan options.  SKF_OPT_SCALAR_MIXED: 1 = run the mixed translations with the
   scalar FP32 kernel even where the packed FP32x2 kernel exists (Laplace), 0 =
   default.  Used to cross-check the two kernels. */
#define SKF_OPT_SCALAR_MIXED 1
/* SKF_OPT_PACKED_SHAPE: block shape of the packed kernel, 0 = 4 warps x 1 row
   pair per thread (default), 1 = 1 warp x 4 pairs, 2 = 2 warps x 2 pairs
   (256-row work items); 3 = 1 warp x 1 pair on 64-row work items (boxes of
   a few dozen to a few hundred entries waste fewer rows). */
#define SKF_OPT_PACKED_SHAPE 2
/* SKF_OPT_SYMMETRIC: 1 (default) = for symmetric point kernels with symmetric
   lists, evaluate each kernel block once for both directions; 0 = off. */
#define SKF_OPT_SYMMETRIC 3
/* SKF_OPT_SYM_SHAPE: tile of the symmetric kernel, 0 = 64 sources per
   shared-memory tile and 5 blocks per SM (default for Helmholtz 3D), 1 = 128
   and 3, 2 = 64 and 4, 3 = 32 and 5; 4 = warps splitting the source tiles of
   256-row items without block barriers (default for Laplace 2D/3D; Helmholtz
   3D plans treat it as 0); 5 = as 4 with persistent blocks taking the items
   from a queue. */
#define SKF_OPT_SYM_SHAPE 4
int skf_plan_set_option(skf_plan* plan, int32_t option, int64_t value);

/* Time the plan's translation kernel alone (device time in ms over `reps`
   launches, measured with events on `stream`).  For roofline reporting. */
int skf_plan_time_translations(skf_plan* plan, int32_t precision, int32_t reps, void* stream, float* ms_out);

/*
 * Batched kernel-block products (the reference's kernel_apply seam):
 * for pair p: out[p, 0:m[p]] = K(xt[p], xs[p]) @ q[p, 0:n[p]], with the
 * diagonal zeroed when self_flag[p] != 0.  Points padded to mmax / nmax per
 * pair, coordinates [npairs, mmax|nmax, ndim]; geometry [.., 3] or NULL.
 * All DEVICE pointers, FP64 (complex: interleaved).  precision as above.
 */
int skf_kernel_apply(int32_t op, double kappa, int32_t npairs, int32_t mmax, int32_t nmax,
                     const int32_t* m, const int32_t* n, const double* xt, const double* xs,
                     const double* gt, const double* gs, const void* q, const int8_t* self_flag,
                     void* out, int32_t precision, void* stream);

/*
 * Proxy-surface interpolative decompositions of a batch of boxes
 * (one level of the build).  For box b: points xb = x[off[b]:off[b+1]] (DEVICE,
 * [.., ndim] FP64), geometry likewise or NULL, box centre centers[b*ndim..],
 * side length `box_length`, `nproxy` requested proxy points, tolerance `tol`
 * (relative, < 1) or fixed rank (>= 1).
 * Outputs (DEVICE): rank[b]; perm[off[b]:off[b+1]] (skeleton first, local
 * indices); T written at t_out + t_off_out[b] as rank x (bs-rank) row-major,
 * where t_off_out[b] = sum over earlier boxes of bs*bs (capacity bound).
 */
int skf_skel_boxes(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x,
                   const double* geom, const double* centers, double box_length, int32_t nproxy,
                   double tol, int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out,
                   void* stream);

/*
 * skf_skel_boxes over the boxes of one level of several trees at once (the
 * builds of independent instances, one launch per level): box b's proxy
 * surface has side 2.95 * box_lengths[b] (DEVICE, FP64 per box) about
 * centers[b]; everything else as skf_skel_boxes (one operator, tolerance
 * and proxy count for all boxes).  Replaces, like skf_skel_boxes, the
 * reference's per-box skel_box_helper calls (skelfmm/util.py:381-437) of
 * several RecursiveSkeletonization.skel_tree level loops.
 */
int skf_skel_boxes_multi(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x,
                         const double* geom, const double* centers, const double* box_lengths, int32_t nproxy,
                         double tol, int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out,
                         void* stream);

/*
 * skf_skel_boxes without any device allocation.  No counterpart in the
 * reference: for callers that may not allocate GPU memory on this code path
 * (their own pool owns the device memory, a host framework's fixed budget, a
 * latency-bound loop).  Same arguments and outputs as skf_skel_boxes; the
 * workspace is a fixed file-scope device array of SKF_NOALLOC_SCRATCH_BYTES
 * that every GPU loading the library keeps until exit.  A box whose FP64
 * proxy matrix (rows x box size, x2 when complex) does not fit returns
 * SKF_ERR_SCRATCH before any kernel launch or scratch write (the call first
 * copies `off` to the host and synchronises `stream`, as skf_skel_boxes
 * does).  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress) and should precede any stream capture on that
 * device; the address is kept for the process, so a cudaDeviceReset of that
 * device invalidates it.  All calls share the array: calls that overlap on
 * the GPU race and must be serialised by the caller.  Every box runs on the
 * 256-thread ID kernel (skf_skel_boxes moves its costliest boxes of 192+
 * points to thread-block clusters), so for such boxes the redundant pivot
 * order, decided at rounding level, can differ from skf_skel_boxes'.
 */
#define SKF_NOALLOC_SCRATCH_BYTES (64ll << 20)
#define SKF_ERR_SCRATCH 7 /* problem exceeds the fixed no-allocation scratch */
int skf_skel_boxes_noalloc(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x,
                           const double* geom, const double* centers, double box_length, int32_t nproxy,
                           double tol, int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out,
                           void* stream);

/* Device segmented copy (build bookkeeping: compacting T blocks written at
   capacity offsets): dst[dst_off[s] + i] = src[src_off[s] + i], i < len[s],
   offsets and lengths in elements of `elem_bytes` (8 or 16).  All DEVICE. */
int skf_copy_segments(int64_t nseg, const int64_t* src_off, const int64_t* dst_off, const int64_t* len,
                      const void* src, void* dst, int32_t elem_bytes, void* stream);

/* Number of rows of the stacked proxy matrix the build uses for `nproxy`
   requested proxy points (cube/sphere surface size, doubled for the
   geometry operators). */
int skf_proxy_rows(int32_t op, int32_t nproxy, int32_t* rows_out);

/*
 * The ID calls keep their freed workspaces in the device's default memory
 * pool between calls (one call per tree level); this returns that memory
 * to the device once a build is done.
 */
int skf_trim_workspace(void);

/*
 * Randomized proxy IDs — the learned-rank build's fast path; no counterpart
 * in the reference, whose IDs are skf_skel_boxes.  Same arguments and outputs
 * as skf_skel_boxes (tol < 1), plus, all DEVICE unless noted:
 *   kpred[nbox]  predicted rank of box b (<= 0: full pivoted-QR ID).  With
 *                k = min(kpred[b], box size) and s = k + oversample <= 3/4
 *                of K's rows, the box factors the sketch Y = S K of its
 *                proxy matrix K, S a sparse sign matrix with `rho` +-1
 *                entries per row at hashed proxy rows (from `seed`): pivoted
 *                QR of Y with the rule |R_kk| <= sketch_tol |R_00|.  A rank
 *                above s - max(2, oversample / 2) means the sketch saturated;
 *                otherwise the ID is kept when its relative Frobenius
 *                residual on `nchk` hashed rows of K is <= resid_tol.
 *                Saturated or rejected boxes, and boxes without a sketch,
 *                get the full pivoted-QR ID of K with the tol rule (in a
 *                second launch over those boxes; boxes factored on a
 *                thread-block cluster fall back in place).
 *   resid[nbox]  (out, may be NULL) that residual; -1 not tried, -2 the
 *                sketch saturated.
 *   status[nbox] (out, may be NULL) 0 full QR; else 10 (one sketch) + 1
 *                (randomized ID kept) or 2 (rejected, full QR used).
 */
int skf_skel_boxes_randomized(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x,
                              const double* geom, const double* centers, double box_length, int32_t nproxy,
                              double tol, const int32_t* kpred, int32_t oversample, int32_t rho, uint64_t seed,
                              int32_t nchk, double sketch_tol, double resid_tol, double* resid, int8_t* status,
                              int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out, void* stream);

/*
 * Rank predictor of the learned-rank build (no counterpart in the
 * reference): a 3-layer perceptron of width 128 with BF16 weights and
 * activations, trained on log2(rank + 1) of pivoted-QR builds.  Parameters
 * are one vector (FP32 master `theta`, BF16 mirror `theta16`) laid out as
 * W1[128 x nin] b1[128] W2[128 x 128] b2[128] w3[128] b3[1]; inputs are
 * BF16 [n x nin], nin <= 32.  All pointers DEVICE.
 */
int64_t skf_mlp_num_params(int32_t nin);                 /* -1 if nin is out of range */
int64_t skf_mlp_scratch_floats(int32_t nin, int64_t n);  /* scratch of skf_mlp_train_step */
int skf_mlp_bf16(const float* src, void* dst, int64_t n, void* stream);  /* FP32 -> BF16 */
int skf_mlp_predict(int32_t nin, const void* theta16, const void* x16, int64_t n, float* y, void* stream);
/* One full-batch step: grad = d/dtheta mean((y - target)^2) (deterministic
   order); with apply != 0 also an Adam step (bias-corrected, `step` >= 1) on
   theta, adam_m, adam_v and the BF16 mirror.  loss (may be NULL) = the
   batch's mean squared error before the step. */
int skf_mlp_train_step(int32_t nin, float* theta, void* theta16, const void* x16, const float* target, int64_t n,
                       float* scratch, float* grad, float* adam_m, float* adam_v, int32_t step, float lr,
                       float beta1, float beta2, float eps, int32_t apply, float* loss, void* stream);

/*
 * Geometric features of the rank network: for box b the points
 * x[off[b] .. off[b+1]) (row-major [.. x ndim], ndim 2 or 3) relative to
 * centers[b], in units of `width`: out[9 b + 0..2] their mean, out[9 b +
 * 3..8] their second central moments (xx yy zz xy xz yz; z terms 0 in 2D).
 * All pointers DEVICE; one block per box.
 */
int skf_box_moments(int32_t nbox, int32_t ndim, const int64_t* off, const double* x, const double* centers,
                    double width, double* out, void* stream);

/*
 * Point-level front end of the tree build (the tree the reference takes from
 * simpletree.BalancedTree, called at skelfmm/skel_fmm.py:150): for point i
 * of x [n x ndim] (DEVICE, FP64) the integer cell q[i, d] = clamp(floor((x -
 * corner[d]) / L0 * 2^depth), 0, 2^depth - 1) of the root box's finest grid
 * and keys[i], its bit interleave (axis 0 most significant in every
 * ndim-bit group).  corner: DEVICE [ndim]; q may be NULL.  ndim 2 or 3,
 * depth * ndim <= 63.
 */
int skf_morton_keys(int32_t ndim, int64_t n, const double* x, const double* corner, double L0, int32_t depth,
                    uint64_t* keys, int64_t* q, void* stream);

/*
 * Stable ascending sort of n keys (DEVICE) on their low `bits` bits:
 * keys_out (DEVICE [n]) and perm_out (DEVICE [n] int64, the input index of
 * each output key; equal keys keep their input order).  The tree's point
 * order (the point sort of simpletree.BalancedTree, skelfmm/skel_fmm.py:150).
 */
int skf_sort_keys(int64_t n, const uint64_t* keys_in, uint64_t* keys_out, int64_t* perm_out, int32_t bits,
                  void* stream);

/*
 * Box levels and neighbour tables of the adaptive 2:1-balanced tree (the
 * tree the reference takes from simpletree.BalancedTree, called at
 * skelfmm/skel_fmm.py:150; its lists are read at
 * skelfmm/recursive_skel.py:643-653, 692-699), on the device, from the
 * point keys of skf_morton_keys sorted ascending (skeys: DEVICE [n]).
 * A box with more than leaf_size points is split (up to level `depth`);
 * then every leaf at level l-2 touching a box at level l is split until none
 * is left.  Children that would be empty are not created.  Boxes are
 * numbered level by level, in Morton order within a level.  *out receives a
 * tree handle (device memory, released by skf_tree_destroy).
 */
int skf_tree_build(int32_t ndim, int64_t n, const uint64_t* skeys, int32_t depth, int64_t leaf_size,
                   skf_tree** out, void* stream);
int skf_tree_query(const skf_tree* tree, int32_t* nlevels, int64_t* nboxes);
/*
 * Copies the tree's arrays (host or device destinations, any may be NULL;
 * returns after the copies are done): level_sep [nlevels + 1] (HOST) —
 * boxes of level l are [level_sep[l], level_sep[l+1]); per box: code (the
 * level's Morton code), coords [ndim] (integer cell at the box's level),
 * start/end (range in the sorted point order), leaf (0/1), parent (-1 at the
 * root), children [2^ndim] (Morton order, -1 padded), colleagues [3^ndim]
 * (same-level boxes at offsets {-1,0,1}^ndim, axis 0 slowest, self
 * included, -1 where absent) and coarse [2^ndim] (leaves one level up
 * touching the box, parent excluded, compacted, -1 padded).
 */
int skf_tree_export(const skf_tree* tree, int64_t* level_sep, uint64_t* code, int64_t* coords, int64_t* start,
                    int64_t* end, uint8_t* leaf, int64_t* parent, int64_t* children, int64_t* colleagues,
                    int64_t* coarse, void* stream);
void skf_tree_destroy(skf_tree* tree);

/*
 * Translation lists of a skeletonized tree on the device, grouped by target
 * box (replaces the list construction of skelfmm/recursive_skel.py:622-712,
 * get_parallel_lists): for a box b below root_level, its colleagues (row
 * order, KIND_COLLEAGUE) then its coarse neighbours (row order,
 * KIND_COARSE_UP); for every box s, the boxes below root_level that list s
 * as a coarse neighbour, ascending (KIND_COARSE_DOWN); for a root box (in
 * root_boxes: leaves above root_level and the boxes at it, ascending),
 * every root box (KIND_ROOT).  Tables as skf_tree_export writes them
 * (colleagues [nb x 3^ndim], coarse and children [nb x 2^ndim], int64);
 * box_level [nb] int64.  All arrays DEVICE.  skf_lists_count writes
 * list_off [nb + 1] (DEVICE) and the list length to *total (HOST; returns
 * after the stream is done); skf_lists_fill writes list_src (int32) and
 * list_kind (int8) at those offsets.
 */
int skf_lists_count(int32_t ndim, int64_t nboxes, const int64_t* colleagues, const int64_t* coarse,
                    const int64_t* children, const int64_t* box_level, int32_t root_level, const int64_t* root_boxes,
                    int64_t nroot, int64_t* list_off, int64_t* total, void* stream);
int skf_lists_fill(int32_t ndim, int64_t nboxes, const int64_t* colleagues, const int64_t* coarse,
                   const int64_t* children, const int64_t* box_level, int32_t root_level, const int64_t* root_boxes,
                   int64_t nroot, const int64_t* list_off, int32_t* list_src, int8_t* list_kind, void* stream);

/*
 * Level bookkeeping of the build (HOST arrays, no device work), the
 * candidate and skeleton-order steps of skelfmm/recursive_skel.py:209-262,
 * 264-324.  skf_level_candidates: for the nbl boxes of a level, a leaf's
 * candidates are its points perm[box_start[b] .. box_end[b]), a parent's the
 * skeletons of its children in child order (children [nbl x nc], global box
 * ids, -1 padded; child c's skeleton = child_ids[child_off[c -
 * child_first_box] ..][:rank[c]]; child_ids NULL: the child level is not
 * skeletonized and parents have none).  Writes off_out [nbl + 1] and *total;
 * with ids_out non-NULL also ids_out [total] and cand_src_out [total] (the
 * child-level entry each candidate comes from, -1 for points).
 * skf_level_reorder: ids_out[off[b] + j] = ids_in[off[b] + perm[off[b] + j]]
 * (perm box-local) and final_pos[off[b] + perm[off[b] + j]] = off[b] + j.
 */
int skf_level_candidates(int64_t nbl, const uint8_t* is_leaf, const int64_t* box_start, const int64_t* box_end,
                         const int64_t* children, int32_t nc, int64_t child_first_box, const int64_t* child_off,
                         const int64_t* child_ids, const int64_t* rank, const int64_t* perm, int64_t npoints,
                         int64_t* off_out, int64_t* ids_out, int64_t* cand_src_out, int64_t* total);
int skf_level_reorder(int64_t nbl, const int64_t* off, const int32_t* perm, const int64_t* ids_in, int64_t* ids_out,
                      int64_t* final_pos);
/*
 * Parent slots of the ragged build (the index maps of
 * skelfmm/recursive_skel.py:714-780; HOST): pslot [nentries] = -1, then for
 * every level l of nlev and candidate t of it with cand_src[l][t] = c >= 0,
 * pslot[base_child[l] + c] = base_parent[l] + (final_pos[l] ? final_pos[l][t]
 * : t).  skf_gather_i64: out[i] = src[idx[i]] (0 <= idx < nsrc).
 */
int skf_parent_slots(int32_t nlev, const int64_t* const* cand_src, const int64_t* const* final_pos,
                     const int64_t* ncand, const int64_t* base_child, const int64_t* base_parent, int64_t nentries,
                     int64_t* pslot);
int skf_gather_i64(int64_t n, const int64_t* idx, const int64_t* src, int64_t nsrc, int64_t* out);

const char* skf_status_string(int32_t status);
int skf_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SKF_H */
