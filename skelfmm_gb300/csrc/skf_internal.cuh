// skf_internal.cuh — plan layout and helpers shared by the CUDA sources.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/skf.h"

#define SKF_CUDA_TRY(expr)                 \
  do {                                     \
    cudaError_t _e = (expr);               \
    if (_e != cudaSuccess) {               \
      skf::set_last_cuda_error_at(_e, __FILE__, __LINE__); \
      return SKF_ERR_CUDA;                 \
    }                                      \
  } while (0)

namespace skf {

void set_last_cuda_error(cudaError_t e);
// as set_last_cuda_error, naming the failing call's source line in the
// status string
void set_last_cuda_error_at(cudaError_t e, const char* file, int line);

// Translation kernel geometry: 128 threads per block; rows per thread depend
// on the precision (FP64: 1, mixed: 2).
constexpr int kTransThreads = 128;  // FP64 translation block
constexpr int kRowsPerThreadF64 = 1;
constexpr int kT32Threads = 64;     // mixed translation block
constexpr int kRowsPerThreadF32 = 4;
constexpr int kTileSrcF64 = 64;
constexpr int kTileSrcF32 = 128;

struct LevelBoxes {
  int32_t* dev = nullptr;  // box ids at this level with rank > 0
  int n = 0;
  int max_red = 0;   // max (bs - rank)
  int max_rank = 0;  // max rank
};

struct WorkList {
  int32_t* box = nullptr;
  int32_t* row = nullptr;
  int n = 0;
};

}  // namespace skf

// HBM layout of a built operator.  Entries of box b occupy
// [box_off[b], box_off[b+1]) in every per-entry array.
struct skf_plan {
  int op = 0, ndim = 3, nboxes = 0, nlevels = 0, root_level = 0;
  bool cplx = false;
  bool scalar_mixed = false;  // force the scalar FP32 translation kernel (comparison/testing)
  int x2_config = 0;          // packed kernel: 0 = 4 warps x 1 pair, 1 = 1 x 4, 2 = 2 x 2, 3 = 1 x 1 (64-row items)
  int sym_shape = 0;          // symmetric kernel tile shape (SKF_OPT_SYM_SHAPE)
  // symmetric translations (mixed path, symmetric point kernels, symmetric lists)
  bool sym_ok = false;  // usable for this plan
  bool sym_on = true;   // option SKF_OPT_SYMMETRIC
  int64_t* sym_list_off = nullptr;
  int32_t* sym_list_src = nullptr;
  int8_t* sym_list_kind = nullptr;
  int64_t* sym_list_poff = nullptr;
  int64_t* box_pbase = nullptr;
  int64_t* box_pstride = nullptr;
  int64_t* in_off = nullptr;
  int64_t* in_blk = nullptr;
  // source-split symmetric kernel (SKF_OPT_SYM_SHAPE 4): items (box, row
  // tile, part), a box's tiles split into box_nparts contiguous parts; parts
  // past the first add their row sums through float-float A-side partial
  // regions at box_apart (4 x bs floats per extra part), listed with the
  // B-side partials in in_off_w / in_blk_w
  int32_t* symw_part = nullptr;
  int32_t* box_ntiles = nullptr;
  int32_t* box_nparts = nullptr;
  int64_t* box_apart = nullptr;
  int64_t* in_off_w = nullptr;
  int64_t* in_blk_w = nullptr;
  int* symw_queue = nullptr;  // item counter of the persistent form (shape 5)
  float* pbuf = nullptr;
  int64_t sym_pairs = 0;  // kernel evaluations per apply on the symmetric path
  int max_bs = 0;         // largest box
  double kappa = 0.0;
  int64_t E = 0, N = 0, nperm = 0, t_len = 0, nlist = 0;
  int64_t pairs = 0;  // kernel evaluations per apply
  double rows_256_over_64 = 1.0;  // padded rows of 256-row over 64-row work items

  // per box
  int64_t* box_off = nullptr;
  int32_t* box_rank = nullptr;
  // per entry
  double4_32a* xyz64 = nullptr;   // (x, y, z, 0)
  double4_32a* geom64 = nullptr;  // (nx, ny, nz, 0) or null
  float4* hi32 = nullptr;     // fl32(s), s = x translated into one binade
  float4* lo32 = nullptr;     // fl32(s - fl32(s))
  float4* geom32 = nullptr;   // fl32(n)
  float4* geom32lo = nullptr; // fl32(n - fl32(n))
  int64_t* pslot = nullptr;
  // leaf permutation
  int64_t* perm_entry = nullptr;
  int64_t* perm_point = nullptr;
  // T blocks
  int64_t* t_off = nullptr;
  double* t64 = nullptr;
  float* t32 = nullptr;    // fl32(T)
  float* t32lo = nullptr;  // fl32(T - fl32(T)): float-float T of the mixed apply
  // interaction lists
  int64_t* list_off = nullptr;
  int32_t* list_src = nullptr;
  int8_t* list_kind = nullptr;
  skf::WorkList work64, work32, worksym, worksymw;
  skf::WorkList work32s;  // 64-row tiles of the packed kernel's one-warp shape (small boxes)
  skf::WorkList red;  // partial reduction items: box, 256-entry chunk (in .row)
  std::vector<skf::LevelBoxes> levels;  // indexed by level
  // apply vectors (scalars; complex: 2 doubles per entry)
  double* q = nullptr;
  double* qh = nullptr;
  // FP32 effective charges for the mixed translations (written after the
  // upward pass): q32 = q; qhn32 = -qskel on skeleton entries, else 0;
  // qd32 = q - qskel on skeleton entries, else q.
  float* q32 = nullptr;
  float* qhn32 = nullptr;
  float* qd32 = nullptr;
  int32_t* entry_skel = nullptr;  // 1 if the entry is in its box's skeleton
  double* u = nullptr;
  double* uh = nullptr;
  double* xbuf = nullptr;  // staging for apply_host
  double* ybuf = nullptr;
  int64_t device_bytes = 0;
  std::vector<void*> allocations;
};
