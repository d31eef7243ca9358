// skf_tree.cu — the point-level front end of the tree build on the device:
// integer cell coordinates of every point on the finest grid of the root box
// and their interleaved (Morton) keys.  The host tree (skelfmm_gb300/tree.py,
// the stand-in for simpletree.BalancedTree called at skelfmm/skel_fmm.py:150)
// sorts by these keys and refines box ranges level by level; computing them
// here gives bit-identical keys (same FP64 operations in the same order, no
// contraction) at HBM speed.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <memory>
#include <new>
#include <vector>

#include "skf_internal.cuh"

namespace skf {

// bit b of v moved to bit b * ndim (v < 2^depth)
__device__ __forceinline__ uint64_t spread_bits(uint64_t v, int ndim, int depth) {
  uint64_t out = 0;
#pragma unroll 4
  for (int b = 0; b < depth; ++b) out |= ((v >> b) & 1ull) << (b * ndim);
  return out;
}

// One thread per point: q = clamp(floor((x - corner) / L0 * 2^depth), 0,
// 2^depth - 1) per axis (FP64, correctly rounded at every step), and the
// key with axis 0 in the most significant bit of every ndim-bit group.
__global__ void k_morton_keys(int ndim, int64_t n, const double* __restrict__ x, const double* __restrict__ corner,
                              double L0, int depth, uint64_t* __restrict__ keys, int64_t* __restrict__ q) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double scale = (double)(1ll << depth);
  const double top = (double)((1ll << depth) - 1);
  uint64_t key = 0;
  for (int d = 0; d < ndim; ++d) {
    double t = __dsub_rn(x[i * ndim + d], corner[d]);
    t = __ddiv_rn(t, L0);
    t = __dmul_rn(t, scale);
    t = floor(t);
    t = fmin(t, top);
    t = fmax(t, 0.0);
    const int64_t c = (int64_t)t;
    if (q) q[i * ndim + d] = c;
    key |= spread_bits((uint64_t)c, ndim, depth) << (ndim - 1 - d);
  }
  keys[i] = key;
}

}  // namespace skf

namespace skf {
__global__ void k_iota64(int64_t n, int64_t* v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}
}  // namespace skf

// Stable sort of the point keys (LSD radix sort over the low `bits` bits,
// CUB, compiled for this GPU): keys_out ascending, perm_out[i] = the input
// index of keys_out[i] (equal keys keep their input order).
extern "C" int skf_sort_keys(int64_t n, const uint64_t* keys_in, uint64_t* keys_out, int64_t* perm_out, int32_t bits,
                             void* stream) {
  if (n < 0 || n > INT32_MAX || bits < 1 || bits > 64) return SKF_ERR_ARG;
  if (n == 0) return SKF_OK;
  if (!keys_in || !keys_out || !perm_out) return SKF_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t* iota = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys_in, keys_out, (const int64_t*)nullptr,
                                                  perm_out, (int)n, 0, bits, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&iota, sizeof(int64_t) * (size_t)n, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&tmp, std::max<size_t>(tmp_bytes, 1), st);
  if (e == cudaSuccess) {
    skf::k_iota64<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, iota);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys_in, keys_out, iota, perm_out, (int)n, 0, bits, st);
  if (tmp) cudaFreeAsync(tmp, st);
  if (iota) cudaFreeAsync(iota, st);
  if (e != cudaSuccess) {
    skf::set_last_cuda_error(e);
    return e == cudaErrorMemoryAllocation ? SKF_ERR_OOM : SKF_ERR_CUDA;
  }
  return SKF_OK;
}

extern "C" int skf_morton_keys(int32_t ndim, int64_t n, const double* x, const double* corner, double L0,
                               int32_t depth, uint64_t* keys, int64_t* q, void* stream) {
  if ((ndim != 2 && ndim != 3) || n < 0 || !(L0 > 0) || depth < 1 || depth * ndim > 63) return SKF_ERR_ARG;
  if (n == 0) return SKF_OK;
  if (!x || !corner || !keys) return SKF_ERR_ARG;
  const int64_t blocks = (n + 255) / 256;
  skf::k_morton_keys<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(ndim, n, x, corner, L0, depth,
                                                                                      keys, q);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

// ---------------------------------------------------------------------------
// Box levels of the tree on the device.  From the sorted point keys alone:
// a box at level l with code k (the top d*l bits of its points' keys) holds
// the contiguous key range whose keys shifted right by d*(depth-l) equal k;
// its non-empty children are found by 2^d - 1 binary searches in that range.
// A level is always regenerated whole from the level above (the children of
// every non-leaf box, in parent order then child order, which is the level's
// Morton order), carrying the leaf flags of boxes that existed before.
//
// Refinement splits every leaf holding more than leaf_size points, level by
// level; the 2:1 balance then splits every leaf at level l-2 that touches a
// box at level l (faces, edges and corners), deepest level first, until no
// such leaf is left.  The tree is the least refinement with both properties,
// so it does not depend on the order the splits are found in; the host tree
// (skelfmm_gb300/tree.py) computes the same one.  Neighbour tables: parent,
// children (Morton order, -1 padded), colleagues (offsets {-1,0,1}^d with
// axis 0 slowest, self included, -1 where absent) and coarse neighbours
// (leaves one level up that touch the box, the parent excluded, candidates
// in the order of offsets {0,1}^d from the lowest touching cell, compacted).
// ---------------------------------------------------------------------------

struct skf_tree {
  int ndim = 0, nlevels = 0;
  int64_t nboxes = 0;
  std::vector<int64_t> level_sep;
  std::vector<void*> allocations;
  uint64_t* code = nullptr;
  int64_t* coords = nullptr;
  int64_t* start = nullptr;
  int64_t* end = nullptr;
  uint8_t* leaf = nullptr;
  int64_t* parent = nullptr;
  int64_t* children = nullptr;
  int64_t* colleagues = nullptr;
  int64_t* coarse = nullptr;
  ~skf_tree() {
    for (void* p : allocations) cudaFree(p);
  }
};

namespace skf {
namespace tree {

// bit b * ndim of v moved to bit b
__device__ __forceinline__ uint64_t compact_bits(uint64_t v, int ndim, int nbits) {
  uint64_t out = 0;
  for (int b = 0; b < nbits; ++b) out |= ((v >> (b * ndim)) & 1ull) << b;
  return out;
}

__device__ __forceinline__ uint64_t encode(const int64_t* c, int ndim, int nbits) {
  uint64_t k = 0;
  for (int d = 0; d < ndim; ++d) k |= spread_bits((uint64_t)c[d], ndim, nbits) << (ndim - 1 - d);
  return k;
}

__device__ __forceinline__ void decode(uint64_t k, int ndim, int nbits, int64_t* c) {
  for (int d = 0; d < ndim; ++d) c[d] = (int64_t)compact_bits(k >> (ndim - 1 - d), ndim, nbits);
}

// first index in [lo, hi) with a[i] >= v (hi when none)
__device__ __forceinline__ int64_t lower_bound(const uint64_t* a, int64_t lo, int64_t hi, uint64_t v) {
  while (lo < hi) {
    const int64_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int64_t find(const uint64_t* a, int64_t n, uint64_t v) {
  const int64_t p = lower_bound(a, 0, n, v);
  return (p < n && a[p] == v) ? p : -1;
}

// floor(a / b) for b > 0
__device__ __forceinline__ int64_t fdiv(int64_t a, int64_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

struct Level {
  uint64_t* code = nullptr;
  int64_t* start = nullptr;
  int64_t* end = nullptr;
  uint8_t* leaf = nullptr;
  int64_t n = 0;
};

__global__ void k_mark_big(int64_t n, const int64_t* start, const int64_t* end, uint8_t* leaf, int64_t leaf_size,
                           int* any) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (leaf[i] && end[i] - start[i] > leaf_size) {
    leaf[i] = 0;
    *any = 1;
  }
}

// Child c of box i: key range [bnd[c], bnd[c+1]) inside [start, end).
__device__ __forceinline__ void child_bounds(const uint64_t* skeys, uint64_t code, int64_t s, int64_t e, int ndim,
                                             int shift, int64_t* bnd) {
  const int nc = 1 << ndim;
  bnd[0] = s;
  bnd[nc] = e;
  for (int c = 1; c < nc; ++c)
    bnd[c] = lower_bound(skeys, bnd[c - 1], e, ((code << ndim) | (uint64_t)c) << shift);
}

__global__ void k_child_count(Level L, const uint64_t* skeys, int ndim, int shift, int64_t* cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  int64_t c = 0;
  if (!L.leaf[i]) {
    int64_t bnd[9];
    child_bounds(skeys, L.code[i], L.start[i], L.end[i], ndim, shift, bnd);
    for (int k = 0; k < (1 << ndim); ++k) c += bnd[k + 1] > bnd[k];
  }
  cnt[i] = c;
}

__global__ void k_child_write(Level L, const uint64_t* skeys, int ndim, int shift, const int64_t* off, Level old,
                              Level out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n || L.leaf[i]) return;
  int64_t bnd[9];
  child_bounds(skeys, L.code[i], L.start[i], L.end[i], ndim, shift, bnd);
  int64_t o = off[i];
  for (int k = 0; k < (1 << ndim); ++k) {
    if (bnd[k + 1] <= bnd[k]) continue;
    const uint64_t code = (L.code[i] << ndim) | (uint64_t)k;
    out.code[o] = code;
    out.start[o] = bnd[k];
    out.end[o] = bnd[k + 1];
    const int64_t p = old.n ? find(old.code, old.n, code) : -1;
    out.leaf[o] = p >= 0 ? old.leaf[p] : 1;
    ++o;
  }
}

// Exclusive prefix sum of cnt[0..n) into off[0..n] (one block).
__global__ void k_scan(int64_t n, const int64_t* cnt, int64_t* off) {
  __shared__ int64_t part[1024];
  const int t = threadIdx.x;
  const int64_t chunk = (n + blockDim.x - 1) / blockDim.x;
  const int64_t a = min(n, (int64_t)t * chunk), b = min(n, a + chunk);
  int64_t s = 0;
  for (int64_t i = a; i < b; ++i) s += cnt[i];
  part[t] = s;
  __syncthreads();
  for (int w = 1; w < (int)blockDim.x; w <<= 1) {
    const int64_t v = t >= w ? part[t - w] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int64_t run = part[t] - s;
  for (int64_t i = a; i < b; ++i) {
    off[i] = run;
    run += cnt[i];
  }
  if (t == (int)blockDim.x - 1) off[n] = part[t];
}

// Leaves at level lev - 2 touching a box of level lev lose their leaf flag.
__global__ void k_balance_mark(Level L, int lev, int ndim, Level up2, int* any) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  int64_t C[3], g0[3], g1[3], G[3];
  decode(L.code[i], ndim, lev, C);
  const int64_t nmax = (1ll << (lev - 2)) - 1;
  for (int d = 0; d < ndim; ++d) {
    g0[d] = max((int64_t)0, -fdiv(4 - C[d], 4));
    g1[d] = min(nmax, fdiv(C[d] + 1, 4));
  }
  for (int t = 0; t < (1 << ndim); ++t) {
    bool ok = true;
    for (int d = 0; d < ndim; ++d) {
      G[d] = g0[d] + ((t >> (ndim - 1 - d)) & 1);
      ok = ok && G[d] <= g1[d];
    }
    if (!ok) continue;
    const int64_t p = find(up2.code, up2.n, encode(G, ndim, lev - 2));
    if (p >= 0 && up2.leaf[p]) {
      up2.leaf[p] = 0;
      *any = 1;
    }
  }
}

// Per box of level lev (global index base + i): coordinates, parent, child
// slot in the parent's row, colleagues and coarse neighbours.
__global__ void k_tables(Level L, int lev, int ndim, int64_t base, Level up, int64_t up_base, int64_t* coords,
                         int64_t* parent, int64_t* children, int64_t* colleagues, int64_t* coarse) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  const int64_t gi = base + i;
  const int nc = 1 << ndim;
  const int nq = ndim == 2 ? 9 : 27;
  int64_t C[3], G[3];
  const uint64_t code = L.code[i];
  decode(code, ndim, lev, C);
  for (int d = 0; d < ndim; ++d) coords[gi * ndim + d] = C[d];
  const int64_t nmax = (1ll << lev) - 1;
  for (int k = 0; k < nq; ++k) {
    bool ok = true;
    int r = k;
    for (int d = ndim - 1; d >= 0; --d) {
      G[d] = C[d] + (r % 3) - 1;
      r /= 3;
      ok = ok && G[d] >= 0 && G[d] <= nmax;
    }
    const int64_t p = ok ? find(L.code, L.n, encode(G, ndim, lev)) : -1;
    colleagues[gi * nq + k] = p >= 0 ? base + p : -1;
  }
  if (lev == 0) {
    parent[gi] = -1;
    for (int t = 0; t < nc; ++t) coarse[gi * nc + t] = -1;
    return;
  }
  const int64_t p = find(up.code, up.n, code >> ndim);
  parent[gi] = p >= 0 ? up_base + p : -1;
  if (p >= 0) {
    const int64_t first = lower_bound(L.code, 0, L.n, (code >> ndim) << ndim);
    children[(up_base + p) * nc + (i - first)] = gi;
  }
  const int64_t nmax_up = (1ll << (lev - 1)) - 1;
  int64_t g0[3], g1[3];
  for (int d = 0; d < ndim; ++d) {
    g0[d] = max((int64_t)0, -fdiv(2 - C[d], 2));
    g1[d] = min(nmax_up, fdiv(C[d] + 1, 2));
  }
  int m = 0;
  for (int t = 0; t < nc; ++t) {
    bool ok = true, is_par = true;
    for (int d = 0; d < ndim; ++d) {
      G[d] = g0[d] + ((t >> (ndim - 1 - d)) & 1);
      ok = ok && G[d] <= g1[d];
      is_par = is_par && G[d] == (C[d] >> 1);
    }
    if (!ok || is_par) continue;
    const int64_t q = find(up.code, up.n, encode(G, ndim, lev - 1));
    if (q >= 0 && up.leaf[q]) coarse[gi * nc + m++] = up_base + q;
  }
  for (; m < nc; ++m) coarse[gi * nc + m] = -1;
}

constexpr int kTB = 256;
inline unsigned nblk(int64_t n) { return (unsigned)((n + kTB - 1) / kTB); }

}  // namespace tree
}  // namespace skf

namespace {

// Device allocations of one build; released unless handed to a tree.
struct Pool {
  std::vector<void*> p;
  template <class T>
  T* get(int64_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * (size_t)std::max<int64_t>(n, 1)) != cudaSuccess) return nullptr;
    p.push_back(q);
    return static_cast<T*>(q);
  }
  void release(void* q) {
    for (auto& x : p)
      if (x == q) {
        cudaFree(x);
        x = nullptr;
      }
  }
  ~Pool() {
    for (void* x : p)
      if (x) cudaFree(x);
  }
};

}  // namespace

extern "C" int skf_tree_build(int32_t ndim, int64_t n, const uint64_t* skeys, int32_t depth, int64_t leaf_size,
                              skf_tree** out, void* stream) {
  using namespace skf::tree;
  if (!out) return SKF_ERR_ARG;
  *out = nullptr;
  if ((ndim != 2 && ndim != 3) || n < 1 || depth < 1 || depth * ndim > 63 || leaf_size < 1 || !skeys)
    return SKF_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Pool pool;
  int* dany = pool.get<int>(1);
  int64_t* dtot = pool.get<int64_t>(1);
  if (!dany || !dtot) return SKF_ERR_OOM;
  auto alloc_level = [&](Level& L, int64_t m) -> bool {
    L.n = m;
    L.code = pool.get<uint64_t>(m);
    L.start = pool.get<int64_t>(m);
    L.end = pool.get<int64_t>(m);
    L.leaf = pool.get<uint8_t>(m);
    return L.code && L.start && L.end && L.leaf;
  };
  auto free_level = [&](Level& L) {
    pool.release(L.code);
    pool.release(L.start);
    pool.release(L.end);
    pool.release(L.leaf);
    L = Level();
  };
  auto read_flag = [&](int* flag) -> int {
    int h = 0;
    if (cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return -1;
    return h;
  };
  std::vector<Level> lv(1);
  if (!alloc_level(lv[0], 1)) return SKF_ERR_OOM;
  {
    const uint64_t c0 = 0;
    const int64_t s0 = 0, e0 = n;
    const uint8_t l0 = 1;
    SKF_CUDA_TRY(cudaMemcpyAsync(lv[0].code, &c0, sizeof(c0), cudaMemcpyHostToDevice, st));
    SKF_CUDA_TRY(cudaMemcpyAsync(lv[0].start, &s0, sizeof(s0), cudaMemcpyHostToDevice, st));
    SKF_CUDA_TRY(cudaMemcpyAsync(lv[0].end, &e0, sizeof(e0), cudaMemcpyHostToDevice, st));
    SKF_CUDA_TRY(cudaMemcpyAsync(lv[0].leaf, &l0, sizeof(l0), cudaMemcpyHostToDevice, st));
  }
  // level lev + 1 rebuilt from level lev (the children of its non-leaf boxes)
  auto regen = [&](int lev) -> int {
    Level& L = lv[lev];
    int64_t* cnt = pool.get<int64_t>(L.n);
    int64_t* off = pool.get<int64_t>(L.n + 1);
    if (!cnt || !off) return SKF_ERR_OOM;
    const int shift = ndim * (depth - lev - 1);
    k_child_count<<<nblk(L.n), kTB, 0, st>>>(L, skeys, ndim, shift, cnt);
    k_scan<<<1, 1024, 0, st>>>(L.n, cnt, off);
    int64_t total = 0;
    SKF_CUDA_TRY(cudaMemcpyAsync(&total, off + L.n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SKF_CUDA_TRY(cudaStreamSynchronize(st));
    Level old = (int)lv.size() > lev + 1 ? lv[lev + 1] : Level();
    Level nw;
    if (!alloc_level(nw, total)) return SKF_ERR_OOM;
    k_child_write<<<nblk(L.n), kTB, 0, st>>>(L, skeys, ndim, shift, off, old, nw);
    SKF_CUDA_TRY(cudaGetLastError());
    SKF_CUDA_TRY(cudaStreamSynchronize(st));
    if ((int)lv.size() > lev + 1) {
      free_level(lv[lev + 1]);
      lv[lev + 1] = nw;
    } else {
      lv.push_back(nw);
    }
    pool.release(cnt);
    pool.release(off);
    return SKF_OK;
  };
  // refinement
  for (int lev = 0; lev < depth; ++lev) {
    SKF_CUDA_TRY(cudaMemsetAsync(dany, 0, sizeof(int), st));
    k_mark_big<<<nblk(lv[lev].n), kTB, 0, st>>>(lv[lev].n, lv[lev].start, lv[lev].end, lv[lev].leaf, leaf_size,
                                                 dany);
    const int any = read_flag(dany);
    if (any < 0) return SKF_ERR_CUDA;
    if (!any) break;
    int s = regen(lev);
    if (s != SKF_OK) return s;
  }
  // 2:1 balance
  for (bool changed = true; changed;) {
    changed = false;
    for (int lev = (int)lv.size() - 1; lev >= 2; --lev) {
      if (lv[lev].n == 0) continue;
      SKF_CUDA_TRY(cudaMemsetAsync(dany, 0, sizeof(int), st));
      k_balance_mark<<<nblk(lv[lev].n), kTB, 0, st>>>(lv[lev], lev, ndim, lv[lev - 2], dany);
      const int any = read_flag(dany);
      if (any < 0) return SKF_ERR_CUDA;
      if (any) {
        int s = regen(lev - 2);
        if (s != SKF_OK) return s;
        changed = true;
      }
    }
  }
  int nlev = (int)lv.size();
  while (nlev > 0 && lv[nlev - 1].n == 0) --nlev;
  auto t = new (std::nothrow) skf_tree();
  if (!t) return SKF_ERR_OOM;
  std::unique_ptr<skf_tree> own(t);
  t->ndim = ndim;
  t->nlevels = nlev;
  t->level_sep.assign(nlev + 1, 0);
  for (int l = 0; l < nlev; ++l) t->level_sep[l + 1] = t->level_sep[l] + lv[l].n;
  const int64_t nb = t->level_sep[nlev];
  t->nboxes = nb;
  const int nc = 1 << ndim, nq = ndim == 2 ? 9 : 27;
  auto talloc = [&](size_t bytes) -> void* {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(bytes, 1)) != cudaSuccess) return nullptr;
    t->allocations.push_back(q);
    return q;
  };
  t->code = (uint64_t*)talloc(8 * nb);
  t->coords = (int64_t*)talloc(8 * nb * ndim);
  t->start = (int64_t*)talloc(8 * nb);
  t->end = (int64_t*)talloc(8 * nb);
  t->leaf = (uint8_t*)talloc(nb);
  t->parent = (int64_t*)talloc(8 * nb);
  t->children = (int64_t*)talloc(8 * nb * nc);
  t->colleagues = (int64_t*)talloc(8 * nb * nq);
  t->coarse = (int64_t*)talloc(8 * nb * nc);
  if (!t->code || !t->coords || !t->start || !t->end || !t->leaf || !t->parent || !t->children || !t->colleagues ||
      !t->coarse)
    return SKF_ERR_OOM;
  SKF_CUDA_TRY(cudaMemsetAsync(t->children, 0xff, 8 * nb * nc, st));
  for (int l = 0; l < nlev; ++l) {
    const int64_t b = t->level_sep[l], m = lv[l].n;
    SKF_CUDA_TRY(cudaMemcpyAsync(t->code + b, lv[l].code, 8 * m, cudaMemcpyDeviceToDevice, st));
    SKF_CUDA_TRY(cudaMemcpyAsync(t->start + b, lv[l].start, 8 * m, cudaMemcpyDeviceToDevice, st));
    SKF_CUDA_TRY(cudaMemcpyAsync(t->end + b, lv[l].end, 8 * m, cudaMemcpyDeviceToDevice, st));
    SKF_CUDA_TRY(cudaMemcpyAsync(t->leaf + b, lv[l].leaf, m, cudaMemcpyDeviceToDevice, st));
    const Level up = l > 0 ? lv[l - 1] : Level();
    k_tables<<<nblk(m), kTB, 0, st>>>(lv[l], l, ndim, b, up, l > 0 ? t->level_sep[l - 1] : 0, t->coords, t->parent,
                                      t->children, t->colleagues, t->coarse);
  }
  SKF_CUDA_TRY(cudaGetLastError());
  SKF_CUDA_TRY(cudaStreamSynchronize(st));
  *out = own.release();
  return SKF_OK;
}

extern "C" int skf_tree_query(const skf_tree* t, int32_t* nlevels, int64_t* nboxes) {
  if (!t) return SKF_ERR_ARG;
  if (nlevels) *nlevels = t->nlevels;
  if (nboxes) *nboxes = t->nboxes;
  return SKF_OK;
}

extern "C" int skf_tree_export(const skf_tree* t, int64_t* level_sep, uint64_t* code, int64_t* coords,
                               int64_t* start, int64_t* end, uint8_t* leaf, int64_t* parent, int64_t* children,
                               int64_t* colleagues, int64_t* coarse, void* stream) {
  if (!t) return SKF_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t nb = t->nboxes;
  const int nc = 1 << t->ndim, nq = t->ndim == 2 ? 9 : 27;
  if (level_sep) std::copy(t->level_sep.begin(), t->level_sep.end(), level_sep);
  auto cp = [&](void* dst, const void* src, size_t bytes) -> int {
    if (!dst || bytes == 0) return SKF_OK;
    SKF_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st));
    return SKF_OK;
  };
  int s = SKF_OK;
  if (s == SKF_OK) s = cp(code, t->code, 8 * nb);
  if (s == SKF_OK) s = cp(coords, t->coords, 8 * nb * t->ndim);
  if (s == SKF_OK) s = cp(start, t->start, 8 * nb);
  if (s == SKF_OK) s = cp(end, t->end, 8 * nb);
  if (s == SKF_OK) s = cp(leaf, t->leaf, nb);
  if (s == SKF_OK) s = cp(parent, t->parent, 8 * nb);
  if (s == SKF_OK) s = cp(children, t->children, 8 * nb * nc);
  if (s == SKF_OK) s = cp(colleagues, t->colleagues, 8 * nb * nq);
  if (s == SKF_OK) s = cp(coarse, t->coarse, 8 * nb * nc);
  if (s != SKF_OK) return s;
  SKF_CUDA_TRY(cudaStreamSynchronize(st));
  return SKF_OK;
}

extern "C" void skf_tree_destroy(skf_tree* t) { delete t; }

// ---------------------------------------------------------------------------
// Translation lists on the device (the lists of
// skelfmm/recursive_skel.py:622-712, grouped by target box): for a target
// box b below the root level, its colleagues (row order, self included,
// KIND_COLLEAGUE) and its coarse neighbours (row order, KIND_COARSE_UP);
// for every box s, the boxes t below the root level that list s as a
// coarse neighbour, ascending (KIND_COARSE_DOWN); for a root box (a leaf
// above the root level or a box at it), every root box ascending
// (KIND_ROOT).  A box t listing s as a coarse neighbour is a child of a
// colleague of s other than s, so the down list is found from s's
// colleagues (sorted) and their children (consecutive, ascending).
// ---------------------------------------------------------------------------

namespace skf {
namespace tree {

struct ListArgs {
  int64_t nb = 0;
  int nq = 0, nc = 0;
  const int64_t* colleagues = nullptr;
  const int64_t* coarse = nullptr;
  const int64_t* children = nullptr;
  const int64_t* level = nullptr;
  int64_t root_level = 0;
  const int64_t* root_boxes = nullptr;
  int64_t nroot = 0;
};

__device__ __forceinline__ bool lists_as_coarse(const ListArgs& a, int64_t t, int64_t s) {
  for (int k = 0; k < a.nc; ++k) {
    const int64_t v = a.coarse[t * a.nc + k];
    if (v < 0) break;
    if (v == s) return true;
  }
  return false;
}

// Visits the coarse-down sources of box s in ascending order.
template <class F>
__device__ __forceinline__ void for_down(const ListArgs& a, int64_t s, F&& f) {
  int64_t col[27];
  int m = 0;
  for (int k = 0; k < a.nq; ++k) {
    const int64_t p = a.colleagues[s * a.nq + k];
    if (p < 0 || p == s) continue;
    int j = m++;
    while (j > 0 && col[j - 1] > p) {
      col[j] = col[j - 1];
      --j;
    }
    col[j] = p;
  }
  for (int i = 0; i < m; ++i)
    for (int c = 0; c < a.nc; ++c) {
      const int64_t t = a.children[col[i] * a.nc + c];
      if (t < 0) break;
      if (a.level[t] > a.root_level && lists_as_coarse(a, t, s)) f(t);
    }
}

__device__ __forceinline__ bool is_root_box(const ListArgs& a, int64_t b) {
  int64_t lo = 0, hi = a.nroot;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a.root_boxes[mid] < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < a.nroot && a.root_boxes[lo] == b;
}

__global__ void k_list_count(ListArgs a, int64_t* cnt) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nb) return;
  int64_t c = 0;
  if (a.level[b] > a.root_level) {
    for (int k = 0; k < a.nq; ++k) c += a.colleagues[b * a.nq + k] >= 0;
    for (int k = 0; k < a.nc; ++k) c += a.coarse[b * a.nc + k] >= 0;
  }
  for_down(a, b, [&](int64_t) { ++c; });
  if (is_root_box(a, b)) c += a.nroot;
  cnt[b] = c;
}

__global__ void k_list_fill(ListArgs a, const int64_t* off, int32_t* src, int8_t* kind) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nb) return;
  int64_t o = off[b];
  if (a.level[b] > a.root_level) {
    for (int k = 0; k < a.nq; ++k) {
      const int64_t v = a.colleagues[b * a.nq + k];
      if (v < 0) continue;
      src[o] = (int32_t)v;
      kind[o++] = SKF_KIND_COLLEAGUE;
    }
    for (int k = 0; k < a.nc; ++k) {
      const int64_t v = a.coarse[b * a.nc + k];
      if (v < 0) continue;
      src[o] = (int32_t)v;
      kind[o++] = SKF_KIND_COARSE_UP;
    }
  }
  for_down(a, b, [&](int64_t t) {
    src[o] = (int32_t)t;
    kind[o++] = SKF_KIND_COARSE_DOWN;
  });
  if (is_root_box(a, b))
    for (int64_t r = 0; r < a.nroot; ++r) {
      src[o] = (int32_t)a.root_boxes[r];
      kind[o++] = SKF_KIND_ROOT;
    }
}

}  // namespace tree
}  // namespace skf

namespace {

int list_args(int32_t ndim, int64_t nboxes, const int64_t* colleagues, const int64_t* coarse, const int64_t* children,
              const int64_t* box_level, int32_t root_level, const int64_t* root_boxes, int64_t nroot,
              skf::tree::ListArgs& a) {
  if ((ndim != 2 && ndim != 3) || nboxes < 1 || nboxes > INT32_MAX || nroot < 0 || nroot > nboxes ||
      root_level < 0 || !colleagues || !coarse || !children || !box_level || (nroot > 0 && !root_boxes))
    return SKF_ERR_ARG;
  a.nb = nboxes;
  a.nq = ndim == 2 ? 9 : 27;
  a.nc = 1 << ndim;
  a.colleagues = colleagues;
  a.coarse = coarse;
  a.children = children;
  a.level = box_level;
  a.root_level = root_level;
  a.root_boxes = root_boxes;
  a.nroot = nroot;
  return SKF_OK;
}

}  // namespace

extern "C" int skf_lists_count(int32_t ndim, int64_t nboxes, const int64_t* colleagues, const int64_t* coarse,
                               const int64_t* children, const int64_t* box_level, int32_t root_level,
                               const int64_t* root_boxes, int64_t nroot, int64_t* list_off, int64_t* total,
                               void* stream) {
  using namespace skf::tree;
  ListArgs a;
  const int s = list_args(ndim, nboxes, colleagues, coarse, children, box_level, root_level, root_boxes, nroot, a);
  if (s != SKF_OK) return s;
  if (!list_off || !total) return SKF_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t* cnt = nullptr;
  SKF_CUDA_TRY(cudaMallocAsync(&cnt, sizeof(int64_t) * nboxes, st));
  k_list_count<<<nblk(nboxes), kTB, 0, st>>>(a, cnt);
  k_scan<<<1, 1024, 0, st>>>(nboxes, cnt, list_off);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(total, list_off + nboxes, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(cnt, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  SKF_CUDA_TRY(e);
  return SKF_OK;
}

extern "C" int skf_lists_fill(int32_t ndim, int64_t nboxes, const int64_t* colleagues, const int64_t* coarse,
                              const int64_t* children, const int64_t* box_level, int32_t root_level,
                              const int64_t* root_boxes, int64_t nroot, const int64_t* list_off, int32_t* list_src,
                              int8_t* list_kind, void* stream) {
  using namespace skf::tree;
  ListArgs a;
  const int s = list_args(ndim, nboxes, colleagues, coarse, children, box_level, root_level, root_boxes, nroot, a);
  if (s != SKF_OK) return s;
  if (!list_off || !list_src || !list_kind) return SKF_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_list_fill<<<nblk(nboxes), kTB, 0, st>>>(a, list_off, list_src, list_kind);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}
