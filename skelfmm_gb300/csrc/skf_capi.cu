// skf_capi.cu — extern "C" entry points (declared in include/skf.h): plan
// creation from a ragged build, apply (device or host buffers), the batched
// kernel-block seam, and status strings.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <thread>
#include <unordered_map>
#include <vector>

#include "skf_internal.cuh"

namespace skf {

int plan_apply_device(skf_plan* p, const double* x, double* y, int precision, cudaStream_t st);
int plan_time_translations(skf_plan* p, bool mixed, int reps, cudaStream_t st, float* ms);
int kernel_apply(int op, double kappa, int npairs, int mmax, int nmax, const int32_t* m, const int32_t* n,
                 const double* xt, const double* xs, const double* gt, const double* gs, const double* q,
                 const int8_t* sf, double* out, bool mixed, cudaStream_t st);
int skel_boxes(int op, double kappa, int nbox, const int64_t* off, const double* x, const double* geom,
               const double* centers, double box_length, const double* box_lens, int nproxy, double tol,
               int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out, cudaStream_t st);
int skel_boxes_randomized(int op, double kappa, int nbox, const int64_t* off, const double* x, const double* geom,
                          const double* centers, double box_length, int nproxy, double tol, const int32_t* kpred,
                          int oversample, int rho, uint64_t seed, int nchk, double sketch_tol, double resid_tol,
                          double* resid, int8_t* status, int32_t* rank, int32_t* perm, const int64_t* t_off_out,
                          void* t_out, cudaStream_t st);
int proxy_rows(int op, int nproxy);
int trim_workspace();
int convert_f64_f32(const double* src, float* dst, int64_t n, cudaStream_t st);
int split_f64(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st);
int copy_segments(int64_t nseg, const int64_t* src_off, const int64_t* dst_off, const int64_t* len,
                  const void* src, void* dst, int elem_bytes, cudaStream_t st);

static thread_local cudaError_t g_last_cuda = cudaSuccess;
static thread_local char g_last_where[192] = "";
void set_last_cuda_error(cudaError_t e) {
  g_last_cuda = e;
  g_last_where[0] = 0;
}
void set_last_cuda_error_at(cudaError_t e, const char* file, int line) {
  g_last_cuda = e;
  const char* base = strrchr(file, '/');
  snprintf(g_last_where, sizeof(g_last_where), "%s (%s:%d)", cudaGetErrorString(e), base ? base + 1 : file, line);
}

static bool op_is_complex(int op) {
  return op == SKF_HELMHOLTZ_2D || op == SKF_HELMHOLTZ_3D || op == SKF_HELMHOLTZ_DOUBLE_LAYER_3D ||
         op == SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D;
}
static bool op_needs_geom(int op) { return op >= SKF_LAPLACE_DOUBLE_LAYER_3D && op <= SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D; }
static int op_dim(int op) { return (op == SKF_LAPLACE_2D || op == SKF_HELMHOLTZ_2D) ? 2 : 3; }

template <typename T>
static int upload(skf_plan* p, T** dst, const T* src, size_t n) {
  *dst = nullptr;
  if (n == 0) return SKF_OK;
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, n * sizeof(T));
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return SKF_ERR_OOM;
  }
  p->allocations.push_back(d);
  p->device_bytes += (int64_t)(n * sizeof(T));
  if (src != nullptr) {
    e = cudaMemcpy(d, src, n * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      return SKF_ERR_CUDA;
    }
  }
  *dst = static_cast<T*>(d);
  return SKF_OK;
}

// f(lo, hi) over [0, n) split across up to 16 host threads (inline below
// `grain` items per thread).
template <class F>
static void parallel_ranges(int64_t n, F&& f, int64_t grain = 1 << 15) {
  const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
  const int nt = (int)std::min<int64_t>(std::min<int64_t>(hw, 16), (n + grain - 1) / grain);
  if (nt <= 1) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; ++t) th.emplace_back([&f, n, nt, t] { f(n * t / nt, n * (t + 1) / nt); });
  for (auto& x : th) x.join();
}

static void free_plan(skf_plan* p) {
  if (!p) return;
  for (void* a : p->allocations) cudaFree(a);
  delete p;
}

// ---- entry preparation and list checks on the device (plan creation)
constexpr int kPrepThreads = 256;
constexpr int kPrepBlocks = 304;  // 2 per SM on 152 SMs

// Per block: min and max of every coordinate (part[6 b + k], part[6 b + 3 +
// k]); *bad = 1 when a coordinate or normal is not finite.
__global__ void __launch_bounds__(kPrepThreads) k_entry_minmax(int64_t E, int ndim, const double* __restrict__ xyz,
                                                               const double* __restrict__ geom,
                                                               double* __restrict__ part, int* bad) {
  __shared__ double smin[3][kPrepThreads], smax[3][kPrepThreads];
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  bool nf = false;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < ndim; ++k) {
      const double c = xyz[e * ndim + k];
      nf |= !isfinite(c);
      lo[k] = fmin(lo[k], c);
      hi[k] = fmax(hi[k], c);
    }
    if (geom) nf |= !(isfinite(geom[3 * e]) && isfinite(geom[3 * e + 1]) && isfinite(geom[3 * e + 2]));
  }
  if (nf) *bad = 1;
  for (int k = 0; k < 3; ++k) {
    smin[k][threadIdx.x] = lo[k];
    smax[k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int w = kPrepThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 3; ++k) {
        smin[k][threadIdx.x] = fmin(smin[k][threadIdx.x], smin[k][threadIdx.x + w]);
        smax[k][threadIdx.x] = fmax(smax[k][threadIdx.x], smax[k][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) {
      part[6 * blockIdx.x + k] = smin[k][0];
      part[6 * blockIdx.x + 3 + k] = smax[k][0];
    }
}

// FP64 (x, y, z, 0) of every entry and the FP32 split of s = (x - cmin) + B
// (hi = fl32(s), lo = fl32(s - hi)); normals as FP64 and as an FP32 pair.
__global__ void k_entry_pack(int64_t E, int ndim, const double* __restrict__ xyz, const double* __restrict__ geom,
                             double cx, double cy, double cz, double B, double4_32a* __restrict__ xyz64,
                             float4* __restrict__ hi, float4* __restrict__ lo, double4_32a* __restrict__ g64,
                             float4* __restrict__ g32, float4* __restrict__ g32lo) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const double cmin[3] = {cx, cy, cz};
  double c[3] = {0, 0, 0};
  float h[3] = {0, 0, 0}, l[3] = {0, 0, 0};
  for (int k = 0; k < ndim; ++k) {
    c[k] = xyz[e * ndim + k];
    const double sk = __dadd_rn(__dsub_rn(c[k], cmin[k]), B);
    h[k] = __double2float_rn(sk);
    l[k] = __double2float_rn(__dsub_rn(sk, (double)h[k]));
  }
  xyz64[e] = make_double4_32a(c[0], c[1], c[2], 0.0);
  hi[e] = make_float4(h[0], h[1], h[2], 0.f);
  lo[e] = make_float4(l[0], l[1], l[2], 0.f);
  if (geom) {
    const double gx = geom[3 * e], gy = geom[3 * e + 1], gz = geom[3 * e + 2];
    g64[e] = make_double4_32a(gx, gy, gz, 0.0);
    const float fx = __double2float_rn(gx), fy = __double2float_rn(gy), fz = __double2float_rn(gz);
    g32[e] = make_float4(fx, fy, fz, 0.f);
    g32lo[e] = make_float4(__double2float_rn(__dsub_rn(gx, (double)fx)), __double2float_rn(__dsub_rn(gy, (double)fy)),
                           __double2float_rn(__dsub_rn(gz, (double)fz)), 0.f);
  }
}

__device__ __forceinline__ int mirror_kind(int k) {
  return k == SKF_KIND_COARSE_UP ? SKF_KIND_COARSE_DOWN : (k == SKF_KIND_COARSE_DOWN ? SKF_KIND_COARSE_UP : k);
}

// *bad = 1 when a box lists a source twice, or lists (B, kind), B != A,
// without B listing (A, mirror kind).  One thread per list entry.
__global__ void k_sym_check(int nb, int64_t L, const int64_t* __restrict__ off, const int32_t* __restrict__ src,
                            const int8_t* __restrict__ kind, int* bad) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  int lo = 0, hi = nb;  // A = the box whose list holds entry l
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= l)
      lo = mid;
    else
      hi = mid;
  }
  const int A = lo, B = src[l];
  for (int64_t k = off[A]; k < l; ++k)
    if (src[k] == B) {
      *bad = 1;
      return;
    }
  if (B == A) return;
  const int want = mirror_kind(kind[l]);
  for (int64_t k = off[B]; k < off[B + 1]; ++k)
    if (src[k] == A) {
      if (kind[k] != want) *bad = 1;
      return;
    }
  *bad = 1;
}

}  // namespace skf

using namespace skf;

#define SKF_TRY(expr)              \
  do {                             \
    int _s = (expr);               \
    if (_s != SKF_OK) {            \
      free_plan(p);                \
      return _s;                   \
    }                              \
  } while (0)

extern "C" {

int skf_version(void) { return 1; }

const char* skf_status_string(int32_t s) {
  switch (s) {
    case SKF_OK: return "ok";
    case SKF_ERR_ARG: return "invalid argument";
    case SKF_ERR_OOM: return "device out of memory";
    case SKF_ERR_CUDA: return g_last_where[0] ? g_last_where : cudaGetErrorString(g_last_cuda);
    case SKF_ERR_UNSUPPORTED: return "unsupported operator or precision";
    case SKF_ERR_ID: return "interpolative decomposition failed (non-finite proxy matrix)";
    case SKF_ERR_SCRATCH: return "a box's proxy matrix exceeds the fixed no-allocation scratch (SKF_NOALLOC_SCRATCH_BYTES)";
    default: return "unknown status";
  }
}

int skf_plan_create(const skf_plan_desc* d, skf_plan** out) {
  if (!d || !out) return SKF_ERR_ARG;
  *out = nullptr;
  if (d->op < 0 || d->op >= SKF_NUM_OPS) return SKF_ERR_ARG;
  if (d->ndim != op_dim(d->op)) return SKF_ERR_ARG;
  if (d->nboxes <= 0 || d->nlevels <= 0 || d->root_level < 0 || d->root_level >= d->nlevels) return SKF_ERR_ARG;
  if (!d->box_level || !d->box_off || !d->box_rank || !d->entry_xyz || !d->entry_pslot || !d->perm_entry ||
      !d->perm_point || !d->t_off || !d->list_off || !d->list_src || !d->list_kind)
    return SKF_ERR_ARG;
  if (op_needs_geom(d->op) && !d->entry_geom) return SKF_ERR_ARG;
  const int nb = d->nboxes;
  const int64_t E = d->box_off[nb];
  if (E <= 0 || d->box_off[0] != 0) return SKF_ERR_ARG;
  if (d->nperm <= 0 || d->npoints <= 0) return SKF_ERR_ARG;
  const int64_t L = d->list_off[nb];
  if (d->list_off[0] != 0 || L < 0) return SKF_ERR_ARG;
  const bool cplx = op_is_complex(d->op);
  const int W = cplx ? 2 : 1;
  {
    // the description's index arrays, checked on the host threads
    std::atomic<bool> bad{false};
    parallel_ranges(nb, [&](int64_t lo, int64_t hi) {
      for (int64_t b = lo; b < hi && !bad; ++b) {
        const int64_t bs = d->box_off[b + 1] - d->box_off[b];
        const int64_t r = d->box_rank[b];
        if (bs < 0 || r < 0 || r > bs || d->box_level[b] < 0 || d->box_level[b] >= d->nlevels ||
            d->list_off[b + 1] < d->list_off[b] ||
            (r > 0 && d->box_level[b] > d->root_level && (d->t_off[b] < 0 || d->t_off[b] + r * (bs - r) > d->t_len)))
          bad = true;
      }
    });
    parallel_ranges(d->nperm, [&](int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi && !bad; ++i)
        if (d->perm_entry[i] < 0 || d->perm_entry[i] >= E || d->perm_point[i] < 0 || d->perm_point[i] >= d->npoints)
          bad = true;
    });
    parallel_ranges(E, [&](int64_t lo, int64_t hi) {
      for (int64_t e = lo; e < hi && !bad; ++e)
        if (d->entry_pslot[e] < -1 || d->entry_pslot[e] >= E) bad = true;
    });
    parallel_ranges(L, [&](int64_t lo, int64_t hi) {
      for (int64_t l = lo; l < hi && !bad; ++l)
        if (d->list_src[l] < 0 || d->list_src[l] >= nb || d->list_kind[l] < 0 || d->list_kind[l] > 3) bad = true;
    });
    if (bad) return SKF_ERR_ARG;
  }

  skf_plan* p = new skf_plan();
  p->op = d->op;
  p->ndim = d->ndim;
  p->nboxes = nb;
  p->nlevels = d->nlevels;
  p->root_level = d->root_level;
  p->cplx = cplx;
  p->kappa = d->kappa;
  p->E = E;
  p->N = d->npoints;
  p->nperm = d->nperm;
  p->t_len = d->t_len;
  p->nlist = L;
  for (int b = 0; b < nb; ++b) p->max_bs = std::max<int>(p->max_bs, (int)(d->box_off[b + 1] - d->box_off[b]));

  if (!d->entries_on_device) {
    // host entries are checked here, before any device work
    for (int64_t e = 0; e < E * d->ndim; ++e)
      if (!std::isfinite(d->entry_xyz[e])) {
        free_plan(p);
        return SKF_ERR_ARG;
      }
    if (d->entry_geom)
      for (int64_t e = 0; e < E * 3; ++e)
        if (!std::isfinite(d->entry_geom[e])) {
          free_plan(p);
          return SKF_ERR_ARG;
        }
  }
  // entry coordinates: FP64 (x,y,z,0) and the FP32 hi/lo split, prepared on
  // the device.  The split is taken of the coordinates translated into one
  // binade [B, 2B), B a power of two above the extent of the entries: every
  // hi then lies on the same FP32 grid (spacing B 2^-23), so hi_i - hi_j is
  // exact for every pair and d = (hi_i - hi_j) + (lo_i - lo_j) carries d to
  // ~B 2^-48 absolute.  The kernels only use differences, so the
  // translation changes nothing else.  Normals: FP64 and an FP32 pair (hi =
  // fl32(n), lo = fl32(n - hi)); the double-layer kernels form (x - y).n
  // from the pair (see dot_dn).  A non-finite coordinate or normal on the
  // device is rejected (SKF_ERR_ARG) before anything else is uploaded.
  {
    const int D = d->ndim;
    const double* xin = d->entry_xyz;
    const double* gin = d->entry_geom;
    double* scratch = nullptr;  // raw host entries staged on the device
    if (!d->entries_on_device) {
      const size_t nx = (size_t)E * D, ng = d->entry_geom ? (size_t)E * 3 : 0;
      cudaError_t e = cudaMalloc(&scratch, sizeof(double) * (nx + ng));
      if (e == cudaSuccess) e = cudaMemcpy(scratch, d->entry_xyz, sizeof(double) * nx, cudaMemcpyHostToDevice);
      if (e == cudaSuccess && ng) e = cudaMemcpy(scratch + nx, d->entry_geom, sizeof(double) * ng, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        cudaFree(scratch);
        set_last_cuda_error(e);
        free_plan(p);
        return e == cudaErrorMemoryAllocation ? SKF_ERR_OOM : SKF_ERR_CUDA;
      }
      xin = scratch;
      gin = ng ? scratch + nx : nullptr;
    }
    double* part = nullptr;
    int* dbad = nullptr;
    std::vector<double> hpart(6 * kPrepBlocks);
    int hbad = 0;
    cudaError_t e = cudaMalloc(&part, sizeof(double) * 6 * kPrepBlocks);
    if (e == cudaSuccess) e = cudaMalloc(&dbad, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(dbad, 0, sizeof(int));
    if (e == cudaSuccess) {
      k_entry_minmax<<<kPrepBlocks, kPrepThreads>>>(E, D, xin, gin, part, dbad);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(hpart.data(), part, sizeof(double) * 6 * kPrepBlocks, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(part);
    cudaFree(dbad);
    if (e != cudaSuccess || hbad) {
      cudaFree(scratch);
      if (e != cudaSuccess) set_last_cuda_error(e);
      free_plan(p);
      return e != cudaSuccess ? SKF_ERR_CUDA : SKF_ERR_ARG;
    }
    double cmin[3] = {0, 0, 0}, cmax[3] = {0, 0, 0};
    for (int k = 0; k < D; ++k) {
      cmin[k] = hpart[k];
      cmax[k] = hpart[3 + k];
      for (int b = 1; b < kPrepBlocks; ++b) {
        cmin[k] = std::min(cmin[k], hpart[6 * b + k]);
        cmax[k] = std::max(cmax[k], hpart[6 * b + 3 + k]);
      }
    }
    double extent = 0.0;
    for (int k = 0; k < D; ++k) extent = std::max(extent, cmax[k] - cmin[k]);
    const double B = extent > 0.0 ? std::ldexp(1.0, std::ilogb(extent) + 1) : 1.0;
    int st = upload(p, &p->xyz64, (const double4_32a*)nullptr, E);
    if (st == SKF_OK) st = upload(p, &p->hi32, (const float4*)nullptr, E);
    if (st == SKF_OK) st = upload(p, &p->lo32, (const float4*)nullptr, E);
    if (st == SKF_OK && gin) st = upload(p, &p->geom64, (const double4_32a*)nullptr, E);
    if (st == SKF_OK && gin) st = upload(p, &p->geom32, (const float4*)nullptr, E);
    if (st == SKF_OK && gin) st = upload(p, &p->geom32lo, (const float4*)nullptr, E);
    if (st == SKF_OK) {
      k_entry_pack<<<(unsigned)((E + kPrepThreads - 1) / kPrepThreads), kPrepThreads>>>(
          E, D, xin, gin, cmin[0], cmin[1], cmin[2], B, p->xyz64, p->hi32, p->lo32, p->geom64, p->geom32,
          p->geom32lo);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
      if (e != cudaSuccess) {
        set_last_cuda_error(e);
        st = SKF_ERR_CUDA;
      }
    }
    cudaFree(scratch);
    SKF_TRY(st);
  }
  SKF_TRY(upload(p, &p->box_off, d->box_off, (size_t)nb + 1));
  SKF_TRY(upload(p, &p->box_rank, d->box_rank, (size_t)nb));
  SKF_TRY(upload(p, &p->pslot, d->entry_pslot, (size_t)E));
  SKF_TRY(upload(p, &p->perm_entry, d->perm_entry, (size_t)d->nperm));
  SKF_TRY(upload(p, &p->perm_point, d->perm_point, (size_t)d->nperm));
  SKF_TRY(upload(p, &p->t_off, d->t_off, (size_t)nb));
  const int64_t tl = std::max<int64_t>(d->t_len, 1);
  SKF_TRY(upload(p, &p->t64, (const double*)nullptr, (size_t)tl * W));
  if (d->t_len > 0) {
    cudaError_t e = cudaMemcpy(p->t64, d->t_data, sizeof(double) * d->t_len * W,
                               d->t_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      free_plan(p);
      return SKF_ERR_CUDA;
    }
  }
  // FP32 pair copy of T (hi = fl32(T), lo = fl32(T - hi)), split on the device
  SKF_TRY(upload(p, &p->t32, (const float*)nullptr, (size_t)tl * W));
  SKF_TRY(upload(p, &p->t32lo, (const float*)nullptr, (size_t)tl * W));
  {
    const int st = split_f64(p->t64, p->t32, p->t32lo, (int64_t)tl * W, nullptr);
    if (st != SKF_OK) {
      free_plan(p);
      return st;
    }
  }
  SKF_TRY(upload(p, &p->list_off, d->list_off, (size_t)nb + 1));
  SKF_TRY(upload(p, &p->list_src, d->list_src, (size_t)std::max<int64_t>(L, 1)));
  SKF_TRY(upload(p, &p->list_kind, d->list_kind, (size_t)std::max<int64_t>(L, 1)));

  // level box lists for the upward/downward passes
  p->levels.assign(d->nlevels, LevelBoxes());
  {
    std::vector<std::vector<int32_t>> lb(d->nlevels);
    for (int b = 0; b < nb; ++b) {
      const int lev = d->box_level[b];
      const int r = d->box_rank[b];
      const int bs = (int)(d->box_off[b + 1] - d->box_off[b]);
      if (lev > d->root_level && r > 0 && bs > 0) {
        lb[lev].push_back(b);
        p->levels[lev].max_red = std::max(p->levels[lev].max_red, bs - r);
        p->levels[lev].max_rank = std::max(p->levels[lev].max_rank, r);
      }
    }
    for (int lev = 0; lev < d->nlevels; ++lev) {
      p->levels[lev].n = (int)lb[lev].size();
      if (!lb[lev].empty()) SKF_TRY(upload(p, &p->levels[lev].dev, lb[lev].data(), lb[lev].size()));
    }
  }

  // translation work items: (target box, row tile), most expensive first
  {
    std::vector<int64_t> src_sum(nb, 0);
    parallel_ranges(nb, [&](int64_t lo, int64_t hi) {
      for (int64_t b = lo; b < hi; ++b) {
        int64_t s = 0;
        for (int64_t l = d->list_off[b]; l < d->list_off[b + 1]; ++l) {
          const int sb = d->list_src[l];
          s += d->box_off[sb + 1] - d->box_off[sb];
        }
        src_sum[b] = s;
      }
    }, 4096);
    int64_t pairs = 0;
    double r256 = 0.0, r64 = 0.0;
    for (int b = 0; b < nb; ++b) {
      const int64_t bs = d->box_off[b + 1] - d->box_off[b];
      pairs += src_sum[b] * bs;
      r256 += (double)((bs + 255) / 256 * 256) * (double)src_sum[b];
      r64 += (double)((bs + 63) / 64 * 64) * (double)src_sum[b];
    }
    p->pairs = pairs;
    p->rows_256_over_64 = r64 > 0.0 ? r256 / r64 : 1.0;
    // FP64 kernel tiles, 256-row mixed tiles, 64-row mixed tiles: one host
    // thread per list
    std::vector<int32_t> wb[3], wr[3];
    auto build_items = [&](int pass) {
      const int tile = pass == 0 ? kTransThreads * kRowsPerThreadF64 : (pass == 1 ? kT32Threads * kRowsPerThreadF32 : 64);
      std::vector<std::pair<int64_t, std::pair<int32_t, int32_t>>> items;
      for (int b = 0; b < nb; ++b) {
        const int bs = (int)(d->box_off[b + 1] - d->box_off[b]);
        if (bs == 0 || d->list_off[b + 1] == d->list_off[b]) continue;
        for (int r0 = 0; r0 < bs; r0 += tile) {
          const int64_t rows = std::min(tile, bs - r0);
          items.push_back({rows * src_sum[b], {b, r0}});
        }
      }
      std::stable_sort(items.begin(), items.end(),
                       [](const auto& a, const auto& b) { return a.first > b.first; });
      wb[pass].resize(items.size());
      wr[pass].resize(items.size());
      for (size_t i = 0; i < items.size(); ++i) {
        wb[pass][i] = items[i].second.first;
        wr[pass][i] = items[i].second.second;
      }
    };
    {
      std::thread t1(build_items, 1), t2(build_items, 2);
      build_items(0);
      t1.join();
      t2.join();
    }
    for (int pass = 0; pass < 3; ++pass) {
      WorkList& w = pass == 0 ? p->work64 : (pass == 1 ? p->work32 : p->work32s);
      w.n = (int)wb[pass].size();
      if (w.n > 0) {
        SKF_TRY(upload(p, &w.box, wb[pass].data(), wb[pass].size()));
        SKF_TRY(upload(p, &w.row, wr[pass].data(), wr[pass].size()));
      }
    }
  }

  // symmetric translations: every pair (A, B) with A != B is evaluated once,
  // by the box with the smaller id, when the lists pair each entry with its
  // mirror (colleague <-> colleague, coarse-up <-> coarse-down, root <-> root)
  if (d->op == SKF_LAPLACE_2D || d->op == SKF_LAPLACE_3D || d->op == SKF_HELMHOLTZ_3D) {
    // partial arrays per owned entry: u, uh (real); u re/im, uh re/im (complex)
    const int nparts = cplx ? 4 : 2;
    // no box lists a source twice, and every (A, B, kind) has its (B, A,
    // mirror kind) in B's list (checked on the device)
    bool ok = true;
    if (L > 0) {
      int* dbad = nullptr;
      int hbad = 0;
      cudaError_t e = cudaMalloc(&dbad, sizeof(int));
      if (e == cudaSuccess) e = cudaMemset(dbad, 0, sizeof(int));
      if (e == cudaSuccess) {
        k_sym_check<<<(unsigned)((L + 255) / 256), 256>>>(nb, L, p->list_off, p->list_src, p->list_kind, dbad);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaMemcpy(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost);
      cudaFree(dbad);
      if (e != cudaSuccess) {
        set_last_cuda_error(e);
        free_plan(p);
        return SKF_ERR_CUDA;
      }
      ok = hbad == 0;
    }
    if (ok) {
      const int tile = kT32Threads * kRowsPerThreadF32;
      // Two passes over the boxes on the host threads: counts (entries with
      // B >= A, incoming partial blocks, work items), prefix sums, then
      // every box fills its own ranges, in the order a single pass would.
      std::vector<int64_t> cnt(nb), nin(nb), stride_v(nb), srcsum_v(nb), ntl(nb);
      parallel_ranges(nb, [&](int64_t lo, int64_t hi) {
        for (int64_t A = lo; A < hi; ++A) {
          int64_t c = 0, cn = 0, stv = 0, ss = 0;
          for (int64_t l = d->list_off[A]; l < d->list_off[A + 1]; ++l) {
            const int B = d->list_src[l];
            if (B < A) continue;
            const int64_t bsB = d->box_off[B + 1] - d->box_off[B];
            ++c;
            if (B != A) {
              ++cn;
              stv += nparts * bsB;
            }
            ss += bsB;
          }
          const int64_t bsA = d->box_off[A + 1] - d->box_off[A];
          const int64_t nt = bsA > 0 ? (bsA + tile - 1) / tile : 0;
          cnt[A] = c;
          nin[A] = nt * cn;
          stride_v[A] = stv;
          srcsum_v[A] = ss;
          ntl[A] = nt;
        }
      }, 2048);
      std::vector<int64_t> soff(nb + 1, 0), pbase(nb, 0), pstride(nb, 0), inb(nb + 1, 0), itb(nb + 1, 0);
      int64_t total = 0, sym_pairs = 0;
      for (int A = 0; A < nb; ++A) {
        const int64_t bsA = d->box_off[A + 1] - d->box_off[A];
        soff[A + 1] = soff[A] + cnt[A];
        pbase[A] = total;
        pstride[A] = stride_v[A];
        total += ntl[A] * stride_v[A];
        sym_pairs += bsA * srcsum_v[A];
        inb[A + 1] = inb[A] + nin[A];
        itb[A + 1] = itb[A] + ((bsA > 0 && cnt[A] > 0) ? ntl[A] : 0);
      }
      std::vector<int32_t> ssrc((size_t)soff[nb]);
      std::vector<int8_t> skind((size_t)soff[nb]);
      std::vector<int64_t> poff((size_t)soff[nb]);
      // B-side partial blocks each box receives, as (box, block) in the
      // order the reduction adds them, grouped into CSR below
      std::vector<std::pair<int32_t, int64_t>> incoming((size_t)inb[nb]);
      std::vector<std::pair<int64_t, std::pair<int32_t, int32_t>>> items((size_t)itb[nb]);
      parallel_ranges(nb, [&](int64_t lo, int64_t hi) {
        for (int64_t A = lo; A < hi; ++A) {
          int64_t k = soff[A], stv = 0;
          for (int64_t l = d->list_off[A]; l < d->list_off[A + 1]; ++l) {
            const int B = d->list_src[l];
            if (B < A) continue;
            const int64_t bsB = d->box_off[B + 1] - d->box_off[B];
            ssrc[k] = B;
            skind[k] = d->list_kind[l];
            poff[k] = B == A ? 0 : stv;
            if (B != A) stv += nparts * bsB;
            ++k;
          }
          int64_t o = inb[A];
          for (int64_t t = 0; t < ntl[A]; ++t)
            for (int64_t k2 = soff[A]; k2 < soff[A + 1]; ++k2)
              if (ssrc[k2] != A) incoming[o++] = {ssrc[k2], pbase[A] + t * stride_v[A] + poff[k2]};
          const int64_t bsA = d->box_off[A + 1] - d->box_off[A];
          int64_t it = itb[A];
          if (bsA > 0 && cnt[A] > 0)
            for (int64_t r0 = 0; r0 < bsA; r0 += tile)
              items[it++] = {std::min<int64_t>(tile, bsA - r0) * srcsum_v[A], {(int32_t)A, (int32_t)r0}};
        }
      }, 2048);
      std::stable_sort(items.begin(), items.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
      std::vector<int32_t> wb(items.size()), wr(items.size());
      for (size_t i = 0; i < items.size(); ++i) {
        wb[i] = items[i].second.first;
        wr[i] = items[i].second.second;
      }
      // CSR by receiving box, keeping the order within each box (counting sort)
      auto to_csr = [nb](const std::vector<std::pair<int32_t, int64_t>>& in, std::vector<int64_t>& off,
                         std::vector<int64_t>& blk) {
        off.assign((size_t)nb + 1, 0);
        for (const auto& e : in) ++off[(size_t)e.first + 1];
        for (int B = 0; B < nb; ++B) off[B + 1] += off[B];
        blk.resize(in.size());
        std::vector<int64_t> fill(off.begin(), off.end() - 1);
        for (const auto& e : in) blk[fill[e.first]++] = e.second;
      };
      std::vector<int64_t> ioff, iblk;
      to_csr(incoming, ioff, iblk);
      SKF_TRY(upload(p, &p->sym_list_off, soff.data(), soff.size()));
      SKF_TRY(upload(p, &p->sym_list_src, ssrc.data(), std::max<size_t>(ssrc.size(), 1)));
      SKF_TRY(upload(p, &p->sym_list_kind, skind.data(), std::max<size_t>(skind.size(), 1)));
      SKF_TRY(upload(p, &p->sym_list_poff, poff.data(), std::max<size_t>(poff.size(), 1)));
      SKF_TRY(upload(p, &p->box_pbase, pbase.data(), pbase.size()));
      SKF_TRY(upload(p, &p->box_pstride, pstride.data(), pstride.size()));
      SKF_TRY(upload(p, &p->in_off, ioff.data(), ioff.size()));
      if (!iblk.empty()) SKF_TRY(upload(p, &p->in_blk, iblk.data(), iblk.size()));
      // Source-split items for the warp-per-tile symmetric kernel (real
      // operators): a box's owned tiles (32 sources, cut where the uh charges
      // end, as the kernel cuts them) are numbered across its list; boxes
      // whose items are far above an even share of the work get up to 8
      // contiguous parts, so the launch has enough items to fill the GPU.
      constexpr int kTileW = 32, kMaxParts = 8;
      std::vector<int32_t> ntil(nb, 0), npart(nb, 1);
      std::vector<int64_t> apart(nb, -1), wc(nb, 0);
      if (!cplx)
        parallel_ranges(nb, [&](int64_t lo, int64_t hi) {
          for (int64_t A = lo; A < hi; ++A) {
            int64_t t = 0;
            for (int64_t k = soff[A]; k < soff[A + 1]; ++k) {
              const int B = ssrc[k];
              const int kind = skind[k];
              const int64_t bsB = d->box_off[B + 1] - d->box_off[B];
              const int64_t nh = (kind == SKF_KIND_COLLEAGUE || kind == SKF_KIND_COARSE_DOWN)
                                     ? d->box_rank[B]
                                     : (kind == SKF_KIND_COARSE_UP ? bsB : 0);
              t += (nh + kTileW - 1) / kTileW + (bsB - nh + kTileW - 1) / kTileW;
            }
            ntil[A] = (int32_t)t;
            wc[A] = (d->box_off[A + 1] - d->box_off[A]) * t;
          }
        }, 2048);
      int64_t wcost_total = 0;
      for (int A = 0; A < nb; ++A) wcost_total += wc[A];
      // an even share for ~4 waves of 3 blocks per SM on 152 SMs
      const double share = (double)wcost_total / (152.0 * 3.0 * 4.0);
      // parts per box, their A-side partial regions and item counts
      int64_t aoff = total;
      std::vector<int64_t> wib(nb + 1, 0), inw(nb + 1, 0);
      for (int A = 0; A < nb; ++A) {
        wib[A + 1] = wib[A];
        inw[A + 1] = inw[A];
        const int64_t bsA = d->box_off[A + 1] - d->box_off[A];
        if (cplx || bsA == 0 || ntil[A] == 0) continue;
        const double c = (double)std::min<int64_t>(tile, bsA) * ntil[A];
        int P = (int)std::min<double>(kMaxParts, std::max(1.0, std::ceil(c / std::max(share, 1.0))));
        P = std::min<int>(P, ntil[A]);
        npart[A] = P;
        if (P > 1) {
          apart[A] = aoff;
          aoff += (int64_t)(P - 1) * 4 * bsA;
          inw[A + 1] += 2 * (int64_t)(P - 1);
        }
        wib[A + 1] += ((bsA + tile - 1) / tile) * P;
      }
      const size_t n_in = incoming.size();
      std::vector<std::pair<int32_t, int64_t>> incoming_w = std::move(incoming);
      incoming_w.resize(n_in + (size_t)inw[nb]);
      std::vector<std::pair<int64_t, std::array<int32_t, 3>>> witems((size_t)wib[nb]);
      if (!cplx)
        parallel_ranges(nb, [&](int64_t lo, int64_t hi) {
          for (int64_t A = lo; A < hi; ++A) {
            const int64_t bsA = d->box_off[A + 1] - d->box_off[A];
            if (bsA == 0 || ntil[A] == 0) continue;
            const int P = npart[A];
            size_t o = n_in + (size_t)inw[A];
            for (int q = 1; q < P; ++q) {
              // hi and lo halves of the part's row sums: two incoming blocks
              incoming_w[o++] = {(int32_t)A, apart[A] + (int64_t)(q - 1) * 4 * bsA};
              incoming_w[o++] = {(int32_t)A, apart[A] + (int64_t)(q - 1) * 4 * bsA + 2 * bsA};
            }
            int64_t w = wib[A];
            for (int64_t r0 = 0; r0 < bsA; r0 += tile)
              for (int q = 0; q < P; ++q)
                witems[w++] = {std::min<int64_t>(tile, bsA - r0) *
                                   ((int64_t)(q + 1) * ntil[A] / P - (int64_t)q * ntil[A] / P),
                               {(int32_t)A, (int32_t)r0, q}};
          }
        }, 2048);
      std::stable_sort(witems.begin(), witems.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
      std::vector<int32_t> wwb(witems.size()), wwr(witems.size()), wwq(witems.size());
      for (size_t i = 0; i < witems.size(); ++i) {
        wwb[i] = witems[i].second[0];
        wwr[i] = witems[i].second[1];
        wwq[i] = witems[i].second[2];
      }
      std::vector<int64_t> ioffw, iblkw;
      to_csr(incoming_w, ioffw, iblkw);
      total = aoff;
      SKF_TRY(upload(p, &p->box_ntiles, ntil.data(), ntil.size()));
      SKF_TRY(upload(p, &p->box_nparts, npart.data(), npart.size()));
      SKF_TRY(upload(p, &p->box_apart, apart.data(), apart.size()));
      SKF_TRY(upload(p, &p->in_off_w, ioffw.data(), ioffw.size()));
      if (!iblkw.empty()) SKF_TRY(upload(p, &p->in_blk_w, iblkw.data(), iblkw.size()));
      SKF_TRY(upload(p, &p->symw_queue, (const int*)nullptr, 1));
      {
        // reduction items: 256-entry chunks of the boxes that receive partials
        // (under either scheme's lists)
        std::vector<int32_t> rb, rc;
        for (int B = 0; B < nb; ++B) {
          const int64_t bsB = d->box_off[B + 1] - d->box_off[B];
          if (bsB == 0 || (ioff[B + 1] == ioff[B] && ioffw[B + 1] == ioffw[B])) continue;
          for (int64_t c = 0; c * 256 < bsB; ++c) {
            rb.push_back(B);
            rc.push_back((int32_t)c);
          }
        }
        p->red.n = (int)rb.size();
        if (p->red.n > 0) {
          SKF_TRY(upload(p, &p->red.box, rb.data(), rb.size()));
          SKF_TRY(upload(p, &p->red.row, rc.data(), rc.size()));
        }
      }
      p->worksymw.n = (int)witems.size();
      if (p->worksymw.n > 0) {
        SKF_TRY(upload(p, &p->worksymw.box, wwb.data(), wwb.size()));
        SKF_TRY(upload(p, &p->worksymw.row, wwr.data(), wwr.size()));
        SKF_TRY(upload(p, &p->symw_part, wwq.data(), wwq.size()));
      }
      SKF_TRY(upload(p, &p->pbuf, (const float*)nullptr, (size_t)std::max<int64_t>(total, 1)));
      {
        // partial slots a kernel never writes (uh partials of tiles without uh
        // charges, skipped by k_translate_symw) must read as zero
        const cudaError_t e = cudaMemset(p->pbuf, 0, sizeof(float) * (size_t)std::max<int64_t>(total, 1));
        if (e != cudaSuccess) {
          set_last_cuda_error(e);
          free_plan(p);
          return SKF_ERR_CUDA;
        }
      }
      // real operators default to the source-split kernel (shape 4)
      if (!cplx) p->sym_shape = 4;
      p->worksym.n = (int)items.size();
      if (p->worksym.n > 0) {
        SKF_TRY(upload(p, &p->worksym.box, wb.data(), wb.size()));
        SKF_TRY(upload(p, &p->worksym.row, wr.data(), wr.size()));
      }
      p->sym_pairs = sym_pairs;
      p->sym_ok = true;
    }
  }

  SKF_TRY(upload(p, &p->q, (const double*)nullptr, (size_t)E * W));
  SKF_TRY(upload(p, &p->qh, (const double*)nullptr, (size_t)E * W));
  SKF_TRY(upload(p, &p->u, (const double*)nullptr, (size_t)E * W));
  SKF_TRY(upload(p, &p->uh, (const double*)nullptr, (size_t)E * W));
  SKF_TRY(upload(p, &p->q32, (const float*)nullptr, (size_t)E * W));
  SKF_TRY(upload(p, &p->qhn32, (const float*)nullptr, (size_t)E * W));
  SKF_TRY(upload(p, &p->qd32, (const float*)nullptr, (size_t)E * W));
  {
    // entry -> rank of its box, needed by the FP32 charge conversion
    std::vector<int32_t> er(E);
    parallel_ranges(nb, [&](int64_t lo, int64_t hi) {
      for (int64_t b = lo; b < hi; ++b)
        for (int64_t e = d->box_off[b]; e < d->box_off[b + 1]; ++e)
          er[e] = (int32_t)(e - d->box_off[b]) < d->box_rank[b] ? 1 : 0;
    }, 1024);
    SKF_TRY(upload(p, &p->entry_skel, er.data(), (size_t)E));
  }
  cudaError_t e1 = cudaMemset(p->q, 0, sizeof(double) * E * W);
  cudaError_t e2 = cudaMemset(p->qh, 0, sizeof(double) * E * W);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    set_last_cuda_error(e1 != cudaSuccess ? e1 : e2);
    free_plan(p);
    return SKF_ERR_CUDA;
  }
  *out = p;
  return SKF_OK;
}

int skf_plan_destroy(skf_plan* p) {
  free_plan(p);
  return SKF_OK;
}

int skf_plan_query(const skf_plan* p, skf_plan_info* info) {
  if (!p || !info) return SKF_ERR_ARG;
  info->nentries = p->E;
  info->npairs_fused = p->pairs;
  info->t_scalars = p->t_len;
  info->device_bytes = p->device_bytes;
  info->nwork = p->work32.n;
  info->is_complex = p->cplx ? 1 : 0;
  const bool sym = p->sym_ok && p->sym_on && !p->scalar_mixed;
  info->npairs_evaluated_mixed = sym ? p->sym_pairs : p->pairs;
  int lv = 0;
  for (int l = p->root_level + 1; l < p->nlevels; ++l) lv += p->levels[l].n > 0 ? 1 : 0;
  info->launches_fp64 = 2 + 2 * lv + (p->work64.n > 0 ? 1 : 0);
  info->launches_mixed = 2 + 2 * lv + 1 + (sym ? (p->worksym.n > 0 ? 1 : 0) + 1 : (p->work32.n > 0 ? 1 : 0));
  info->rows_256_over_64 = p->rows_256_over_64;
  return SKF_OK;
}

int skf_plan_apply(skf_plan* p, const void* x, void* y, int32_t precision, void* stream) {
  if (!p || !x || !y) return SKF_ERR_ARG;
  if (precision < SKF_PREC_FP64 || precision > SKF_PREC_MIXED_T32) return SKF_ERR_ARG;
  return plan_apply_device(p, static_cast<const double*>(x), static_cast<double*>(y), precision,
                           static_cast<cudaStream_t>(stream));
}

int skf_plan_apply_host(skf_plan* p, const void* xh, void* yh, int32_t precision, void* stream) {
  if (!p || !xh || !yh) return SKF_ERR_ARG;
  if (precision < SKF_PREC_FP64 || precision > SKF_PREC_MIXED_T32) return SKF_ERR_ARG;
  const int W = p->cplx ? 2 : 1;
  const size_t bytes = sizeof(double) * (size_t)p->N * W;
  if (!p->xbuf) {
    if (upload(p, &p->xbuf, (const double*)nullptr, (size_t)p->N * W) != SKF_OK) return SKF_ERR_OOM;
    if (upload(p, &p->ybuf, (const double*)nullptr, (size_t)p->N * W) != SKF_OK) return SKF_ERR_OOM;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SKF_CUDA_TRY(cudaMemcpyAsync(p->xbuf, xh, bytes, cudaMemcpyHostToDevice, st));
  int s = plan_apply_device(p, p->xbuf, p->ybuf, precision, st);
  if (s != SKF_OK) return s;
  SKF_CUDA_TRY(cudaMemcpyAsync(yh, p->ybuf, bytes, cudaMemcpyDeviceToHost, st));
  SKF_CUDA_TRY(cudaStreamSynchronize(st));
  return SKF_OK;
}

int skf_plan_set_option(skf_plan* p, int32_t option, int64_t value) {
  if (!p) return SKF_ERR_ARG;
  switch (option) {
    case SKF_OPT_SCALAR_MIXED: p->scalar_mixed = value != 0; return SKF_OK;
    case SKF_OPT_SYMMETRIC: p->sym_on = value != 0; return SKF_OK;
    case SKF_OPT_SYM_SHAPE:
      if (value < 0 || value > 5) return SKF_ERR_ARG;
      p->sym_shape = (int)value;
      return SKF_OK;
    case SKF_OPT_PACKED_SHAPE:
      if (value < 0 || value > 3) return SKF_ERR_ARG;
      p->x2_config = (int)value;
      return SKF_OK;
    default: return SKF_ERR_ARG;
  }
}

int skf_plan_time_translations(skf_plan* p, int32_t precision, int32_t reps, void* stream, float* ms_out) {
  if (!p || !ms_out || reps <= 0) return SKF_ERR_ARG;
  return plan_time_translations(p, precision != SKF_PREC_FP64, reps, static_cast<cudaStream_t>(stream), ms_out);
}

int skf_kernel_apply(int32_t op, double kappa, int32_t npairs, int32_t mmax, int32_t nmax, const int32_t* m,
                     const int32_t* n, const double* xt, const double* xs, const double* gt, const double* gs,
                     const void* q, const int8_t* self_flag, void* out, int32_t precision, void* stream) {
  if (op < 0 || op >= SKF_NUM_OPS || npairs < 0 || mmax < 0 || nmax < 0) return SKF_ERR_ARG;
  if (npairs == 0 || mmax == 0) return SKF_OK;
  if (!m || !n || !xt || !xs || !q || !out) return SKF_ERR_ARG;
  if ((mmax + 127) / 128 > 65535) return SKF_ERR_ARG;  // row tiles run on gridDim.y
  if (op_needs_geom(op) && ((op == SKF_LAPLACE_DOUBLE_LAYER_3D || op == SKF_HELMHOLTZ_DOUBLE_LAYER_3D) ? !gs : !gt))
    return SKF_ERR_ARG;
  if (precision != SKF_PREC_FP64 && precision != SKF_PREC_MIXED) return SKF_ERR_ARG;
  return kernel_apply(op, kappa, npairs, mmax, nmax, m, n, xt, xs, gt, gs, static_cast<const double*>(q), self_flag,
                      static_cast<double*>(out), precision == SKF_PREC_MIXED, static_cast<cudaStream_t>(stream));
}

int skf_skel_boxes(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x, const double* geom,
                   const double* centers, double box_length, int32_t nproxy, double tol, int32_t* rank, int32_t* perm,
                   const int64_t* t_off_out, void* t_out, void* stream) {
  if (op < 0 || op >= SKF_NUM_OPS || nbox < 0 || nproxy <= 0 || !(box_length > 0) || !(tol > 0)) return SKF_ERR_ARG;
  if (nbox == 0) return SKF_OK;
  if (!off || !x || !centers || !rank || !perm || !t_off_out || !t_out) return SKF_ERR_ARG;
  if (op_needs_geom(op) && !geom) return SKF_ERR_ARG;
  return skel_boxes(op, kappa, nbox, off, x, geom, centers, box_length, nullptr, nproxy, tol, rank, perm, t_off_out,
                    t_out, static_cast<cudaStream_t>(stream));
}

int skf_skel_boxes_multi(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x,
                         const double* geom, const double* centers, const double* box_lengths, int32_t nproxy,
                         double tol, int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out,
                         void* stream) {
  if (op < 0 || op >= SKF_NUM_OPS || nbox < 0 || nproxy <= 0 || !(tol > 0)) return SKF_ERR_ARG;
  if (nbox == 0) return SKF_OK;
  if (!off || !x || !centers || !box_lengths || !rank || !perm || !t_off_out || !t_out) return SKF_ERR_ARG;
  if (op_needs_geom(op) && !geom) return SKF_ERR_ARG;
  return skel_boxes(op, kappa, nbox, off, x, geom, centers, 1.0, box_lengths, nproxy, tol, rank, perm, t_off_out,
                    t_out, static_cast<cudaStream_t>(stream));
}

int skf_copy_segments(int64_t nseg, const int64_t* src_off, const int64_t* dst_off, const int64_t* len,
                      const void* src, void* dst, int32_t elem_bytes, void* stream) {
  if (nseg < 0 || (elem_bytes != 8 && elem_bytes != 16)) return SKF_ERR_ARG;
  if (nseg == 0) return SKF_OK;
  if (!src_off || !dst_off || !len || !src || !dst) return SKF_ERR_ARG;
  return copy_segments(nseg, src_off, dst_off, len, src, dst, elem_bytes, static_cast<cudaStream_t>(stream));
}

int skf_trim_workspace(void) { return trim_workspace(); }

int skf_proxy_rows(int32_t op, int32_t nproxy, int32_t* rows_out) {
  if (op < 0 || op >= SKF_NUM_OPS || nproxy <= 0 || !rows_out) return SKF_ERR_ARG;
  *rows_out = proxy_rows(op, nproxy);
  return SKF_OK;
}

int skf_skel_boxes_randomized(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x,
                              const double* geom, const double* centers, double box_length, int32_t nproxy,
                              double tol, const int32_t* kpred, int32_t oversample, int32_t rho, uint64_t seed,
                              int32_t nchk, double sketch_tol, double resid_tol, double* resid, int8_t* status,
                              int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out, void* stream) {
  if (op < 0 || op >= SKF_NUM_OPS || nbox < 0 || nproxy <= 0 || !(box_length > 0) || !(tol > 0) || !(tol < 1))
    return SKF_ERR_ARG;
  if (oversample < 2 || rho < 1 || nchk < 0 || !(resid_tol >= 0) || !(sketch_tol > 0) || !(sketch_tol < 1))
    return SKF_ERR_ARG;
  if (nbox == 0) return SKF_OK;
  if (!off || !x || !centers || !rank || !perm || !t_off_out || !t_out || !kpred) return SKF_ERR_ARG;
  if (op_needs_geom(op) && !geom) return SKF_ERR_ARG;
  return skel_boxes_randomized(op, kappa, nbox, off, x, geom, centers, box_length, nproxy, tol, kpred, oversample, rho,
                               seed, nchk, sketch_tol, resid_tol, resid, status, rank, perm, t_off_out, t_out,
                               static_cast<cudaStream_t>(stream));
}

// ---- level bookkeeping of the build (host, no device work) --------------

int skf_level_candidates(int64_t nbl, const uint8_t* is_leaf, const int64_t* box_start, const int64_t* box_end,
                         const int64_t* children, int32_t nc, int64_t child_first_box, const int64_t* child_off,
                         const int64_t* child_ids, const int64_t* rank, const int64_t* perm, int64_t npoints,
                         int64_t* off_out, int64_t* ids_out, int64_t* cand_src_out, int64_t* total) {
  if (nbl < 0 || nc < 1 || nc > 8 || !is_leaf || !box_start || !box_end || !children || !rank || !perm || !off_out ||
      !total || (child_ids && !child_off))
    return SKF_ERR_ARG;
  // sizes: a leaf holds its points; a parent the skeletons of its children
  // (in child order), when the child level is skeletonized
  std::vector<int64_t> sz((size_t)nbl, 0);
  parallel_ranges(nbl, [&](int64_t lo, int64_t hi) {
    for (int64_t b = lo; b < hi; ++b) {
      if (is_leaf[b]) {
        sz[b] = box_end[b] - box_start[b];
      } else if (child_ids) {
        int64_t t = 0;
        for (int k = 0; k < nc; ++k) {
          const int64_t c = children[b * nc + k];
          if (c >= 0) t += rank[c];
        }
        sz[b] = t;
      }
    }
  }, 4096);
  off_out[0] = 0;
  for (int64_t b = 0; b < nbl; ++b) off_out[b + 1] = off_out[b] + sz[b];
  *total = off_out[nbl];
  if (!ids_out) return SKF_OK;  // sizes only
  if (!cand_src_out) return SKF_ERR_ARG;
  for (int64_t b = 0; b < nbl; ++b)
    if (is_leaf[b] && (box_start[b] < 0 || box_end[b] > npoints)) return SKF_ERR_ARG;
  parallel_ranges(nbl, [&](int64_t lo, int64_t hi) {
    for (int64_t b = lo; b < hi; ++b) {
      int64_t o = off_out[b];
      if (is_leaf[b]) {
        for (int64_t i = box_start[b]; i < box_end[b]; ++i, ++o) {
          ids_out[o] = perm[i];
          cand_src_out[o] = -1;
        }
      } else if (child_ids) {
        for (int k = 0; k < nc; ++k) {
          const int64_t c = children[b * nc + k];
          if (c < 0) continue;
          const int64_t c0 = child_off[c - child_first_box];
          for (int64_t t = 0; t < rank[c]; ++t, ++o) {
            ids_out[o] = child_ids[c0 + t];
            cand_src_out[o] = c0 + t;
          }
        }
      }
    }
  }, 1024);
  return SKF_OK;
}

int skf_level_reorder(int64_t nbl, const int64_t* off, const int32_t* perm, const int64_t* ids_in, int64_t* ids_out,
                      int64_t* final_pos) {
  if (nbl < 0 || !off || !perm || !ids_in || !ids_out || !final_pos) return SKF_ERR_ARG;
  std::atomic<bool> bad{false};
  parallel_ranges(nbl, [&](int64_t lo, int64_t hi) {
    for (int64_t b = lo; b < hi && !bad; ++b) {
      const int64_t o = off[b], n = off[b + 1] - off[b];
      for (int64_t j = 0; j < n; ++j) {
        const int64_t p = perm[o + j];
        if (p < 0 || p >= n) {
          bad = true;
          break;
        }
        ids_out[o + j] = ids_in[o + p];
        final_pos[o + p] = o + j;
      }
    }
  }, 1024);
  return bad ? SKF_ERR_ARG : SKF_OK;
}

int skf_parent_slots(int32_t nlev, const int64_t* const* cand_src, const int64_t* const* final_pos,
                     const int64_t* ncand, const int64_t* base_child, const int64_t* base_parent, int64_t nentries,
                     int64_t* pslot) {
  if (nlev < 0 || nentries < 0 || !pslot || (nlev > 0 && (!cand_src || !final_pos || !ncand || !base_child ||
                                                         !base_parent)))
    return SKF_ERR_ARG;
  parallel_ranges(nentries, [&](int64_t lo, int64_t hi) {
    for (int64_t e = lo; e < hi; ++e) pslot[e] = -1;
  });
  std::atomic<bool> bad{false};
  for (int l = 0; l < nlev; ++l) {
    const int64_t* cs = cand_src[l];
    const int64_t* fp = final_pos[l];
    if (!cs || ncand[l] <= 0) continue;
    parallel_ranges(ncand[l], [&](int64_t lo, int64_t hi) {
      for (int64_t t = lo; t < hi; ++t) {
        const int64_t c = cs[t];
        if (c < 0) continue;
        const int64_t dst = base_child[l] + c, val = base_parent[l] + (fp ? fp[t] : t);
        if (dst < 0 || dst >= nentries || val < 0 || val >= nentries) {
          bad = true;
          return;
        }
        pslot[dst] = val;
      }
    });
  }
  return bad ? SKF_ERR_ARG : SKF_OK;
}

int skf_gather_i64(int64_t n, const int64_t* idx, const int64_t* src, int64_t nsrc, int64_t* out) {
  if (n < 0 || (n > 0 && (!idx || !src || !out))) return SKF_ERR_ARG;
  std::atomic<bool> bad{false};
  parallel_ranges(n, [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      const int64_t j = idx[i];
      if (j < 0 || j >= nsrc) {
        bad = true;
        return;
      }
      out[i] = src[j];
    }
  });
  return bad ? SKF_ERR_ARG : SKF_OK;
}

}  // extern "C"
