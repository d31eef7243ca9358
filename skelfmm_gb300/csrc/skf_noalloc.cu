// skf_noalloc.cu — one level of proxy interpolative decompositions without
// allocating device memory.
//
// Who needs this: callers that are not allowed to allocate GPU memory on the
// code path that builds the operator — an application that has handed the
// device's memory to its own pool allocator and forbids cudaMalloc behind its
// back, a plug-in that runs inside a host framework's fixed memory budget, or
// a latency-bound loop where an allocation and the synchronisation it can
// imply are not acceptable.  skf_skel_boxes_noalloc does the work of
// skf_skel_boxes, but its workspace (the proxy template, the per-box offsets
// and the proxy matrices of a batch of boxes) lives in one fixed, file-scope
// device array instead of stream-ordered allocations.  Inputs and outputs are
// still the caller's buffers.
//
// Contract:
// * The array holds SKF_NOALLOC_SCRATCH_BYTES (64 MiB) on every GPU that
//   loads the library, for the life of the process.
// * Boxes are processed in batches that fit; one box whose proxy matrix
//   (rows x box size, x2 for complex kernels, FP64) does not fit beside the
//   proxy template is rejected with SKF_ERR_SCRATCH before any kernel launch
//   or scratch write (the call first copies `off` to the host and
//   synchronises the stream).
// * The first call on a device looks up the array's device address with
//   cudaGetSymbolAddress while that device is current; make that first call
//   before starting any stream capture on the device.  The address is kept
//   for the life of the process: a cudaDeviceReset of the device invalidates
//   it.
// * Every box runs on the 256-thread ID kernel; skf_skel_boxes moves the
//   costliest boxes of 192+ points to thread-block clusters, whose pivot order
//   past the rank (decided at rounding level) can differ.
// * Every call shares the array and it keeps the last call's contents.
//   Nothing in it has to start at zero (each call writes everything it
//   reads), but calls that overlap on the GPU (other streams, other host
//   threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "skf_internal.cuh"

namespace skf {
int skel_boxes_scratch(int op, double kappa, int nbox, const int64_t* off, const double* x, const double* geom,
                       const double* centers, double box_length, int nproxy, double tol, int32_t* rank,
                       int32_t* perm, const int64_t* t_off_out, void* t_out, double* scratch, int64_t cap,
                       cudaStream_t st);
}  // namespace skf

namespace {

constexpr int64_t kScratchDoubles = SKF_NOALLOC_SCRATCH_BYTES / (int64_t)sizeof(double);
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
int scratch_address(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    skf::set_last_cuda_error(e);
    return SKF_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return SKF_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      skf::set_last_cuda_error(e);
      return SKF_ERR_CUDA;
    }
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return SKF_OK;
}

}  // namespace

extern "C" int skf_skel_boxes_noalloc(int32_t op, double kappa, int32_t nbox, const int64_t* off, const double* x,
                                      const double* geom, const double* centers, double box_length, int32_t nproxy,
                                      double tol, int32_t* rank, int32_t* perm, const int64_t* t_off_out,
                                      void* t_out, void* stream) {
  if (op < 0 || op >= SKF_NUM_OPS || nbox < 0 || nproxy <= 0 || !(box_length > 0) || !(tol > 0)) return SKF_ERR_ARG;
  if (nbox == 0) return SKF_OK;
  if (!off || !x || !centers || !rank || !perm || !t_off_out || !t_out) return SKF_ERR_ARG;
  if (op >= SKF_LAPLACE_DOUBLE_LAYER_3D && !geom) return SKF_ERR_ARG;
  double* scratch = nullptr;
  const int s = scratch_address(&scratch);
  if (s != SKF_OK) return s;
  return skf::skel_boxes_scratch(op, kappa, nbox, off, x, geom, centers, box_length, nproxy, tol, rank, perm,
                                 t_off_out, t_out, scratch, kScratchDoubles, static_cast<cudaStream_t>(stream));
}
