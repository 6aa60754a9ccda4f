// otfem_noalloc.cu -- an allocation-free form of the matrix-free operator
// y = A x, for callers that cannot allocate device memory at the point of
// the call: code running while a stream is being captured into a CUDA graph
// (cudaMalloc is not allowed there), real-time loops that must not allocate
// after start-up, or hosts whose memory pool is owned by another framework.
//
// otfem_apply_operator copies host arrays into temporary device buffers it
// allocates; this variant takes device arrays and keeps its scratch (the
// packed operand and the force accumulator) in the file-scope array below,
// which every GPU that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "otfem_internal.h"

namespace {

// 64 bytes per node (FP64 operand + accumulator; FP32 uses 48) for up to
// kNoAllocMaxNodes nodes: 16 MiB.
constexpr long long kNoAllocMaxNodes = 1 << 18;
constexpr size_t kNoAllocScratchBytes = size_t(kNoAllocMaxNodes) * 64;

static __device__ __align__(256) unsigned char g_apply_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

int noalloc_fail(int code, const std::string& msg) { return otfem::record_error(code, msg); }

}  // namespace

extern "C" {

// See include/otfem_gpu.h.
OTFEM_API int otfem_apply_operator_noalloc(otfem_handle h, int solver, double dt, double mass_damping,
                                           const double* x_device, double* y_device) {
  otfem::Context* c = otfem::context_of(h);
  if (!c) return noalloc_fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  // x_device == y_device == NULL: the per-device set-up alone (below), so a
  // caller can run it before capturing a stream without real buffers
  const bool setup_only = !x_device && !y_device;
  if (!setup_only && (!x_device || !y_device)) return noalloc_fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  if (c->N > kNoAllocMaxNodes)
    return noalloc_fail(OTFEM_ERR_INVALID_ARGUMENT,
                        "mesh has " + std::to_string(c->N) + " nodes; otfem_apply_operator_noalloc supports at most " +
                            std::to_string(kNoAllocMaxNodes));
  if (!c->initialized) return noalloc_fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  if (solver != OTFEM_SOLVER_MIXED && solver != OTFEM_SOLVER_FP64)
    return noalloc_fail(OTFEM_ERR_INVALID_ARGUMENT, "solver must be OTFEM_SOLVER_MIXED or OTFEM_SOLVER_FP64");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(OTFEM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev != c->device || dev < 0 || dev >= kMaxDevices)
    return noalloc_fail(OTFEM_ERR_INVALID_ARGUMENT, "call with the handle's device current");
  void* scratch = nullptr;
  {
    // set-up, once per device and with that device current: the address of
    // the scratch array on this device (in host code its name is only a
    // host-side stand-in, not a device address)
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_apply_scratch);
      if (e != cudaSuccess)
        return noalloc_fail(OTFEM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = ptr;
    }
    scratch = g_scratch_ptr[dev];
  }
  if (setup_only) return OTFEM_OK;
  // both arrays must be device (or managed) memory of the handle's device:
  // a host pointer or another device's pointer would fault inside the
  // kernels instead of returning an error (the query allocates nothing)
  const double* ptrs[2] = {x_device, y_device};
  for (const double* ptr : ptrs) {
    cudaPointerAttributes at;
    e = cudaPointerGetAttributes(&at, ptr);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return noalloc_fail(OTFEM_ERR_INVALID_ARGUMENT,
                          std::string("x_device/y_device: not a device pointer (") + cudaGetErrorString(e) + ")");
    }
    if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) || at.device != c->device)
      return noalloc_fail(OTFEM_ERR_INVALID_ARGUMENT,
                          "x_device and y_device must be device memory of the handle's device");
  }
  // the pack kernel clears the accumulator before the sweep
  e = otfem::launch_apply_operator_scratch(*c, solver, dt, mass_damping, x_device, y_device, scratch);
  if (e != cudaSuccess) return noalloc_fail(OTFEM_ERR_CUDA, std::string("apply: ") + cudaGetErrorString(e));
  c->launches += 3;
  return OTFEM_OK;
}

}  // extern "C"
