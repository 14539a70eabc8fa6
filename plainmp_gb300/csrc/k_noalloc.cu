// pmgpu_cst_is_valid_fast_noalloc: the FP32 + FP64-recheck validity check for callers that must
// not allocate device memory during the call.
//
// Who needs it: code that runs inside a real-time planning loop, on a device whose memory another
// allocator owns (a framework's caching allocator), or where an implicit device synchronisation
// from cudaMalloc/cudaFree would stall other streams.  Such callers set the constraint up once
// (any batch call builds its device tables) and afterwards call this entry point, which uses
// only the caller's buffers and the fixed scratch array below.
//
// The recheck queue, its counters and the per-configuration overflow flags live in one
// file-scope __device__ array of PM_NOALLOC_SCRATCH_BYTES (about 2 MB).  Every device that loads
// the library holds a copy until the process exits.  Host code must not pass the symbol itself
// to a kernel (it names a host-side stand-in); the device address comes from
// cudaGetSymbolAddress, taken once per device, with that device current, on the first call made
// on it.  That first call also uploads the warp search's block-offset table to the device (a
// synchronous cudaMemcpyToSymbol, unless an allocating fast call did it before) -- so make that
// first call before any stream capture and outside any section that must not block.  All calls
// share the array and it
// keeps the last call's contents: the counters and flags are cleared (cudaMemsetAsync) at the
// start of every call, and calls that overlap on the GPU (two streams, or two constraints at
// once) race on it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "pm_launch.h"
#include "pmgpu.h"

namespace pmg {  // host.cpp: device view of an already-prepared constraint, and the error text
bool cst_device_view(pmgpu_cst* c, const PmTablesHdr** T, PmTablesHdr* hdr, const double** state, int* cpb, int* nt);
void set_last_error(const char* msg);
}  // namespace pmg

namespace {

constexpr unsigned kQueueItems = 1u << 16;  // queued uncertain terms (16 B each)
constexpr int64_t kMaxConfigs = (int64_t)1 << 20;  // per call
constexpr size_t kCtlBytes = 256;
constexpr size_t kQueueBytes = (size_t)kQueueItems * sizeof(int4);
constexpr size_t kScratchBytes = kCtlBytes + kQueueBytes + (size_t)kMaxConfigs;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {nullptr};

}  // namespace

extern "C" int pmgpu_cst_is_valid_fast_noalloc(pmgpu_cst* c, const double* q, int64_t B, uint8_t* out, float* dist32, void* stream) {
  auto fail = [](int code, const char* msg) {
    pmg::set_last_error(msg);
    return code;
  };
  if (!c || (!q && B > 0) || (!out && B > 0)) return fail(PMGPU_ERR_INVALID, "pmgpu_cst_is_valid_fast_noalloc: NULL argument");
  if (B < 0 || B > kMaxConfigs)
    return fail(PMGPU_ERR_INVALID, "pmgpu_cst_is_valid_fast_noalloc: batch size must be in [0, 1048576]");
  const PmTablesHdr* T = nullptr;
  PmTablesHdr hdr;
  const double* state = nullptr;
  int cpb = 32, nt = 256;
  if (!pmg::cst_device_view(c, &T, &hdr, &state, &cpb, &nt))
    return fail(PMGPU_ERR_RUNTIME,
                "pmgpu_cst_is_valid_fast_noalloc: the constraint's tables are not on the current CUDA device, or the scene "
                "changed since they were built; make one allocating batch call first, with the model's device current");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(PMGPU_ERR_CUDA, "pmgpu_cst_is_valid_fast_noalloc: no current CUDA device");
  }
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {  // once per device, with that device current
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(PMGPU_ERR_CUDA, cudaGetErrorString(e));
      }
      const cudaError_t eo = pmg::upload_offsets();  // once per device too; later calls find it done
      if (eo != cudaSuccess) {
        cudaGetLastError();
        return fail(PMGPU_ERR_CUDA, cudaGetErrorString(eo));
      }
      g_addr[dev] = static_cast<unsigned char*>(p);
    }
    base = g_addr[dev];
  }
  if (B == 0) return PMGPU_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  unsigned int* count = reinterpret_cast<unsigned int*>(base);
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(base + 16);
  int4* items = reinterpret_cast<int4*>(base + kCtlBytes);
  uint8_t* overflow = base + kCtlBytes + kQueueBytes;
  cudaError_t e = cudaMemsetAsync(base, 0, kCtlBytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(overflow, 0, (size_t)B, s);
  if (e == cudaSuccess)
    e = pmg::launch_fast_valid(T, hdr, state, q, B, out, dist32, 0.1f, items, count, kQueueItems, overflow, stats, cpb, nt, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PMGPU_ERR_CUDA, cudaGetErrorString(e));
  }
  pmg::set_last_error("");
  return PMGPU_OK;
}
