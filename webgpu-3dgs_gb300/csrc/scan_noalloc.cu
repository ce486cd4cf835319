// scan_noalloc.cu - the exclusive prefix scan without any allocation.
//
// gs3d_prefix_scan_noalloc runs the same single-pass decoupled look-back scan
// as gs3d_prefix_scan (scan.cu), but needs no context: its scratch (the
// per-tile look-back status words, the tile ticket and an error word) is a
// file-scope device array that every GPU loading this library holds until
// the process exits.  It is for callers that cannot let a library call
// cudaMalloc: applications whose device memory is owned by their own pool or
// caching allocator, and frame loops that must not hit the implicit device
// synchronisation of cudaMalloc/cudaFree.
#include <cstdio>
#include <mutex>

#include "gs3d_internal.cuh"

namespace {

constexpr uint32_t kNoAllocMaxCounts = 1u << 26;  // 67,108,864 counts per call
constexpr uint32_t kScanTileCounts = 2048;        // counts per look-back tile (scan.cu)
constexpr uint32_t kNoAllocTiles = kNoAllocMaxCounts / kScanTileCounts + 1;

struct NoAllocScratch {
  unsigned long long status[kNoAllocTiles];  // epoch-tagged look-back words (256 KB)
  uint32_t ticket;                           // tile ticket: cleared by every call
  uint32_t error;                            // device error latch: cleared by every call
  uint32_t total;                            // the call's total (also written to offsets[n])
  uint32_t pad;
};

// Shared by every call on a device and left holding the last call's contents.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_mutex;
bool g_ran[gs3d::kMaxDevices] = {};        // a scan has been launched on the device
uint32_t g_epoch[gs3d::kMaxDevices] = {};  // look-back epoch, per device

// The scratch block's device address on the current device, queried on
// every call: the query allocates nothing, and a context that was reset may
// load the module at another address.
cudaError_t scratch_address(NoAllocScratch** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  *out = static_cast<NoAllocScratch*>(p);
  return e;
}
thread_local char g_error[256] = "no error";

int fail(int code, const char* msg) {
  snprintf(g_error, sizeof(g_error), "%s", msg);
  return code;
}

}  // namespace

namespace gs3d {
const char* noalloc_last_error() { return g_error; }
void set_context_free_error(const char* msg) { snprintf(g_error, sizeof(g_error), "%s", msg); }
}  // namespace gs3d

extern "C" int gs3d_prefix_scan_noalloc(const uint32_t* counts, uint32_t* offsets, uint32_t n,
                                        void* stream) {
  char msg[200];
  if (offsets == nullptr || (n > 0 && counts == nullptr))
    return fail(GS3D_ERR_INVALID_ARG, "gs3d_prefix_scan_noalloc: null counts or offsets");
  if (n > kNoAllocMaxCounts) {
    snprintf(msg, sizeof(msg),
             "gs3d_prefix_scan_noalloc: n = %u exceeds the maximum of %u counts per call", n,
             kNoAllocMaxCounts);
    return fail(GS3D_ERR_INVALID_ARG, msg);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= gs3d::kMaxDevices)
    return fail(GS3D_ERR_NO_DEVICE, "gs3d_prefix_scan_noalloc: no current CUDA device");
  // the host-side symbol is only a stand-in: the kernel needs the device address
  NoAllocScratch* scratch = nullptr;
  e = scratch_address(&scratch);
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "gs3d_prefix_scan_noalloc: cudaGetSymbolAddress failed: %s",
             cudaGetErrorString(e));
    cudaGetLastError();
    return fail(e == cudaErrorNoKernelImageForDevice ? GS3D_ERR_NO_DEVICE : GS3D_ERR_CUDA, msg);
  }
  uint32_t epoch = 0;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    g_epoch[dev] = (g_epoch[dev] % ((1u << 30) - 1)) + 1;  // 1 .. 2^30-1, never 0
    epoch = g_epoch[dev];
    g_ran[dev] = true;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the ticket and the error word must start at zero; the status words are
  // epoch-tagged, so earlier calls' entries read as "not ready"
  e = cudaMemsetAsync(&scratch->ticket, 0, 2 * sizeof(uint32_t), s);
  if (e == cudaSuccess)
    e = gs3d::launch_scan(counts, nullptr, offsets, n, scratch->status, &scratch->ticket, epoch,
                          &scratch->total, &scratch->error, s);
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "gs3d_prefix_scan_noalloc: launch failed: %s",
             cudaGetErrorString(e));
    cudaGetLastError();
    return fail(GS3D_ERR_CUDA, msg);
  }
  return GS3D_OK;
}

// The device errors of the last gs3d_prefix_scan_noalloc call on the current
// device: the error word is copied out behind the work already on `stream`
// (into pageable host memory, so the copy has landed when it returns).
extern "C" int gs3d_prefix_scan_noalloc_status(void* stream) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= gs3d::kMaxDevices)
    return fail(GS3D_ERR_NO_DEVICE, "gs3d_prefix_scan_noalloc_status: no current CUDA device");
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_ran[dev]) return GS3D_OK;  // no scan has run on this device
  }
  NoAllocScratch* scratch = nullptr;
  e = scratch_address(&scratch);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t word = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&word, &scratch->error, sizeof(word), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    char msg[200];
    snprintf(msg, sizeof(msg), "gs3d_prefix_scan_noalloc_status: reading the error word failed: %s",
             cudaGetErrorString(e));
    cudaGetLastError();
    return fail(GS3D_ERR_CUDA, msg);
  }
  if (word & gs3d::DEVERR_CAPACITY)
    return fail(GS3D_ERR_CAPACITY,
                "gs3d_prefix_scan_noalloc: the counts sum to 2^32 or more; offsets[n] was "
                "written as 0xffffffff and the offsets past the overflow are not valid");
  if (word & gs3d::DEVERR_TIMEOUT)
    return fail(GS3D_ERR_TIMEOUT,
                "gs3d_prefix_scan_noalloc: a bounded look-back wait gave up; the offsets are "
                "incomplete");
  return GS3D_OK;
}
