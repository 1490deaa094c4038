// Visibility compaction that allocates nothing: gs3d_compact_visible_static.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// enqueue work. Examples are code running while a CUDA graph is being
// captured (allocation is not a capturable operation), hosts that hand all
// device memory to their own arena or allocator (a game engine, a GPU process
// managing memory on behalf of sandboxed clients), and real-time render loops
// that must not stall on the driver's allocator. They pass their own input
// and output buffers; the kernel's scratch (the decoupled look-back status
// words and the per-call control block) lives in the fixed device array
// below instead of memory allocated per pipeline.
//
// Cost of the array: kStaticScratchWords * 8 bytes (about 40 KB), held on
// every GPU that loads the library until the process exits.
//
// Rules for callers:
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (with that device current). Make that first call
//    before any stream capture begins; later calls only enqueue a memset, one
//    kernel and one 4-byte copy, all capturable.
//  * Every call on a device shares the one array, which keeps the previous
//    call's contents. Each call clears the control block it needs zeroed;
//    the look-back status words carry a per-call epoch instead. Calls that
//    overlap on the GPU (two streams, or two host threads without ordering)
//    race on the array and give wrong results: order them on one stream.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "../../include/gs3d.h"
#include "pass_common.cuh"

using namespace gs;

namespace {

constexpr size_t kControlWords = (sizeof(Control) + 7) / 8;
constexpr size_t kStatusWords = 4096;  // one per chunk of k_compact; the grid is capped to this
constexpr size_t kStaticScratchWords = kControlWords + kStatusWords;
static_assert(sizeof(Control) % 8 == 0, "control block must be a whole number of words");

// The scratch: control block first, then the status words.
static __device__ __align__(256) unsigned long long g_compact_scratch[kStaticScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned long long* g_scratch_ptr[kMaxDevices] = {};
uint32_t g_epoch[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

}  // namespace

extern "C" gs3d_status gs3d_compact_visible_static(const uint32_t* keys, uint32_t n, uint32_t* visible_offsets,
                                                   uint32_t* keys_out, uint32_t* ids_out, uint32_t* result,
                                                   void* stream) {
  if (n > GS3D_STATIC_COMPACT_MAX_ITEMS) return GS3D_ERROR_RANGE;
  if (!result || (n > 0 && (!keys || !visible_offsets || !keys_out || !ids_out)))
    return GS3D_ERROR_INVALID_ARGUMENT;
  if (((uintptr_t)keys & 15u) != 0) return GS3D_ERROR_INVALID_ARGUMENT;  // read as uint4
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return GS3D_ERROR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* scratch = nullptr;
  uint32_t epoch = 0;
  int sms = 1;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[device]) {
      // One-time set-up on this device (the current device).
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_compact_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return GS3D_ERROR_CUDA;
      }
      g_scratch_ptr[device] = (unsigned long long*)p;
      if (cudaDeviceGetAttribute(&g_sms[device], cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        g_scratch_ptr[device] = nullptr;
        return GS3D_ERROR_CUDA;
      }
    }
    scratch = g_scratch_ptr[device];
    sms = g_sms[device];
    uint32_t e = (g_epoch[device] + 1u) & ((1u << 30) - 1u);
    if (e == 0) {
      // Epoch wrapped: clear the status words so no stale word can match.
      if (cudaMemsetAsync(scratch + kControlWords, 0, kStatusWords * 8, st) != cudaSuccess) return GS3D_ERROR_CUDA;
      e = 1;
    }
    g_epoch[device] = e;
    epoch = e;
  }
  Control* ctl = reinterpret_cast<Control*>(scratch);
  unsigned long long* status = scratch + kControlWords;
  if (cudaMemsetAsync(ctl, 0, sizeof(Control), st) != cudaSuccess) return GS3D_ERROR_CUDA;
  const uint32_t chunks = std::min<uint32_t>(scan_chunks(n, sms), (uint32_t)kStatusWords);
  launch_compact(keys, n, visible_offsets, keys_out, ids_out, ctl, status, Epoch{nullptr, epoch}, chunks, st);
  if (cudaMemcpyAsync(result, &ctl->visible_state[0], sizeof(uint32_t), cudaMemcpyDeviceToDevice, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(result + 1, &ctl->error, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return GS3D_ERROR_CUDA;
  if (cudaGetLastError() != cudaSuccess) return GS3D_ERROR_CUDA;
  return GS3D_OK;
}
