// Visibility compaction that allocates nothing: gs3d_compact_visible_static.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// enqueue work. A host that hands all device memory to its own arena or
// allocator (a game engine, a GPU process that manages memory on behalf of
// sandboxed clients) must not see allocations it did not make, and a
// real-time render loop must not stall on the driver's allocator, which may
// synchronise the device. Such callers pass their own input and output
// buffers; the kernel's scratch (the decoupled look-back status words, the
// per-call control block and the look-back epoch counter) lives in the fixed
// device array below instead of memory allocated per pipeline.
//
// Cost of the array: kStaticScratchWords * 8 bytes (about 41 KB), held on
// every GPU that loads the library until the process exits.
//
// Rules for callers:
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (with that device current) and reads the device's
//    SM count; later calls skip that set-up. Each call enqueues, on the
//    caller's stream: a one-block kernel that advances the epoch counter, a
//    memset of the control block, the compaction kernel and two 4-byte
//    device-to-device copies (count and error word into `result`).
//  * Every call on a device shares the one array, which keeps the previous
//    call's contents. Each call clears the control block it needs zeroed;
//    the look-back status words instead carry an epoch that the device
//    advances before every call, so a previous call's words never count as
//    published (when the 30-bit epoch wraps, the same kernel clears the
//    words). Calls that overlap on the GPU (two streams, or two host threads
//    without ordering) race on the array and give wrong results: order them
//    on one stream.
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
constexpr size_t kEpochWords = 1;      // the look-back epoch counter (low 32 bits of the word)
constexpr size_t kStaticScratchWords = kControlWords + kStatusWords + kEpochWords;
static_assert(sizeof(Control) % 8 == 0, "control block must be a whole number of words");

// The scratch: control block, status words, epoch counter.
static __device__ __align__(256) unsigned long long g_compact_scratch[kStaticScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned long long* g_scratch_ptr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

// Advances the epoch counter by one. Status words hold 30-bit epochs; when
// the counter wraps, every status word is cleared first so that no word left
// by an earlier call can carry the new epoch.
__global__ void __launch_bounds__(256) k_static_epoch_begin(unsigned long long* status, uint32_t* epoch) {
  const uint32_t next = (*epoch + 1u) & ((1u << 30) - 1u);
  __syncthreads();  // every thread has read the counter before it changes
  if (next == 0u) {
    for (uint32_t i = threadIdx.x; i < kStatusWords; i += blockDim.x) status[i] = 0ull;
  }
  if (threadIdx.x == 0) *epoch = next == 0u ? 1u : next;
}

}  // namespace

extern "C" gs3d_status gs3d_compact_visible_static(const uint32_t* keys, uint32_t n, uint32_t* visible_offsets,
                                                   uint32_t* keys_out, uint32_t* ids_out, uint32_t* result,
                                                   void* stream) {
  if (n > GS3D_STATIC_COMPACT_MAX_ITEMS) return GS3D_ERROR_RANGE;
  if (!result || (n > 0 && (!keys || !visible_offsets || !keys_out || !ids_out)))
    return GS3D_ERROR_INVALID_ARGUMENT;
  if (((uintptr_t)keys & 3u) != 0) return GS3D_ERROR_INVALID_ARGUMENT;  // read as 4-byte words
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return GS3D_ERROR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* scratch = nullptr;
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
      if (cudaDeviceGetAttribute(&g_sms[device], cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return GS3D_ERROR_CUDA;
      }
      g_scratch_ptr[device] = (unsigned long long*)p;
    }
    scratch = g_scratch_ptr[device];
    sms = g_sms[device];
  }
  Control* ctl = reinterpret_cast<Control*>(scratch);
  unsigned long long* status = scratch + kControlWords;
  uint32_t* epoch = reinterpret_cast<uint32_t*>(scratch + kControlWords + kStatusWords);
  k_static_epoch_begin<<<1, 256, 0, st>>>(status, epoch);
  if (cudaMemsetAsync(ctl, 0, sizeof(Control), st) != cudaSuccess) return GS3D_ERROR_CUDA;
  const uint32_t chunks = std::min<uint32_t>(scan_chunks(n, sms), (uint32_t)kStatusWords);
  launch_compact(keys, n, visible_offsets, keys_out, ids_out, ctl, status, Epoch{epoch, 0u, 0u}, chunks, st);
  if (cudaMemcpyAsync(result, &ctl->visible_state[0], sizeof(uint32_t), cudaMemcpyDeviceToDevice, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(result + 1, &ctl->error, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return GS3D_ERROR_CUDA;
  if (cudaGetLastError() != cudaSuccess) return GS3D_ERROR_CUDA;
  return GS3D_OK;
}
