// Stage 2 for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at all: an
// application that hands every device byte to its own pool allocator at
// start-up, a plugin hosted by a program that forbids allocation on the
// streams it lends out, or a real-time loop where an allocation (and the
// device synchronisation it can cause) is not allowed.  owm_stage2_noalloc
// gives them the stage-2 sort/unique with no allocation: its working memory
// is the file-scope device array below, which every GPU that loads this
// library reserves once and keeps until the process exits.
//
// Rules of use (also in include/owm_gb300.h):
//   * at most kNoAllocMaxCells (1,048,576) window results per call; larger
//     inputs get OWM_ERANGE and nothing runs;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before any stream capture;
//   * every call shares the one array, which keeps the previous call's data:
//     calls whose GPU work overlaps (two streams, two threads) race and
//     corrupt each other's results -- serialise them;
//   * inputs and outputs are the caller's device memory.
#include <cuda_runtime.h>

#include <mutex>

#include "owm_query.cuh"

namespace owm {

namespace {

constexpr int64_t kNoAllocMaxCells = 1 << 20;
constexpr size_t kArr = (size_t)kNoAllocMaxCells * 4;  // one uint32 array
constexpr size_t kTempBytes = (size_t)3 << 19;         // sort + scan temp (1.5 MB)
// win/k0 | k1 | flags | pos | llp | temp | count word
constexpr size_t kTempOff = 5 * kArr;
constexpr size_t kCountOff = kTempOff + kTempBytes;
constexpr size_t kScratchBytes = kCountOff + 256;  // 21.5 MB

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
void* g_addr[kMaxDevices] = {};  // device address of g_noalloc_scratch, per device

// One-time per-device set-up: the host-side name of a __device__ array is not
// a device address, so look the address up with the device current.
int scratch_for_current_device(void** out) {
  int dev = 0;
  OWM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return OWM_ECUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    OWM_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return OWM_OK;
}

}  // namespace

}  // namespace owm

extern "C" int owm_stage2_noalloc(void* stream, const int64_t* d_win_min, int64_t ncells, double overlap,
                                  int64_t npoints, int64_t* d_llp, int64_t* n_llp) {
  using namespace owm;
  if (!d_win_min || !d_llp || !n_llp || ncells <= 0 || !(overlap >= 0.0 && overlap < 1.0) || npoints <= 0 ||
      npoints >= 0xFFFFFFFFLL)
    return OWM_EINVAL;
  if (ncells > kNoAllocMaxCells) return OWM_ERANGE;
  if (align256ul(radix_sort_temp_bytes(kNoAllocMaxCells)) + scan_temp_bytes(kNoAllocMaxCells) > kTempBytes)
    return OWM_ENOMEM;  // sizing guard of the static array
  void* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* b = static_cast<char*>(base);
  uint32_t* k0 = reinterpret_cast<uint32_t*>(b);
  uint32_t* k1 = reinterpret_cast<uint32_t*>(b + kArr);
  uint32_t* flags = reinterpret_cast<uint32_t*>(b + 2 * kArr);
  uint32_t* pos = reinterpret_cast<uint32_t*>(b + 3 * kArr);
  uint32_t* llp = reinterpret_cast<uint32_t*>(b + 4 * kArr);
  uint32_t* count = reinterpret_cast<uint32_t*>(b + kCountOff);
  int64_t launches = 0;
  // the count word must start at zero (the array keeps the last call's data)
  OWM_CUDA_TRY(cudaMemsetAsync(count, 0, 4, s));
  rc = i64_to_u32_ids(d_win_min, ncells, k0, s, &launches);
  if (!rc)
    rc = run_stage2_into(k0, k0, k1, flags, pos, ncells, npoints, overlap, llp, count, b + kTempOff, kTempBytes, s,
                         &launches);
  if (!rc) rc = u32_to_i64_ids(llp, count, ncells, d_llp, s, &launches);
  if (rc) return rc;
  uint32_t h = 0;
  OWM_CUDA_TRY(cudaMemcpyAsync(&h, count, 4, cudaMemcpyDeviceToHost, s));
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  *n_llp = (int64_t)h;
  return OWM_OK;
}
