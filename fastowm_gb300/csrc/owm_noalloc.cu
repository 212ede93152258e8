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
//   * window ids must lie in [0, npoints] (negative = no minimum); a larger id
//     makes the call return OWM_EINVAL, with d_llp undefined;
//   * the work runs on the device that owns `stream` (for the legacy default
//     stream: the current device); the call makes that device current for its
//     duration and restores the caller's device before it returns;
//   * the first call in each CUDA context of a device looks up the array's
//     device address with cudaGetSymbolAddress (with that device current);
//   * every call shares the one array, which keeps the previous call's data:
//     calls whose GPU work overlaps (two streams, two threads) race and
//     corrupt each other's results -- serialise them;
//   * inputs and outputs are the caller's device memory.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "owm_query.cuh"

namespace owm {

namespace {

constexpr int64_t kNoAllocMaxCells = 1 << 20;
constexpr size_t kArr = (size_t)kNoAllocMaxCells * 4;  // one uint32 array
constexpr size_t kTempBytes = (size_t)3 << 19;         // sort + scan temp (1.5 MB)
// win/k0 | k1 | flags | pos | llp | temp | count word, bad-id word
constexpr size_t kTempOff = 5 * kArr;
constexpr size_t kCountOff = kTempOff + kTempBytes;
constexpr size_t kScratchBytes = kCountOff + 256;  // 21.5 MB

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr uint32_t kNoneId = 0xFFFFFFFFu;

// Caller's int64 window ids -> the uint32 form of stage 2: negative -> none;
// an id above npoints (no point has it) sets *bad and is written as none.
__global__ void k_noalloc_ids(const int64_t* __restrict__ in, int64_t n, int64_t npoints, uint32_t* __restrict__ out,
                              uint32_t* __restrict__ bad) {
  bool over = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = in[i];
    over |= v > npoints;
    out[i] = (v < 0 || v > npoints) ? kNoneId : (uint32_t)v;
  }
  if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

// Address cache of g_noalloc_scratch, keyed by device and by the unique id of
// the CUDA context current on it (cuCtxGetId): a __device__ array's address
// belongs to one context, and a context destroyed by cudaDeviceReset is
// replaced by one with a new id.  Where the driver entry points cannot be
// had, the address is looked up on every call instead (it allocates nothing).
using CtxGetCurrentFn = CUresult(CUDAAPI*)(CUcontext*);
using CtxGetIdFn = CUresult(CUDAAPI*)(CUcontext, unsigned long long*);

std::mutex g_mu;
constexpr int kMaxDevices = 64;
void* g_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};
bool g_fns_tried = false;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

bool current_context_id(unsigned long long* id) {
  if (!g_fns_tried) {
    g_fns_tried = true;
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qb == cudaDriverEntryPointSuccess) {
      g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(a);
      g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(b);
    }
    cudaGetLastError();  // a failed query leaves no sticky error
  }
  if (!g_ctx_get_current || !g_ctx_get_id) return false;
  CUcontext c = nullptr;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c) return false;
  return g_ctx_get_id(c, id) == CUDA_SUCCESS;
}

// Device address of the array in the context current on `dev` (which is the
// current device when this runs).
int scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= kMaxDevices) return OWM_ECUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  // no context current on this thread yet (no runtime call made it so):
  // cudaGetSymbolAddress below binds the device's primary context, and the
  // address is cached from the next call on
  unsigned long long id = 0;
  const bool have_id = current_context_id(&id);
  if (have_id && g_addr[dev] && g_ctx_id[dev] == id) {
    *out = g_addr[dev];
    return OWM_OK;
  }
  void* p = nullptr;
  OWM_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  if (have_id) {
    g_addr[dev] = p;
    g_ctx_id[dev] = id;
  }
  *out = p;
  return OWM_OK;
}

// The device that owns `s`: the current device for the legacy and per-thread
// default streams.
int stream_device(cudaStream_t s, int* dev) {
  OWM_CUDA_TRY(cudaGetDevice(dev));
  if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) return OWM_OK;
  OWM_CUDA_TRY(cudaStreamGetDevice(s, dev));
  return OWM_OK;
}

// Makes `dev` current for one scope and restores the caller's device.
struct DeviceScope {
  int prev = -1;
  int set(int dev) {
    OWM_CUDA_TRY(cudaGetDevice(&prev));
    if (prev != dev) OWM_CUDA_TRY(cudaSetDevice(dev));
    return OWM_OK;
  }
  ~DeviceScope() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

int stage2_noalloc(cudaStream_t s, const int64_t* d_win_min, int64_t ncells, double overlap, int64_t npoints,
                   int64_t* d_llp, int64_t* n_llp) {
  int dev = 0;
  int rc = stream_device(s, &dev);
  if (rc) return rc;
  DeviceScope scope;
  rc = scope.set(dev);
  if (rc) return rc;
  void* base = nullptr;
  rc = scratch_address(dev, &base);
  if (rc) return rc;
  char* b = static_cast<char*>(base);
  uint32_t* k0 = reinterpret_cast<uint32_t*>(b);
  uint32_t* k1 = reinterpret_cast<uint32_t*>(b + kArr);
  uint32_t* flags = reinterpret_cast<uint32_t*>(b + 2 * kArr);
  uint32_t* pos = reinterpret_cast<uint32_t*>(b + 3 * kArr);
  uint32_t* llp = reinterpret_cast<uint32_t*>(b + 4 * kArr);
  uint32_t* words = reinterpret_cast<uint32_t*>(b + kCountOff);  // [0] count, [1] bad-id flag
  int64_t launches = 0;
  // both words must start at zero (the array keeps the last call's data)
  OWM_CUDA_TRY(cudaMemsetAsync(words, 0, 8, s));
  int64_t grid = (ncells + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  OWM_LAUNCH("k_noalloc_ids", s, k_noalloc_ids<<<(unsigned)grid, 256, 0, s>>>(d_win_min, ncells, npoints, k0,
                                                                               words + 1));
  count_launch(&launches);
  OWM_CUDA_TRY(cudaGetLastError());
  rc = run_stage2_into(k0, k0, k1, flags, pos, ncells, npoints, overlap, llp, words, b + kTempOff, kTempBytes, s,
                       &launches);
  if (!rc) rc = u32_to_i64_ids(llp, words, ncells, d_llp, s, &launches);
  if (rc) return rc;
  uint32_t h[2] = {0, 0};
  OWM_CUDA_TRY(cudaMemcpyAsync(h, words, 8, cudaMemcpyDeviceToHost, s));
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  if (h[1]) return OWM_EINVAL;  // an id above npoints: no such point
  *n_llp = (int64_t)h[0];
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
  return stage2_noalloc(static_cast<cudaStream_t>(stream), d_win_min, ncells, overlap, npoints, d_llp, n_llp);
}
