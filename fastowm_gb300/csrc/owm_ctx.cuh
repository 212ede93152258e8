// Context object and the whole-path pipeline shared by API, batch and server.
#pragma once

#include <vector>

#include "owm_query.cuh"

namespace owm {

// Stream-ordered device allocation that only grows.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t cap = 0;
  int reserve(size_t bytes, cudaStream_t s);
  void release(cudaStream_t s);
};

// Slots of the context's small device word array (uint32 indices).
constexpr int kStatusSlot = 0;  // bit 0: non-finite input coordinate
constexpr int kCheckSlot = 1;
constexpr int kCountSlot = 2;
constexpr int kLlpSlot = 3;
constexpr int kS3Slot = 4;
constexpr int kBboxSlot = 8;  // 4 x int64 (8-byte aligned)

bool is_device_ptr(const void* p);
int64_t total_launches();
int tree_alloc(TreeStore* t, DeviceBuffer* mem, int64_t n, const owm_tree_cfg& cfg, cudaStream_t s);
int validate_tree_cfg(const owm_tree_cfg* cfg);

}  // namespace owm

namespace owm {
// Event pairs recorded around kernels while profiling is on.
struct Profiler {
  struct Rec {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  const char* pending = nullptr;
  cudaEvent_t pending_ev = nullptr;
  cudaEvent_t take();
  void clear();
};
// Sets the calling thread's active profiler for one API call.
struct ProfScope {
  Profiler* prev;
  explicit ProfScope(Profiler* p) : prev(tls_profiler()) { tls_profiler() = p; }
  ~ProfScope() { tls_profiler() = prev; }
};
}  // namespace owm

struct owm_ctx {
  owm::Profiler prof;
  bool profiling = false;
  owm::Profiler* active_prof() { return profiling ? &prof : nullptr; }
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  uint32_t* d_small = nullptr;  // [1024] device words (counts, status)
  uint32_t* h_small = nullptr;  // [1024] pinned host mirror
  owm::QueryJob* d_job = nullptr;
  owm::DeviceBuffer scratch, tree_mem, input, outbuf;
  owm::TreeStore tree;  // tree of the last owm_run
  cudaEvent_t ev[8] = {};
};

namespace owm {

int clear_status(owm_ctx* c);
// Reads the status word (syncs); OWM_EINVAL if the input had a non-finite value.
int check_input_status(owm_ctx* c);
int device_bbox(owm_ctx* c, const double* d_xyz, int64_t n, owm_bbox* out);
int run_stage1(owm_ctx* c, const TreeStore& t, const owm_params& p, Edge* ex, Edge* ey, uint32_t* d_win);
int run_pipeline(owm_ctx* c, const double* d_xyz, int64_t n, const owm_bbox& bb, const owm_run_cfg& cfg,
                 int64_t* seeds, int64_t cap, int64_t* n_seeds, owm_run_info* info);

}  // namespace owm
