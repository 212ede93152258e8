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
// Device memory of the given device (or managed memory), which that device's
// kernels may read and write directly.
bool device_ptr_on(const void* p, int device);
// Device ingest of .xyz text (owm_ingest.cu): the header of host text, and
// the parse of device text (16-byte aligned, 16 readable bytes of slack) into
// a cloud's two point buffers (records, x, y array) of *n_out points.
int xyz_header(const char* text, int64_t nbytes, int64_t* data_off, int64_t* declared, owm_bbox* hb);
int parse_device_text(owm_ctx* c, const char* dtext, int64_t nbytes, int64_t data_off, int64_t declared,
                      DeviceBuffer* out_mem, DeviceBuffer* out_xy, int64_t* n_out, int64_t* launches);
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
  // owm_run_host_submit / _wait: two runs in flight, each with its own input
  // buffer and pinned result staging; the host->device copy of one runs on
  // copy_stream while the other computes on `stream`.
  struct AsyncSlot {
    int64_t ticket = 0;  // 0 = free
    owm::DeviceBuffer input;
    cudaEvent_t ready = nullptr, done = nullptr;
    int64_t* h_seeds = nullptr;  // pinned [h_cap]
    int64_t h_cap = 0;
    uint32_t* h_words = nullptr;  // pinned [8]: status, counts
    int64_t* seeds = nullptr;     // caller's output
    int64_t cap = 0, room = 0;
    owm_params p{};
    int rc = 0;
  };
  cudaStream_t copy_stream = nullptr;
  AsyncSlot aslot[2];
  // owm_run prepares the stage-1 class tables on side_stream while the tree's
  // keys are sorted on `stream` (fork and join by the two events).
  // Then stage 1's last kernels and stage 2 run there too, while the tree's
  // hierarchy is built on `stream` (stage12_side: the last owm_run did so).
  cudaStream_t side_stream = nullptr;
  cudaEvent_t side_fork = nullptr, side_join = nullptr;
  bool stage12_side = false;
  int64_t next_ticket = 1;
  // > 0: step limit of the bounded tree walks (owm_ctx_set_walk_limit)
  int32_t walk_limit = 0;
  // launch shapes (owm_ctx_set_tuning); always complete (no zero fields)
  owm_tuning tuning = {4, 4, 256, 0};
};

namespace owm {

int clear_status(owm_ctx* c);
// Reads the status word (syncs); OWM_EINVAL if the input had a non-finite value.
int check_input_status(owm_ctx* c);
// A cloud keeps its points twice: as 32-byte records (x, y, z, pad: one DRAM
// sector per point for the build's random gather) and as a compact x, y array
// (16 bytes a point, for the passes that stream x and y only).  A caller's
// device array or host input copied in is read as plain x, y, z.
constexpr int kCloudStride = 4;
constexpr int kCloudXyStride = 2;
// n plain points (device, 8-byte aligned) into records and the x, y array
// (both 32-byte aligned), and records back to plain points; queued on s.
int pad_points(const double* src, int64_t n, double* rec, double* xy, cudaStream_t s, int64_t* launches);
int unpad_points(const double* src, int64_t n, double* dst, cudaStream_t s, int64_t* launches);
// bbox of n points whose x, y lie at d_xy[stride * i] and the next double.
int device_bbox(owm_ctx* c, const double* d_xy, int stride, int64_t n, owm_bbox* out);
int run_stage1(owm_ctx* c, const TreeStore& t, const owm_params& p, Edge* ex, Edge* ey, uint32_t* d_win);
int run_pipeline(owm_ctx* c, const PointsView& pts, int64_t n, const owm_bbox& bb, const owm_run_cfg& cfg,
                 int64_t* seeds, int64_t cap, int64_t* n_seeds, owm_run_info* info);
// The device part of run_pipeline: enqueues the whole run on c->stream and
// leaves the status words in c->d_small and the assembled seeds (room slots)
// at *d_seeds; no host sync (except inside the min-radius build).
int run_pipeline_enqueue(owm_ctx* c, const PointsView& pts, int64_t n, const owm_bbox& bb, const owm_run_cfg& cfg,
                         owm_params* p, int64_t** d_seeds, int64_t* room);

}  // namespace owm
