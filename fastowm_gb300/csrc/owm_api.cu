// C ABI: contexts, device clouds, trees, stages and the whole-path run.
//
// Reference entry points replaced (CPP-TBB-CPU/include/optim3_func.hpp:73-93,
// driven by CPP-TBB-CPU/application/owm_optim3.cpp):
//   readXYZfile -> owm_xyz_read + owm_cloud_create
//   parallel_qtree + storeMinAndNumPoints -> owm_tree_build
//   stage1 / stage2 / grid + stage3 -> owm_stage1 / owm_stage2 / owm_stage3
//   the application's loop body -> owm_run
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "owm_ctx.cuh"

namespace owm {

namespace {
std::atomic<int64_t> g_launches{0};
thread_local std::string g_last_error;
}  // namespace

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
  g_last_error = buf;
  cudaGetLastError();  // clear sticky-free errors so the context stays usable
}

void count_launch(int64_t* ctx_counter, int64_t k) {
  g_launches.fetch_add(k, std::memory_order_relaxed);
  if (ctx_counter) *ctx_counter += k;
}

int64_t total_launches() { return g_launches.load(); }

const char* last_cuda_error() { return g_last_error.c_str(); }

void set_last_error_text(const char* what) { g_last_error = what; }

Profiler*& tls_profiler() {
  static thread_local Profiler* p = nullptr;
  return p;
}

cudaEvent_t Profiler::take() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void Profiler::clear() {
  for (auto& r : recs) {
    pool.push_back(r.a);
    pool.push_back(r.b);
  }
  recs.clear();
}

void prof_begin(const char* name, cudaStream_t s) {
  Profiler* p = tls_profiler();
  p->pending = name;
  p->pending_ev = p->take();
  cudaEventRecord(p->pending_ev, s);
}

void prof_end(cudaStream_t s) {
  Profiler* p = tls_profiler();
  cudaEvent_t b = p->take();
  cudaEventRecord(b, s);
  p->recs.push_back({p->pending, p->pending_ev, b});
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool device_ptr_on(const void* p, int device) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == device);
}

int DeviceBuffer::reserve(size_t bytes, cudaStream_t s) {
  if (bytes <= cap) return OWM_OK;
  if (ptr) {
    cudaFreeAsync(ptr, s);
    ptr = nullptr;
    cap = 0;
  }
  size_t want = bytes + bytes / 8 + 4096;
  cudaError_t e = cudaMallocAsync(&ptr, want, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ptr = nullptr;
    return OWM_ENOMEM;
  }
  cap = want;
  return OWM_OK;
}

void DeviceBuffer::release(cudaStream_t s) {
  if (ptr) cudaFreeAsync(ptr, s);
  ptr = nullptr;
  cap = 0;
}

int tree_alloc(TreeStore* t, DeviceBuffer* mem, int64_t n, const owm_tree_cfg& cfg, cudaStream_t s) {
  int64_t ncap = tree_node_cap(n, cfg);
  size_t bytes = 0;
  auto sz = [](size_t b) { return (b + 255) & ~(size_t)255; };
  bytes += 3 * sz((size_t)n * 8) + sz((size_t)n * 4) + sz((size_t)ncap * sizeof(Node));
  int rc = mem->reserve(bytes, s);
  if (rc) return rc;
  char* p = static_cast<char*>(mem->ptr);
  t->xk = (int64_t*)p;
  p += sz((size_t)n * 8);
  t->yk = (int64_t*)p;
  p += sz((size_t)n * 8);
  t->zk = (int64_t*)p;
  p += sz((size_t)n * 8);
  t->pid = (uint32_t*)p;
  p += sz((size_t)n * 4);
  t->nodes = (Node*)p;
  t->point_cap = n;
  t->node_cap = ncap;
  return OWM_OK;
}

int validate_tree_cfg(const owm_tree_cfg* cfg) {
  if (!cfg) return OWM_EINVAL;
  if (cfg->policy == OWM_TREE_MAX_NUMBER) {
    return cfg->max_number >= 1 ? OWM_OK : OWM_EINVAL;  // any capacity; leaves use leaf_size()
  }
  if (cfg->policy == OWM_TREE_MIN_RADIUS) return cfg->min_radius > 0.0f && std::isfinite(cfg->min_radius) ? OWM_OK : OWM_EINVAL;
  return OWM_EINVAL;
}

}  // namespace owm

using namespace owm;

struct owm_cloud {
  owm_ctx* ctx;
  int device;  // destroy needs no context (it may already be gone)
  DeviceBuffer mem;  // n records of kCloudStride doubles (x, y, z, pad)
  DeviceBuffer xy;   // n (x, y) pairs
  int64_t n;
  owm_bbox bbox;
};

namespace {
// The kernels' view of a cloud: its records and its x, y array.
PointsView cloud_points(const owm_cloud* cl) {
  return PointsView{static_cast<const double*>(cl->mem.ptr), kCloudStride, static_cast<const double*>(cl->xy.ptr),
                    kCloudXyStride};
}
}  // namespace

struct owm_tree {
  owm_ctx* ctx;
  int device;
  DeviceBuffer mem;
  TreeStore t;
  const double* d_xy;  // borrowed from the cloud: its x, y array (stage 3 reads LLP coordinates)
  owm_bbox bbox;
  owm_tree_cfg cfg;
};

extern "C" {

int owm_ctx_create(int device, owm_ctx** out) {
  if (!out) return OWM_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || device < 0 || device >= ndev) {
    cudaGetLastError();
    return OWM_ECUDA;
  }
  OWM_CUDA_TRY(cudaSetDevice(device));
  owm_ctx* c = new owm_ctx();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return OWM_ECUDA;
  }
  // keep freed pool memory cached: repeated runs then allocate nothing new
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  cudaGetLastError();
  if (cudaMalloc(&c->d_small, 4096) != cudaSuccess || cudaMallocHost(&c->h_small, 4096) != cudaSuccess ||
      cudaMalloc(&c->d_job, 4 * sizeof(QueryJob)) != cudaSuccess) {
    cudaGetLastError();
    owm_ctx_destroy(c);
    return OWM_ENOMEM;
  }
  cudaMemset(c->d_small, 0, 4096);
  for (auto& e : c->ev) cudaEventCreate(&e);
  if (cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->side_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->side_join, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    owm_ctx_destroy(c);
    return OWM_ECUDA;
  }
  cudaStreamSynchronize(c->stream);
  *out = c;
  return OWM_OK;
}

int owm_ctx_destroy(owm_ctx* c) {
  if (!c) return OWM_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  c->scratch.release(c->stream);
  c->tree_mem.release(c->stream);
  c->input.release(c->stream);
  c->outbuf.release(c->stream);
  for (auto& a : c->aslot) {
    a.input.release(c->copy_stream ? c->copy_stream : c->stream);
    if (a.ready) cudaEventDestroy(a.ready);
    if (a.done) cudaEventDestroy(a.done);
    if (a.h_seeds) cudaFreeHost(a.h_seeds);
    if (a.h_words) cudaFreeHost(a.h_words);
  }
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  if (c->side_stream) {
    cudaStreamSynchronize(c->side_stream);
    cudaStreamDestroy(c->side_stream);
  }
  if (c->side_fork) cudaEventDestroy(c->side_fork);
  if (c->side_join) cudaEventDestroy(c->side_join);
  c->prof.clear();
  for (cudaEvent_t e : c->prof.pool) cudaEventDestroy(e);
  c->prof.pool.clear();
  if (c->d_small) cudaFree(c->d_small);
  if (c->d_job) cudaFree(c->d_job);
  if (c->h_small) cudaFreeHost(c->h_small);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  cudaGetLastError();
  delete c;
  return OWM_OK;
}

int owm_ctx_sync(owm_ctx* c) {
  if (!c) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return OWM_OK;
}

void* owm_ctx_stream(owm_ctx* c) { return c ? (void*)c->stream : nullptr; }

int64_t owm_ctx_launches(const owm_ctx* c) { return c ? c->launches : owm::total_launches(); }

const char* owm_last_error(void) { return owm::last_cuda_error(); }

int owm_ctx_device_status(owm_ctx* c, int32_t* status) {
  if (!c || !status) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaMemcpyAsync(c->h_small, c->d_small + kStatusSlot, 4, cudaMemcpyDeviceToHost, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  *status = (int32_t)c->h_small[0];
  return OWM_OK;
}

int owm_ctx_set_tuning(owm_ctx* c, const owm_tuning* t) {
  if (!c || !t) return OWM_EINVAL;
  owm_tuning u = c->tuning;
  if (t->walk_patch_x) {
    const int32_t p = t->walk_patch_x;
    if (p < 1 || p > 32 || (p & (p - 1))) return OWM_EINVAL;
    u.walk_patch_x = p;
  }
  if (t->cell_warps) {
    if (t->cell_warps != 2 && t->cell_warps != 4 && t->cell_warps != 8) return OWM_EINVAL;
    u.cell_warps = t->cell_warps;
  }
  if (t->gather_block) {
    if (t->gather_block != 128 && t->gather_block != 256 && t->gather_block != 512) return OWM_EINVAL;
    u.gather_block = t->gather_block;
  }
  c->tuning = u;
  return OWM_OK;
}

int owm_ctx_get_tuning(owm_ctx* c, owm_tuning* t) {
  if (!c || !t) return OWM_EINVAL;
  *t = c->tuning;
  return OWM_OK;
}

int owm_ctx_set_walk_limit(owm_ctx* c, int32_t limit) {
  if (!c || limit < 0) return OWM_EINVAL;
  c->walk_limit = limit;
  return OWM_OK;
}

int owm_ctx_set_profiling(owm_ctx* c, int on) {
  if (!c) return OWM_EINVAL;
  if (!on) {
    cudaStreamSynchronize(c->stream);
    c->prof.clear();
  }
  c->profiling = on != 0;
  return OWM_OK;
}

int owm_ctx_kernel_times(owm_ctx* c, int32_t cap, char (*names)[64], double* ms, int64_t* calls, int32_t* n) {
  if (!c || !n || cap < 0) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  std::vector<std::string> nm;
  std::vector<double> tot;
  std::vector<int64_t> cnt;
  for (auto& r : c->prof.recs) {
    float t = 0;
    if (cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    size_t k = 0;
    while (k < nm.size() && nm[k] != r.name) ++k;
    if (k == nm.size()) {
      nm.push_back(r.name);
      tot.push_back(0);
      cnt.push_back(0);
    }
    tot[k] += t;
    cnt[k] += 1;
  }
  c->prof.clear();
  int32_t m = (int32_t)nm.size();
  *n = m;
  for (int32_t k = 0; k < m && k < cap; ++k) {
    if (names) {
      std::strncpy(names[k], nm[k].c_str(), 63);
      names[k][63] = 0;
    }
    if (ms) ms[k] = tot[k];
    if (calls) calls[k] = cnt[k];
  }
  return m > cap ? OWM_ERANGE : OWM_OK;
}

int owm_cloud_create(owm_ctx* c, const double* xyz, int64_t n, const owm_bbox* bbox, owm_cloud** out) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !xyz || !out || n <= 0 || n >= 0x7FFFFFFFLL) return OWM_EINVAL;
  *out = nullptr;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  // The kernels read xyz itself only when it is device memory of this
  // context's device, 8-byte aligned; host memory, another device's memory or
  // an unaligned pointer go through a device copy first (DeviceBuffer's
  // stream-ordered free releases it on every return).
  const bool host = !is_device_ptr(xyz);
  const bool direct = device_ptr_on(xyz, c->device) && (reinterpret_cast<uintptr_t>(xyz) & 7u) == 0;
  struct Stage {
    DeviceBuffer b;
    cudaStream_t s;
    ~Stage() { b.release(s); }
  } stage{{}, c->stream};
  const double* src = xyz;
  if (!direct) {
    if (stage.b.reserve((size_t)n * 24, c->stream) != OWM_OK) return OWM_ENOMEM;
    OWM_CUDA_TRY(cudaMemcpyAsync(stage.b.ptr, xyz, (size_t)n * 24, cudaMemcpyDefault, c->stream));
    src = static_cast<const double*>(stage.b.ptr);
  }
  owm_bbox bb;
  if (bbox) {
    bb = *bbox;
  } else if (host) {
    owm_bbox_of(xyz, n, &bb);
  } else {
    int rc = device_bbox(c, src, 3, n, &bb);
    if (rc) return rc;
  }
  if (!std::isfinite(bb.min_x) || !std::isfinite(bb.max_x) || !std::isfinite(bb.min_y) ||
      !std::isfinite(bb.max_y) || bb.max_x < bb.min_x || bb.max_y < bb.min_y) {
    cudaStreamSynchronize(c->stream);
    return OWM_EINVAL;
  }
  owm_cloud* cl = new owm_cloud();
  cl->ctx = c;
  cl->device = c->device;
  cl->n = n;
  cl->bbox = bb;
  if (cl->mem.reserve((size_t)n * 8 * kCloudStride, c->stream) != OWM_OK ||
      cl->xy.reserve((size_t)n * 8 * kCloudXyStride, c->stream) != OWM_OK) {
    cl->mem.release(c->stream);
    cudaStreamSynchronize(c->stream);
    delete cl;
    return OWM_ENOMEM;
  }
  // the points as 32-byte records and the x, y array
  int rc = pad_points(src, n, static_cast<double*>(cl->mem.ptr), static_cast<double*>(cl->xy.ptr), c->stream,
                      &c->launches);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (rc || e != cudaSuccess) {
    if (e != cudaSuccess) set_last_cuda_error(e, "cloud copy", __FILE__, __LINE__);
    cudaStreamSynchronize(c->stream);
    cl->mem.release(c->stream);
    cl->xy.release(c->stream);
    delete cl;
    return rc ? rc : OWM_ECUDA;
  }
  *out = cl;
  return OWM_OK;
}

int owm_cloud_destroy(owm_cloud* cl) {
  if (!cl) return OWM_OK;
  cudaSetDevice(cl->device);
  if (cl->mem.ptr) cudaFree(cl->mem.ptr);  // synchronising free; no stream or context needed
  if (cl->xy.ptr) cudaFree(cl->xy.ptr);
  cudaGetLastError();
  delete cl;
  return OWM_OK;
}

int64_t owm_cloud_size(const owm_cloud* cl) { return cl ? cl->n : 0; }

int owm_cloud_bbox(const owm_cloud* cl, owm_bbox* out) {
  if (!cl || !out) return OWM_EINVAL;
  *out = cl->bbox;
  return OWM_OK;
}

int owm_cloud_copy_out(const owm_cloud* cl, double* xyz, int64_t n) {
  if (!cl || !xyz || n < 0 || n > cl->n) return OWM_EINVAL;
  if (n == 0) return OWM_OK;
  OWM_CUDA_TRY(cudaSetDevice(cl->device));
  // the records' x, y, z into plain points: in a device copy, then to xyz
  // (its own stream and memory: the cloud's context may be busy or gone)
  double* tmp = nullptr;
  cudaStream_t s = nullptr;
  int64_t launches = 0;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&tmp), (size_t)n * 24, s);
  int rc = e == cudaSuccess ? unpad_points(static_cast<const double*>(cl->mem.ptr), n, tmp, s, &launches) : OWM_ECUDA;
  if (!rc) e = cudaMemcpyAsync(xyz, tmp, (size_t)n * 24, cudaMemcpyDefault, s);
  if (s) {
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (tmp) cudaFreeAsync(tmp, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  if (rc) return rc;
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "owm_cloud_copy_out", __FILE__, __LINE__);
    return OWM_ECUDA;
  }
  return OWM_OK;
}

namespace {
// Wraps parsed device points as a cloud (bbox: the header's, else the data's).
int finish_parsed_cloud(owm_ctx* c, DeviceBuffer& mem, DeviceBuffer& xy, int64_t n, int64_t declared,
                        const owm_bbox& hb, owm_cloud** out) {
  owm_bbox bb = hb;
  if (declared < 0) {
    int rc = device_bbox(c, static_cast<const double*>(xy.ptr), kCloudXyStride, n, &bb);
    if (rc) return rc;
  }
  if (!std::isfinite(bb.min_x) || !std::isfinite(bb.max_x) || !std::isfinite(bb.min_y) ||
      !std::isfinite(bb.max_y) || bb.max_x < bb.min_x || bb.max_y < bb.min_y)
    return OWM_EIO;
  owm_cloud* cl = new owm_cloud();
  cl->ctx = c;
  cl->device = c->device;
  cl->n = n;
  cl->bbox = bb;
  cl->mem = mem;
  mem.ptr = nullptr;
  mem.cap = 0;
  cl->xy = xy;
  xy.ptr = nullptr;
  xy.cap = 0;
  *out = cl;
  return OWM_OK;
}
}  // namespace

int owm_cloud_parse_xyz(owm_ctx* c, const char* text, int64_t nbytes, owm_cloud** out) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !text || !out || nbytes < 0) return OWM_EINVAL;
  *out = nullptr;
  if (nbytes == 0) return OWM_EIO;  // like an empty file
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  // device text: the header is read from a host copy of its first MB (the
  // header's lines are short; a first data line only needs three numbers)
  const bool on_device = is_device_ptr(text);
  std::vector<char> head;
  const char* htext = text;
  int64_t hbytes = nbytes;
  if (on_device) {
    hbytes = std::min<int64_t>(nbytes, (int64_t)1 << 20);
    head.resize((size_t)hbytes);
    OWM_CUDA_TRY(cudaMemcpy(head.data(), text, (size_t)hbytes, cudaMemcpyDeviceToHost));
    htext = head.data();
  }
  int64_t data_off = 0, declared = -1;
  owm_bbox hb{};
  int rc = xyz_header(htext, hbytes, &data_off, &declared, &hb);
  if (rc) return rc;
  DeviceBuffer dt, pts, pxy;
  // the parser's 16-byte loads want an aligned copy with readable slack
  rc = dt.reserve((size_t)((nbytes + 15) & ~(int64_t)15) + 32, c->stream);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(dt.ptr, text, (size_t)nbytes, cudaMemcpyDefault, c->stream);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "text copy", __FILE__, __LINE__);
    dt.release(c->stream);
    return OWM_ECUDA;
  }
  int64_t n = 0;
  rc = parse_device_text(c, static_cast<const char*>(dt.ptr), nbytes, data_off, declared, &pts, &pxy, &n,
                         &c->launches);
  dt.release(c->stream);
  if (!rc) rc = finish_parsed_cloud(c, pts, pxy, n, declared, hb, out);
  if (rc) {
    pts.release(c->stream);
    pxy.release(c->stream);
  }
  return rc;
}

int owm_cloud_load_xyz(owm_ctx* c, const char* path, owm_cloud** out) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !path || !out) return OWM_EINVAL;
  *out = nullptr;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  const int fd = ::open(path, O_RDONLY);
  if (fd < 0) return OWM_EIO;
  struct stat sb;
  if (::fstat(fd, &sb) != 0 || sb.st_size <= 0) {
    ::close(fd);
    return OWM_EIO;
  }
  const int64_t nbytes = (int64_t)sb.st_size;
  // the file moves through two pinned chunks: reading chunk k + 1 overlaps the
  // device copy of chunk k
  constexpr int64_t kChunk = (int64_t)64 << 20;
  char* pin[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  DeviceBuffer dt, pts, pxy;
  int rc = OWM_OK;
  int64_t data_off = 0, declared = -1;
  owm_bbox hb{};
  auto cleanup = [&]() {
    cudaStreamSynchronize(c->stream);
    for (int i = 0; i < 2; ++i) {
      if (pin[i]) cudaFreeHost(pin[i]);
      if (done[i]) cudaEventDestroy(done[i]);
    }
    dt.release(c->stream);
    ::close(fd);
  };
  for (int i = 0; i < 2 && !rc; ++i) {
    if (cudaHostAlloc(reinterpret_cast<void**>(&pin[i]), (size_t)kChunk, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess)
      rc = OWM_ENOMEM;
  }
  if (!rc) rc = dt.reserve((size_t)((nbytes + 15) & ~(int64_t)15) + 32, c->stream);
  for (int64_t off = 0, k = 0; !rc && off < nbytes; off += kChunk, ++k) {
    const int b = (int)(k & 1);
    if (k >= 2 && cudaEventSynchronize(done[b]) != cudaSuccess) rc = OWM_ECUDA;
    const int64_t len = std::min<int64_t>(kChunk, nbytes - off);
    for (int64_t got = 0; !rc && got < len;) {
      const ssize_t r = ::pread(fd, pin[b] + got, (size_t)(len - got), (off_t)(off + got));
      if (r <= 0) rc = OWM_EIO;
      got += r > 0 ? r : 0;
    }
    if (!rc && k == 0) rc = xyz_header(pin[0], len, &data_off, &declared, &hb);  // the header lies in the first chunk
    if (!rc && (cudaMemcpyAsync(static_cast<char*>(dt.ptr) + off, pin[b], (size_t)len, cudaMemcpyHostToDevice,
                                c->stream) != cudaSuccess ||
                cudaEventRecord(done[b], c->stream) != cudaSuccess))
      rc = OWM_ECUDA;
  }
  int64_t n = 0;
  if (!rc)
    rc = parse_device_text(c, static_cast<const char*>(dt.ptr), nbytes, data_off, declared, &pts, &pxy, &n,
                           &c->launches);
  cleanup();
  if (!rc) rc = finish_parsed_cloud(c, pts, pxy, n, declared, hb, out);
  if (rc) {
    pts.release(c->stream);
    pxy.release(c->stream);
  }
  return rc;
}

int owm_tree_build(owm_ctx* c, const owm_cloud* cl, const owm_tree_cfg* cfg, owm_tree** out) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !cl || !out || validate_tree_cfg(cfg) != OWM_OK) return OWM_EINVAL;
  *out = nullptr;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  owm_tree* tr = new owm_tree();
  tr->ctx = c;
  tr->device = c->device;
  tr->cfg = *cfg;
  tr->d_xy = static_cast<const double*>(cl->xy.ptr);
  tr->bbox = cl->bbox;
  int rc = tree_alloc(&tr->t, &tr->mem, cl->n, *cfg, c->stream);
  tr->t.gather_block = c->tuning.gather_block;
  if (!rc) rc = c->scratch.reserve(tree_scratch_bytes(cl->n), c->stream);
  if (!rc) rc = clear_status(c);
  if (!rc)
    rc = build_tree(cloud_points(cl), cl->n, cl->bbox, *cfg, &tr->t, c->scratch.ptr, c->scratch.cap,
                    c->d_small + kStatusSlot, c->stream, &c->launches);
  if (!rc) rc = check_input_status(c);
  if (rc) {
    tr->mem.release(c->stream);
    cudaStreamSynchronize(c->stream);
    delete tr;
    return rc;
  }
  *out = tr;
  return OWM_OK;
}

int owm_tree_get_info(owm_ctx* c, const owm_tree* tr, owm_tree_info* info) {
  if (!c || !tr || !info) return OWM_EINVAL;
  std::memset(info, 0, sizeof(*info));
  info->npoints = tr->t.n;
  info->nleaves = tr->t.nleaves;
  info->nnodes = 2 * (int64_t)tr->t.nleaves - 1;
  info->key_bits = tr->t.key_bits;
  info->max_leaf = tr->t.max_leaf;
  Node root;
  OWM_CUDA_TRY(cudaMemcpyAsync(&root, tr->t.nodes + tr->t.root, sizeof(Node), cudaMemcpyDeviceToHost, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  info->root_count = root.count;
  info->root_min_id = root.min_id;
  return OWM_OK;
}

int owm_tree_check(owm_ctx* c, const owm_tree* tr) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !tr) return OWM_EINVAL;
  int32_t bad = 0;
  int rc = check_tree(&tr->t, reinterpret_cast<int32_t*>(c->d_small + kCheckSlot), c->stream, &c->launches, &bad);
  if (rc) return rc;
  Node root;
  OWM_CUDA_TRY(cudaMemcpyAsync(&root, tr->t.nodes + tr->t.root, sizeof(Node), cudaMemcpyDeviceToHost, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (bad != 0 || (int64_t)root.count != tr->t.n) return OWM_EINVAL;
  return OWM_OK;
}

int owm_tree_destroy(owm_tree* tr) {
  if (!tr) return OWM_OK;
  cudaSetDevice(tr->device);
  if (tr->mem.ptr) cudaFree(tr->mem.ptr);
  cudaGetLastError();
  delete tr;
  return OWM_OK;
}

int owm_stage1(owm_ctx* c, const owm_tree* tr, const owm_params* p, int64_t* win_min) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !tr || !p || !win_min || p->ncells <= 0) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  const int64_t nc = p->ncells;
  size_t need = 2 * sizeof(Edge) * 65536 + (size_t)nc * 4 + (size_t)nc * 8 + 4096;
  int rc = c->outbuf.reserve(need, c->stream);
  if (rc) return rc;
  char* base = static_cast<char*>(c->outbuf.ptr);
  Edge* ex = (Edge*)base;
  Edge* ey = ex + 65536;
  uint32_t* win = (uint32_t*)(ey + 65536);
  int64_t* w64 = (int64_t*)(((uintptr_t)(win + nc) + 255) & ~(uintptr_t)255);
  rc = clear_status(c);
  if (!rc) rc = run_stage1(c, tr->t, *p, ex, ey, win);
  if (!rc) rc = check_input_status(c);
  if (rc) return rc;
  bool dev = device_ptr_on(win_min, c->device);  // written by a kernel only on this device
  rc = u32_to_i64_ids(win, nullptr, nc, dev ? win_min : w64, c->stream, &c->launches);
  if (rc) return rc;
  if (!dev) OWM_CUDA_TRY(cudaMemcpyAsync(win_min, w64, (size_t)nc * 8, cudaMemcpyDeviceToHost, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return OWM_OK;
}

int owm_stage2(owm_ctx* c, int64_t* win_min, int64_t ncells, double overlap, int64_t* n_llp) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !win_min || !n_llp || ncells <= 0 || !(overlap >= 0.0 && overlap < 1.0) || ncells >= 0x7FFFFFFFLL)
    return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  size_t need = (size_t)ncells * 8 + 2 * (size_t)ncells * 4 + 4096;
  int rc = c->outbuf.reserve(need, c->stream);
  if (!rc) rc = c->scratch.reserve(stage2_scratch_bytes(ncells), c->stream);
  if (rc) return rc;
  char* base = static_cast<char*>(c->outbuf.ptr);
  int64_t* w64 = (int64_t*)base;
  uint32_t* win = (uint32_t*)(((uintptr_t)(w64 + ncells) + 255) & ~(uintptr_t)255);
  uint32_t* llp = (uint32_t*)(((uintptr_t)(win + ncells) + 255) & ~(uintptr_t)255);
  uint32_t* d_cnt = c->d_small + kCountSlot;
  OWM_CUDA_TRY(cudaMemcpyAsync(w64, win_min, (size_t)ncells * 8, cudaMemcpyDefault, c->stream));
  rc = i64_to_u32_ids(w64, ncells, win, c->stream, &c->launches);
  if (!rc)
    rc = run_stage2(win, ncells, 0xFFFFFFFELL, overlap, llp, d_cnt, c->scratch.ptr, c->scratch.cap, c->stream,
                    &c->launches);
  if (rc) return rc;
  rc = u32_to_i64_ids(llp, d_cnt, ncells, w64, c->stream, &c->launches);
  if (rc) return rc;
  OWM_CUDA_TRY(cudaMemcpyAsync(c->h_small, d_cnt, 4, cudaMemcpyDeviceToHost, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  int64_t m = c->h_small[0];
  if (m > 0) OWM_CUDA_TRY(cudaMemcpyAsync(win_min, w64, (size_t)m * 8, cudaMemcpyDefault, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  *n_llp = m;
  return OWM_OK;
}

int owm_stage3(owm_ctx* c, const owm_tree* tr, const owm_params* p, const int64_t* llp, int64_t n_llp, int64_t* out,
               int64_t cap, int64_t* n_out) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !tr || !p || (!llp && n_llp > 0) || n_llp < 0 || !n_out || (!out && cap > 0)) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  *n_out = 0;
  if (p->bsize == 0 || p->ngrid <= 0) return OWM_OK;
  const int64_t ng = p->ngrid;
  const int64_t m = std::max<int64_t>(n_llp, 1);
  size_t need = (size_t)m * 8 + (size_t)m * 4 + (size_t)ng * 4 + (size_t)ng * 8 + 8192;
  int rc = c->outbuf.reserve(need, c->stream);
  if (!rc) rc = c->scratch.reserve(stage3_scratch_bytes(ng), c->stream);
  if (rc) return rc;
  char* base = static_cast<char*>(c->outbuf.ptr);
  auto al = [](void* q) { return (char*)(((uintptr_t)q + 255) & ~(uintptr_t)255); };
  int64_t* l64 = (int64_t*)base;
  uint32_t* l32 = (uint32_t*)al(l64 + m);
  uint32_t* s3 = (uint32_t*)al(l32 + m);
  int64_t* s64 = (int64_t*)al(s3 + ng);
  uint32_t* d_nllp = c->d_small + kLlpSlot;
  uint32_t* d_cnt = c->d_small + kCountSlot;
  c->h_small[1] = (uint32_t)n_llp;
  OWM_CUDA_TRY(cudaMemcpyAsync(d_nllp, &c->h_small[1], 4, cudaMemcpyHostToDevice, c->stream));
  if (n_llp > 0) {
    OWM_CUDA_TRY(cudaMemcpyAsync(l64, llp, (size_t)n_llp * 8, cudaMemcpyDefault, c->stream));
    rc = i64_to_u32_ids(l64, n_llp, l32, c->stream, &c->launches);
    if (rc) return rc;
  }
  rc = clear_status(c);
  if (!rc)
    rc = run_stage3(tr->t.view(c->walk_limit, c->tuning.cell_warps), tr->d_xy, kCloudXyStride, *p, l32, d_nllp, n_llp, s3, d_cnt, c->scratch.ptr, c->scratch.cap,
                    c->d_job, c->d_small + kStatusSlot, c->stream, &c->launches);
  if (!rc) rc = check_input_status(c);
  if (rc) return rc;
  OWM_CUDA_TRY(cudaMemcpyAsync(c->h_small + 2, d_cnt, 4, cudaMemcpyDeviceToHost, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  int64_t k = c->h_small[2];
  *n_out = k;
  if (k > cap) return OWM_ERANGE;
  if (k > 0) {
    rc = u32_to_i64_ids(s3, nullptr, k, s64, c->stream, &c->launches);
    if (rc) return rc;
    OWM_CUDA_TRY(cudaMemcpyAsync(out, s64, (size_t)k * 8, cudaMemcpyDefault, c->stream));
    OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  return OWM_OK;
}

int owm_run(owm_ctx* c, const owm_cloud* cl, const owm_run_cfg* cfg, int64_t* seeds, int64_t cap, int64_t* n_seeds,
            owm_run_info* info) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !cl || !cfg || !n_seeds || (!seeds && cap > 0)) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  return run_pipeline(c, cloud_points(cl), cl->n, cl->bbox, *cfg, seeds, cap,
                      n_seeds, info);
}

int owm_run_host(owm_ctx* c, const double* xyz, int64_t n, const owm_bbox* bbox, const owm_run_cfg* cfg,
                 int64_t* seeds, int64_t cap, int64_t* n_seeds, owm_run_info* info) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !xyz || !cfg || !n_seeds || n <= 0 || n >= 0x7FFFFFFFLL || (!seeds && cap > 0)) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  // device input: its bbox from the copy on this device (xyz may be another device's memory)
  const bool host = !is_device_ptr(xyz);
  owm_bbox bb;
  if (bbox)
    bb = *bbox;
  else if (host)
    owm_bbox_of(xyz, n, &bb);
  int rc = c->input.reserve((size_t)n * 24 + kXyzSlack, c->stream);
  if (rc) return rc;
  OWM_CUDA_TRY(cudaMemcpyAsync(c->input.ptr, xyz, (size_t)n * 24, cudaMemcpyDefault, c->stream));
  if (!bbox && !host) {
    rc = device_bbox(c, static_cast<const double*>(c->input.ptr), 3, n, &bb);
    if (rc) return rc;
  }
  return run_pipeline(c, plain_points(static_cast<const double*>(c->input.ptr)), n, bb, *cfg, seeds, cap, n_seeds,
                      info);
}

}  // extern "C"

namespace {

// Queues the run of slot a on the context's stream (after whatever is queued
// there: a copy-stream event for host input), then the device->host copy of
// its status words and of the whole seed buffer into the slot's pinned
// staging, and hands out the ticket.  On failure the caller's fail() waits
// for everything queued so far.
template <class Fail>
int submit_slot(owm_ctx* c, owm_ctx::AsyncSlot& a, const PointsView& pts, int64_t n, const owm_bbox& bb,
                const owm_run_cfg& cfg, int64_t* seeds, int64_t cap, int64_t* ticket, const char* fn, Fail fail) {
  int64_t* d_seeds = nullptr;
  int64_t room = 0;
  int rc = run_pipeline_enqueue(c, pts, n, bb, cfg, &a.p, &d_seeds, &room);
  if (rc) return fail(rc);
  if (a.h_cap < room) {
    // growth only: the old staging may still be a copy target
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(OWM_ECUDA);
    if (a.h_seeds) cudaFreeHost(a.h_seeds);
    a.h_seeds = nullptr;
    a.h_cap = 0;
    if (cudaMallocHost(&a.h_seeds, (size_t)room * 8) != cudaSuccess) {
      cudaGetLastError();
      return fail(OWM_ENOMEM);
    }
    a.h_cap = room;
  }
  cudaError_t e = cudaMemcpyAsync(a.h_words, c->d_small, 32, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a.h_seeds, d_seeds, (size_t)room * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(a.done, c->stream);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, fn, __FILE__, __LINE__);
    return fail(OWM_ECUDA);
  }
  a.seeds = seeds;
  a.cap = cap;
  a.room = room;
  a.ticket = c->next_ticket++;
  *ticket = a.ticket;
  return OWM_OK;
}

// The slot the next ticket uses, with its events and pinned status words
// created; nullptr (and *rc) when both runs are still in flight or creation
// failed.
owm_ctx::AsyncSlot* next_slot(owm_ctx* c, int* rc) {
  owm_ctx::AsyncSlot& a = c->aslot[c->next_ticket & 1];
  *rc = OWM_OK;
  if (a.ticket != 0) {
    *rc = OWM_EAGAIN;  // both runs in flight: wait for the older one first
    return nullptr;
  }
  cudaError_t e = cudaSuccess;
  if (!a.ready) e = cudaEventCreateWithFlags(&a.ready, cudaEventDisableTiming);
  if (e == cudaSuccess && !a.done) e = cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming);
  if (e == cudaSuccess && !a.h_words) e = cudaMallocHost(&a.h_words, 32);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "owm_run_submit", __FILE__, __LINE__);
    *rc = OWM_ECUDA;
    return nullptr;
  }
  return &a;
}

}  // namespace

extern "C" {

int owm_run_submit(owm_ctx* c, const owm_cloud* cl, const owm_run_cfg* cfg, int64_t* seeds, int64_t cap,
                   int64_t* ticket) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !cl || !cfg || !ticket || (!seeds && cap > 0)) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  int rc = OWM_OK;
  owm_ctx::AsyncSlot* a = next_slot(c, &rc);
  if (!a) return rc;
  auto fail = [&](int code) {
    cudaStreamSynchronize(c->side_stream);
    cudaStreamSynchronize(c->stream);
    return code;
  };
  return submit_slot(c, *a, cloud_points(cl), cl->n, cl->bbox, *cfg, seeds, cap,
                     ticket,
                     "owm_run_submit", fail);
}

int owm_run_host_submit(owm_ctx* c, const double* xyz, int64_t n, const owm_bbox* bbox, const owm_run_cfg* cfg,
                        int64_t* seeds, int64_t cap, int64_t* ticket) {
  ProfScope prof_scope(c ? c->active_prof() : nullptr);
  if (!c || !xyz || !cfg || !ticket || n <= 0 || n >= 0x7FFFFFFFLL || (!seeds && cap > 0)) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  int rc = OWM_OK;
  owm_ctx::AsyncSlot* ap = next_slot(c, &rc);
  if (!ap) return rc;
  owm_ctx::AsyncSlot& a = *ap;
  // device input: its bbox from the copy on this device, below (xyz may be another device's memory)
  const bool host = !is_device_ptr(xyz);
  owm_bbox bb;
  if (bbox)
    bb = *bbox;
  else if (host)
    owm_bbox_of(xyz, n, &bb);
  if (!c->copy_stream) OWM_CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  // This slot's previous run has been waited for, so nothing reads its input
  // buffer any more.  Reserving on the copy stream orders a (re)allocation
  // before the copy without making the copy wait for the other run's compute.
  rc = a.input.reserve((size_t)n * 24 + kXyzSlack, c->copy_stream);
  if (rc) return rc;
  OWM_CUDA_TRY(cudaMemcpyAsync(a.input.ptr, xyz, (size_t)n * 24, cudaMemcpyDefault, c->copy_stream));
  // From here on the copy may still be reading xyz: a failed submit waits for
  // it before returning, so the caller may free xyz after any return.
  auto fail = [&](int code) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamSynchronize(c->side_stream);
    cudaStreamSynchronize(c->stream);
    return code;
  };
  cudaError_t e = cudaEventRecord(a.ready, c->copy_stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, a.ready, 0);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "owm_run_host_submit", __FILE__, __LINE__);
    return fail(OWM_ECUDA);
  }
  if (!bbox && !host) {  // on c->stream after the copy; synchronous
    rc = device_bbox(c, static_cast<const double*>(a.input.ptr), 3, n, &bb);
    if (rc) return fail(rc);
  }
  return submit_slot(c, a, plain_points(static_cast<const double*>(a.input.ptr)), n, bb, *cfg, seeds, cap, ticket,
                     "owm_run_host_submit", fail);
}

int owm_run_host_wait(owm_ctx* c, int64_t ticket, int64_t* n_seeds, owm_run_info* info) {
  if (!c || !n_seeds || ticket <= 0) return OWM_EINVAL;
  owm_ctx::AsyncSlot& a = c->aslot[ticket & 1];
  if (a.ticket != ticket) return OWM_EINVAL;  // unknown or already collected
  OWM_CUDA_TRY(cudaSetDevice(c->device));
  cudaError_t e = cudaEventSynchronize(a.done);
  a.ticket = 0;
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "owm_run_host_wait", __FILE__, __LINE__);
    return OWM_ECUDA;
  }
  const uint32_t st = a.h_words[kStatusSlot];
  if (st & kStatusNonFinite) return OWM_EINVAL;
  if (st & kStatusWalkBound) return OWM_ETIMEOUT;
  const int64_t nllp = a.h_words[kLlpSlot], ns3 = a.h_words[kS3Slot];
  const int64_t total = nllp + ns3;
  *n_seeds = total;
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->n_llp = nllp;
    info->n_stage3 = ns3;
    info->n_seeds = total;
    info->params = a.p;
  }
  if (total > a.cap || total > a.room) return OWM_ERANGE;
  if (total > 0) std::memcpy(a.seeds, a.h_seeds, (size_t)total * 8);
  return OWM_OK;
}

int owm_run_wait(owm_ctx* c, int64_t ticket, int64_t* n_seeds, owm_run_info* info) {
  return owm_run_host_wait(c, ticket, n_seeds, info);
}

}  // extern "C"
