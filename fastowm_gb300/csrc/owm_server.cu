// Serving: a continuous-batching request loop over device-resident tiles.
//
// Requests (one tile each) are copied to pinned staging at submit and queued.
// A worker thread keeps up to `max_inflight_batches` batches on the GPU, each
// on its own stream: as soon as a slot frees up, the requests that arrived
// meanwhile are admitted as the next batch (bounded by tiles, points and the
// HBM budget) and launched while the other slots' batches are still running,
// so their work overlaps on the device.  A slot keeps its device buffers --
// the finished batch's trees -- resident until that slot is reused; when a
// new batch does not fit the budget, idle slots' buffers are evicted first.
// Per-request latency is submit -> result ready (host steady clock).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "owm_batch.cuh"

namespace owm {

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Pinned host blocks in power-of-two size classes, reused across requests.
class PinnedPool {
 public:
  ~PinnedPool() {
    for (auto& kv : free_)
      for (void* p : kv.second) cudaFreeHost(p);
  }
  void* get(size_t bytes, size_t* cls) {
    size_t c = 4096;
    while (c < bytes) c <<= 1;
    *cls = c;
    std::lock_guard<std::mutex> lk(mu_);
    auto& v = free_[c];
    if (!v.empty()) {
      void* p = v.back();
      v.pop_back();
      return p;
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, c) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return p;
  }
  void put(void* p, size_t cls) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    free_[cls].push_back(p);
  }

 private:
  std::mutex mu_;
  std::map<size_t, std::vector<void*>> free_;
};

struct Request {
  int64_t ticket = 0;
  double* pts = nullptr;
  size_t pts_cls = 0;
  owm_tile_desc desc{};
  double t_submit = 0, t_done = 0;
  int status = OWM_EAGAIN;
  std::vector<int64_t> seeds;
  size_t est_bytes = 0;
};

struct Slot {
  BatchRun run;
  std::vector<Request*> reqs;
  bool busy = false;
  double t_launch = 0;
};

}  // namespace

}  // namespace owm

using namespace owm;

struct owm_server {
  owm_server_cfg cfg{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> pending;
  std::unordered_map<int64_t, Request*> reqs;
  std::vector<std::unique_ptr<Slot>> slots;
  PinnedPool pinned;
  std::thread worker;
  bool stop = false;
  int64_t next_ticket = 1;
  owm_server_stats st{};
  std::vector<owm_tile_desc> scratch_descs;
  std::vector<int64_t> out_seeds, out_off;

  size_t slot_bytes() const {
    size_t b = 0;
    for (auto& s : slots) b += s->run.mem.cap;
    return b;
  }

  // Finish every completed slot; called with mu held.
  void reap() {
    for (auto& sp : slots) {
      Slot& s = *sp;
      if (!s.busy || !s.run.ready()) continue;
      int64_t cap = 0;
      for (Request* r : s.reqs) cap += r->desc.n;  // generous bound refined below
      cap = 0;
      for (Request* r : s.reqs) {
        owm_params p;
        owm_params_compute(&r->desc.bbox, r->desc.n, r->desc.cfg.wsize, r->desc.cfg.overlap, r->desc.cfg.bsize, &p);
        cap += p.ncells + p.ngrid + 1;
      }
      out_seeds.resize((size_t)std::max<int64_t>(cap, 1));
      out_off.resize(s.reqs.size() + 1);
      int rc = s.run.finish(out_seeds.data(), cap, out_off.data(), nullptr);
      double t = now_ms();
      for (size_t k = 0; k < s.reqs.size(); ++k) {
        Request* r = s.reqs[k];
        r->status = rc;
        if (rc == OWM_OK) r->seeds.assign(out_seeds.begin() + out_off[k], out_seeds.begin() + out_off[k + 1]);
        r->t_done = t;
        pinned.put(r->pts, r->pts_cls);
        r->pts = nullptr;
        st.completed++;
        st.points_done += r->desc.n;
      }
      st.busy_ms += t - s.t_launch;
      s.reqs.clear();
      s.busy = false;
      cv_done.notify_all();
    }
  }

  // Form and launch one batch into a free slot; called with mu held.
  bool admit() {
    if (pending.empty()) return false;
    Slot* free_slot = nullptr;
    for (auto& sp : slots)
      if (!sp->busy) {
        free_slot = sp.get();
        break;
      }
    if (!free_slot) return false;
    std::vector<Request*> take;
    int64_t pts = 0, maxn = 0;
    for (Request* r : pending) {
      if ((int32_t)take.size() >= cfg.max_tiles_per_batch) break;
      if (!take.empty() && pts + r->desc.n > cfg.max_points_per_batch) break;
      // (tile, id) keys of stage 2 must fit 32 bits
      int64_t mx = std::max(maxn, r->desc.n);
      int tb = 1, ib = 1;
      while (((int64_t)1 << tb) < (int64_t)take.size() + 1) ++tb;
      while (((int64_t)1 << ib) <= mx + 1) ++ib;
      if (!take.empty() && tb + ib > 32) break;
      take.push_back(r);
      pts += r->desc.n;
      maxn = mx;
    }
    scratch_descs.clear();
    for (Request* r : take) scratch_descs.push_back(r->desc);
    size_t need = BatchRun::estimate_bytes(scratch_descs.data(), (int32_t)scratch_descs.size());
    if (need == (size_t)-1) {  // malformed request: fail it alone
      Request* r = take.front();
      pending.erase(std::find(pending.begin(), pending.end(), r));
      r->status = OWM_EINVAL;
      r->t_done = now_ms();
      pinned.put(r->pts, r->pts_cls);
      r->pts = nullptr;
      cv_done.notify_all();
      return true;
    }
    // budget: other slots' resident buffers + this slot's (grown) buffer
    size_t others = slot_bytes() - free_slot->run.mem.cap;
    size_t mine = std::max(need, free_slot->run.mem.cap);
    if (others + mine > (size_t)cfg.hbm_budget_bytes) {
      // evict idle slots' resident trees
      for (auto& sp : slots)
        if (!sp->busy && sp.get() != free_slot && sp->run.mem.ptr) {
          cudaSetDevice(device);
          sp->run.mem.release(sp->run.stream);
        }
      others = slot_bytes() - free_slot->run.mem.cap;
      if (others + mine > (size_t)cfg.hbm_budget_bytes) {
        if (free_slot->run.mem.cap > need) {
          // shrink this slot to what the batch needs
          free_slot->run.mem.release(free_slot->run.stream);
          mine = need;
        }
        if (others + mine > (size_t)cfg.hbm_budget_bytes) return false;  // wait for a slot to finish
      }
    }
    for (Request* r : take) pending.erase(std::find(pending.begin(), pending.end(), r));
    free_slot->reqs = take;
    free_slot->busy = true;
    free_slot->t_launch = now_ms();
    int rc = free_slot->run.launch(scratch_descs.data(), (int32_t)scratch_descs.size());
    st.batches++;
    st.bytes_in_use = (int64_t)slot_bytes();
    st.peak_bytes = std::max(st.peak_bytes, st.bytes_in_use);
    if (rc) {
      double t = now_ms();
      for (Request* r : take) {
        r->status = rc;
        r->t_done = t;
        pinned.put(r->pts, r->pts_cls);
        r->pts = nullptr;
        st.completed++;
      }
      free_slot->reqs.clear();
      free_slot->busy = false;
      cv_done.notify_all();
    }
    return true;
  }

  void loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      reap();
      bool did = admit();
      if (did) continue;
      bool any_busy = false;
      for (auto& sp : slots) any_busy |= sp->busy;
      if (any_busy)
        cv_work.wait_for(lk, std::chrono::microseconds(50));
      else
        cv_work.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
};

extern "C" {

int owm_server_create(int device, const owm_server_cfg* cfg, owm_server** out) {
  if (!cfg || !out || cfg->hbm_budget_bytes <= 0 || cfg->max_tiles_per_batch <= 0 ||
      cfg->max_inflight_batches <= 0 || cfg->max_inflight_batches > 16 || cfg->max_points_per_batch <= 0)
    return OWM_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return OWM_ECUDA;
  }
  owm_server* s = new owm_server();
  s->cfg = *cfg;
  s->device = device;
  for (int k = 0; k < cfg->max_inflight_batches; ++k) {
    auto sl = std::make_unique<Slot>();
    if (sl->run.init(device, nullptr) != OWM_OK) {
      for (auto& q : s->slots) q->run.destroy();
      sl->run.destroy();
      delete s;
      return OWM_ECUDA;
    }
    sl->run.use_graphs = cfg->use_graphs != 0;
    s->slots.push_back(std::move(sl));
  }
  s->worker = std::thread([s] { s->loop(); });
  *out = s;
  return OWM_OK;
}

int owm_server_destroy(owm_server* s) {
  if (!s) return OWM_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& sl : s->slots) sl->run.destroy();
  for (auto& kv : s->reqs) {
    if (kv.second->pts) s->pinned.put(kv.second->pts, kv.second->pts_cls);
    delete kv.second;
  }
  delete s;
  return OWM_OK;
}

int owm_server_submit(owm_server* s, const owm_tile_desc* tile, int64_t* ticket) {
  if (!s || !tile || !ticket || !tile->xyz || tile->n <= 0 || tile->n >= 0x7FFFFFFFLL) return OWM_EINVAL;
  if (validate_tree_cfg(&tile->cfg.tree) != OWM_OK || tile->cfg.tree.policy != OWM_TREE_MAX_NUMBER)
    return OWM_EINVAL;
  Request* r = new Request();
  r->desc = *tile;
  if (!(r->desc.bbox.min_x <= r->desc.bbox.max_x)) {
    if (is_device_ptr(tile->xyz)) {
      delete r;
      return OWM_EINVAL;  // device tiles must carry their bbox
    }
    owm_bbox_of(tile->xyz, tile->n, &r->desc.bbox);
  }
  owm_params p;
  if (owm_params_compute(&r->desc.bbox, tile->n, tile->cfg.wsize, tile->cfg.overlap, tile->cfg.bsize, &p) != OWM_OK) {
    delete r;
    return OWM_EINVAL;
  }
  r->est_bytes = BatchRun::estimate_bytes(&r->desc, 1);
  if (r->est_bytes == (size_t)-1) {
    delete r;
    return OWM_EINVAL;
  }
  if (r->est_bytes > (size_t)s->cfg.hbm_budget_bytes) {
    delete r;
    return OWM_ENOMEM;  // this tile alone exceeds the budget
  }
  size_t bytes = (size_t)tile->n * 24;
  if (!s->cfg.copy_on_submit) {
    r->pts = nullptr;  // borrowed: the caller keeps tile->xyz alive until the result is taken
  } else if (!(r->pts = static_cast<double*>(s->pinned.get(bytes, &r->pts_cls)))) {
    delete r;
    return OWM_ENOMEM;
  } else if (is_device_ptr(tile->xyz)) {
    if (cudaMemcpy(r->pts, tile->xyz, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
      cudaGetLastError();
      s->pinned.put(r->pts, r->pts_cls);
      delete r;
      return OWM_ECUDA;
    }
  } else {
    std::memcpy(r->pts, tile->xyz, bytes);
  }
  if (r->pts) r->desc.xyz = r->pts;
  r->t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    s->reqs[r->ticket] = r;
    s->pending.push_back(r);
    s->st.submitted++;
  }
  s->cv_work.notify_all();
  *ticket = r->ticket;
  return OWM_OK;
}

static int take_result(owm_server* s, Request* r, int64_t* seeds, int64_t cap, int64_t* n_seeds, double* lat) {
  int rc = r->status;
  int64_t n = (int64_t)r->seeds.size();
  if (n_seeds) *n_seeds = n;
  if (lat) *lat = r->t_done - r->t_submit;
  if (rc == OWM_OK && n > cap) return OWM_ERANGE;  // keep the result for a retry with more room
  if (rc == OWM_OK && n > 0) std::memcpy(seeds, r->seeds.data(), (size_t)n * 8);
  s->reqs.erase(r->ticket);
  delete r;
  return rc;
}

int owm_server_poll(owm_server* s, int64_t ticket, int64_t* seeds, int64_t cap, int64_t* n_seeds, double* latency_ms) {
  if (!s || (!seeds && cap > 0)) return OWM_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return OWM_EINVAL;
  if (it->second->status == OWM_EAGAIN) return OWM_EAGAIN;
  return take_result(s, it->second, seeds, cap, n_seeds, latency_ms);
}

int owm_server_wait(owm_server* s, int64_t ticket, int64_t* seeds, int64_t cap, int64_t* n_seeds, double* latency_ms,
                    double timeout_ms) {
  if (!s || (!seeds && cap > 0)) return OWM_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds((int64_t)(timeout_ms * 1000.0));
  for (;;) {
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return OWM_EINVAL;
    if (it->second->status != OWM_EAGAIN) return take_result(s, it->second, seeds, cap, n_seeds, latency_ms);
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) {
      it = s->reqs.find(ticket);
      if (it != s->reqs.end() && it->second->status != OWM_EAGAIN)
        return take_result(s, it->second, seeds, cap, n_seeds, latency_ms);
      return OWM_ETIMEOUT;
    }
  }
}

int owm_server_get_stats(owm_server* s, owm_server_stats* out) {
  if (!s || !out) return OWM_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  s->st.bytes_in_use = (int64_t)s->slot_bytes();
  *out = s->st;
  return OWM_OK;
}

}  // extern "C"
