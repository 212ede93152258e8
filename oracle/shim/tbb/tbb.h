// Minimal stand-in for the subset of oneTBB that the OWM reference's CPU
// path uses, so that the reference sources compile unmodified where TBB is
// not installed.  TEST INFRASTRUCTURE ONLY: it schedules work and nothing
// else; it carries no arithmetic of the algorithm.
//
// Names provided (exactly those used by CPP-TBB-CPU/src/optim3_func.cpp and
// CPP-TBB-CPU/include/optim3_func.hpp, plus the reference application's global_control and
// tick_count):
//   blocked_range<T>, blocked_range2d<R,C>, parallel_for (range form and
//   index-step form), parallel_reduce (functional form, 2-D range),
//   task_group, concurrent_vector (push_back + iteration), tick_count,
//   global_control.
//
// Scheduling: ranges are cut into contiguous chunks that std::threads pull
// from a shared atomic counter.  global_control::max_allowed_parallelism sets
// the thread count; with 1 thread every call runs serially in index order, so
// the reference's outputs are then byte-for-byte reproducible.
#ifndef OWM_ORACLE_TBB_SHIM_H
#define OWM_ORACLE_TBB_SHIM_H

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

namespace tbb {

namespace shim_detail {
inline std::atomic<int>& max_threads() {
  static std::atomic<int> n{(int)std::max(1u, std::thread::hardware_concurrency())};
  return n;
}

// Runs body(chunk) for chunk in [0, nchunks) on up to max_threads() threads.
template <class F>
void run_chunks(long nchunks, F&& body) {
  int nt = (int)std::min<long>(max_threads().load(), nchunks);
  if (nt <= 1) {
    for (long c = 0; c < nchunks; ++c) body(c);
    return;
  }
  std::atomic<long> next{0};
  auto worker = [&]() {
    for (;;) {
      long c = next.fetch_add(1);
      if (c >= nchunks) break;
      body(c);
    }
  };
  std::vector<std::thread> ts;
  ts.reserve(nt - 1);
  for (int t = 1; t < nt; ++t) ts.emplace_back(worker);
  worker();
  for (auto& t : ts) t.join();
}

inline long chunk_count(long n) {
  long nt = max_threads().load();
  long want = nt <= 1 ? 1 : nt * 8;
  return std::max(1L, std::min(n, want));
}
}  // namespace shim_detail

template <class T>
class blocked_range {
 public:
  blocked_range(T b, T e, size_t grain = 1) : b_(b), e_(e), grain_(grain) {}
  T begin() const { return b_; }
  T end() const { return e_; }
  size_t size() const { return (size_t)(e_ - b_); }
  bool empty() const { return !(b_ < e_); }
  size_t grainsize() const { return grain_; }

 private:
  T b_, e_;
  size_t grain_;
};

template <class R, class C = R>
class blocked_range2d {
 public:
  blocked_range2d(R r0, R r1, C c0, C c1) : rows_(r0, r1), cols_(c0, c1) {}
  const blocked_range<R>& rows() const { return rows_; }
  const blocked_range<C>& cols() const { return cols_; }

 private:
  blocked_range<R> rows_;
  blocked_range<C> cols_;
};

// Range form: body(blocked_range<T>) over contiguous sub-ranges.
template <class T, class Body>
void parallel_for(const blocked_range<T>& r, const Body& body) {
  long n = (long)(r.end() - r.begin());
  if (n <= 0) return;
  long nc = shim_detail::chunk_count(n);
  shim_detail::run_chunks(nc, [&](long c) {
    T b = r.begin() + (T)(n * c / nc);
    T e = r.begin() + (T)(n * (c + 1) / nc);
    if (b < e) body(blocked_range<T>(b, e));
  });
}

// 2-D range form: split along rows.
template <class R, class C, class Body>
void parallel_for(const blocked_range2d<R, C>& r, const Body& body) {
  long n = (long)(r.rows().end() - r.rows().begin());
  if (n <= 0) return;
  long nc = shim_detail::chunk_count(n);
  shim_detail::run_chunks(nc, [&](long c) {
    R b = r.rows().begin() + (R)(n * c / nc);
    R e = r.rows().begin() + (R)(n * (c + 1) / nc);
    if (b < e) body(blocked_range2d<R, C>(b, e, r.cols().begin(), r.cols().end()));
  });
}

// Index-step form: f(i) for i = first, first+step, ... < last.
template <class Index, class Func>
void parallel_for(Index first, Index last, Index step, const Func& f) {
  if (!(first < last) || step <= 0) return;
  long n = (long)((last - first + step - 1) / step);
  long nc = shim_detail::chunk_count(n);
  shim_detail::run_chunks(nc, [&](long c) {
    long b = n * c / nc, e = n * (c + 1) / nc;
    for (long k = b; k < e; ++k) f((Index)(first + k * step));
  });
}

// Functional reduce over a 2-D range, split along rows; partial results are
// joined in row order.
template <class R, class C, class Value, class RealBody, class Reduction>
Value parallel_reduce(const blocked_range2d<R, C>& r, const Value& identity,
                      const RealBody& body, const Reduction& join) {
  long n = (long)(r.rows().end() - r.rows().begin());
  if (n <= 0) return identity;
  long nc = shim_detail::chunk_count(n);
  std::vector<Value> parts((size_t)nc, identity);
  shim_detail::run_chunks(nc, [&](long c) {
    R b = r.rows().begin() + (R)(n * c / nc);
    R e = r.rows().begin() + (R)(n * (c + 1) / nc);
    if (b < e)
      parts[(size_t)c] = body(blocked_range2d<R, C>(b, e, r.cols().begin(), r.cols().end()), identity);
  });
  Value acc = identity;
  for (auto& p : parts) acc = join(acc, p);
  return acc;
}

template <class T, class Value, class RealBody, class Reduction>
Value parallel_reduce(const blocked_range<T>& r, const Value& identity,
                      const RealBody& body, const Reduction& join) {
  long n = (long)(r.end() - r.begin());
  if (n <= 0) return identity;
  long nc = shim_detail::chunk_count(n);
  std::vector<Value> parts((size_t)nc, identity);
  shim_detail::run_chunks(nc, [&](long c) {
    T b = r.begin() + (T)(n * c / nc);
    T e = r.begin() + (T)(n * (c + 1) / nc);
    if (b < e) parts[(size_t)c] = body(blocked_range<T>(b, e), identity);
  });
  Value acc = identity;
  for (auto& p : parts) acc = join(acc, p);
  return acc;
}

// task_group: each run() gets its own thread when more than one thread is
// allowed, otherwise it runs inline.
class task_group {
 public:
  ~task_group() { wait(); }
  template <class F>
  void run(F&& f) {
    if (shim_detail::max_threads().load() <= 1) {
      f();
      return;
    }
    ts_.emplace_back(std::forward<F>(f));
  }
  void wait() {
    for (auto& t : ts_) t.join();
    ts_.clear();
  }

 private:
  std::vector<std::thread> ts_;
};

// Growable vector with thread-safe push_back.  Storage is a list of
// segments of doubling size (8, 16, 32, ...), so existing elements never
// move; the slot index is reserved with one atomic add.  Iteration is only
// valid once all pushes have finished (which is how the reference uses it).
template <class T>
class concurrent_vector {
  static constexpr int kSegs = 48;
  static constexpr size_t kFirst = 8;

 public:
  concurrent_vector() : n_(0) {
    for (auto& s : segs_) s.store(nullptr);
  }
  ~concurrent_vector() { clear(); }
  concurrent_vector(const concurrent_vector&) = delete;
  concurrent_vector& operator=(const concurrent_vector&) = delete;

  void push_back(const T& v) {
    size_t k = n_.fetch_add(1);
    int s;
    size_t off;
    locate(k, s, off);
    T* seg = segs_[s].load(std::memory_order_acquire);
    if (!seg) {
      T* fresh = new T[kFirst << s];
      if (segs_[s].compare_exchange_strong(seg, fresh, std::memory_order_acq_rel)) {
        seg = fresh;
      } else {
        delete[] fresh;  // another thread installed it; seg now holds theirs
      }
    }
    seg[off] = v;
  }
  size_t size() const { return n_.load(); }
  bool empty() const { return size() == 0; }
  void clear() {
    for (auto& s : segs_) {
      delete[] s.load();
      s.store(nullptr);
    }
    n_.store(0);
  }
  T& operator[](size_t k) {
    int s;
    size_t off;
    locate(k, s, off);
    return segs_[s].load()[off];
  }
  const T& operator[](size_t k) const { return const_cast<concurrent_vector*>(this)->operator[](k); }

  class const_iterator {
   public:
    const_iterator(const concurrent_vector* v, size_t k) : v_(v), k_(k) {}
    const T& operator*() const { return (*v_)[k_]; }
    const_iterator& operator++() {
      ++k_;
      return *this;
    }
    bool operator!=(const const_iterator& o) const { return k_ != o.k_; }
    bool operator==(const const_iterator& o) const { return k_ == o.k_; }

   private:
    const concurrent_vector* v_;
    size_t k_;
  };
  const_iterator begin() const { return const_iterator(this, 0); }
  const_iterator end() const { return const_iterator(this, size()); }

 private:
  static void locate(size_t k, int& s, size_t& off) {
    // segment s holds indices [kFirst*(2^s - 1), kFirst*(2^(s+1) - 1))
    size_t q = k / kFirst + 1;
    s = 63 - __builtin_clzll((unsigned long long)q);
    off = k - kFirst * ((size_t(1) << s) - 1);
  }
  std::atomic<size_t> n_;
  std::atomic<T*> segs_[kSegs];
};

class tick_count {
 public:
  class interval_t {
   public:
    explicit interval_t(double s = 0) : s_(s) {}
    double seconds() const { return s_; }

   private:
    double s_;
  };
  static tick_count now() {
    tick_count t;
    t.t_ = std::chrono::steady_clock::now();
    return t;
  }
  interval_t operator-(const tick_count& o) const {
    return interval_t(std::chrono::duration<double>(t_ - o.t_).count());
  }

 private:
  std::chrono::steady_clock::time_point t_;
};

class global_control {
 public:
  enum parameter { max_allowed_parallelism, thread_stack_size };
  global_control(parameter p, size_t v) : p_(p) {
    if (p_ == max_allowed_parallelism) {
      prev_ = shim_detail::max_threads().load();
      shim_detail::max_threads().store((int)std::max<size_t>(1, v));
    }
  }
  ~global_control() {
    if (p_ == max_allowed_parallelism) shim_detail::max_threads().store(prev_);
  }

 private:
  parameter p_;
  int prev_ = 1;
};

}  // namespace tbb

#endif
