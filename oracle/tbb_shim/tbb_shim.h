// Oracle-only stand-in for the subset of oneTBB (pinned 2021.5.0 by the
// reference's superbuild) that Open PGL v0.6.0 and its vendored Embree
// helpers include.  It exists so that the reference library can be compiled
// from its own sources, unmodified, to pin the CPU restatement in oracle/.
// TBB only schedules work in the reference; none of the path's arithmetic is
// in TBB.  This header is test infrastructure and never part of the product.
//
// Two modes, chosen by tbb::global_control(max_allowed_parallelism, n):
//   n == 1 : every construct runs inline on the calling thread, in program
//            order (deterministic region numbering: depth-first, left first).
//   n  > 1 : a fork-join pool of n-1 worker threads plus the caller; a thread
//            that waits for its children executes queued tasks meanwhile, so
//            nested parallel_invoke / parallel_for cannot deadlock.
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <deque>
#include <functional>
#include <iterator>
#include <mutex>
#include <new>
#include <thread>
#include <utility>
#include <vector>

#define TBB_INTERFACE_VERSION 12050
#define TBB_INTERFACE_VERSION_MAJOR 12
#define TBB_VERSION_MAJOR 2021
#define TBB_VERSION_MINOR 5

namespace tbb {

namespace shim {

// ---------------------------------------------------------------- thread pool
class Pool {
 public:
  static Pool &get() {
    static Pool p;
    return p;
  }

  int threads() const { return m_threads; }

  void set_threads(int n) {
    std::unique_lock<std::mutex> lk(m_mutex);
    if (n < 1) n = 1;
    if (n == m_threads) return;
    stop_locked(lk);
    m_threads = n;
    m_stop = false;
    for (int i = 1; i < n; ++i) m_workers.emplace_back([this, i] { worker(i); });
  }

  struct Group {
    std::atomic<int> pending{0};
  };

  void spawn(Group &g, std::function<void()> fn) {
    g.pending.fetch_add(1);
    {
      std::lock_guard<std::mutex> lk(m_mutex);
      m_queue.emplace_back(Task{&g, std::move(fn)});
    }
    m_cv.notify_one();
  }

  void wait(Group &g) {
    while (g.pending.load() > 0) {
      Task t;
      bool have = false;
      {
        std::lock_guard<std::mutex> lk(m_mutex);
        if (!m_queue.empty()) {
          t = std::move(m_queue.back());  // newest first: depth-first help
          m_queue.pop_back();
          have = true;
        }
      }
      if (have)
        run(t);
      else
        std::this_thread::yield();
    }
  }

  static int &thread_index() {
    static thread_local int idx = 0;
    return idx;
  }

  ~Pool() {
    std::unique_lock<std::mutex> lk(m_mutex);
    stop_locked(lk);
  }

 private:
  struct Task {
    Task() = default;
    Task(Group *grp, std::function<void()> f) : g(grp), fn(std::move(f)) {}
    Group *g = nullptr;
    std::function<void()> fn;
  };

  Pool() {
    const char *env = std::getenv("PGL_ORACLE_THREADS");
    int n = env ? std::atoi(env) : 1;
    std::unique_lock<std::mutex> lk(m_mutex);
    m_threads = n < 1 ? 1 : n;
    for (int i = 1; i < m_threads; ++i) m_workers.emplace_back([this, i] { worker(i); });
  }

  void stop_locked(std::unique_lock<std::mutex> &lk) {
    m_stop = true;
    lk.unlock();
    m_cv.notify_all();
    for (auto &w : m_workers) w.join();
    m_workers.clear();
    lk.lock();
  }

  void run(Task &t) {
    t.fn();
    t.g->pending.fetch_sub(1);
  }

  void worker(int idx) {
    thread_index() = idx;
    for (;;) {
      Task t;
      {
        std::unique_lock<std::mutex> lk(m_mutex);
        m_cv.wait(lk, [this] { return m_stop || !m_queue.empty(); });
        if (m_stop && m_queue.empty()) return;
        t = std::move(m_queue.front());  // oldest first: breadth for thieves
        m_queue.pop_front();
      }
      run(t);
    }
  }

  int m_threads = 1;
  bool m_stop = false;
  std::mutex m_mutex;
  std::condition_variable m_cv;
  std::deque<Task> m_queue;
  std::vector<std::thread> m_workers;
};

inline bool serial() { return Pool::get().threads() <= 1; }

}  // namespace shim

// ---------------------------------------------------------------- controls
class global_control {
 public:
  enum parameter { max_allowed_parallelism, thread_stack_size };
  global_control(parameter p, size_t value) : m_p(p) {
    if (p == max_allowed_parallelism) {
      m_prev = shim::Pool::get().threads();
      shim::Pool::get().set_threads((int)value);
    }
  }
  ~global_control() {
    if (m_p == max_allowed_parallelism) shim::Pool::get().set_threads(m_prev);
  }
  static size_t active_value(parameter p) {
    return p == max_allowed_parallelism ? (size_t)shim::Pool::get().threads() : 0;
  }

 private:
  parameter m_p;
  int m_prev = 1;
};

namespace this_task_arena {
inline int max_concurrency() {
  const char *env = std::getenv("PGL_ORACLE_THREADS");
  if (env) return std::max(1, std::atoi(env));
  unsigned hc = std::thread::hardware_concurrency();
  return hc ? (int)hc : 1;
}
inline int current_thread_index() { return shim::Pool::thread_index(); }
}  // namespace this_task_arena

class task_scheduler_init {
 public:
  enum { automatic = -1, deferred = -2 };
  explicit task_scheduler_init(int = automatic) {}
  void initialize(int n) { shim::Pool::get().set_threads(n); }
  void terminate() {}
  static int default_num_threads() { return this_task_arena::max_concurrency(); }
};

class task_group_context {
 public:
  task_group_context() = default;
  bool is_group_execution_cancelled() const { return false; }
};

class task_scheduler_observer {
 public:
  virtual ~task_scheduler_observer() = default;
  void observe(bool = true) {}
  virtual void on_scheduler_entry(bool) {}
  virtual void on_scheduler_exit(bool) {}
};

struct simple_partitioner {};
struct auto_partitioner {};
struct static_partitioner {};
struct affinity_partitioner {};

// ---------------------------------------------------------------- ranges
template <typename Value>
class blocked_range {
 public:
  typedef Value const_iterator;
  typedef size_t size_type;
  blocked_range() = default;
  blocked_range(Value b, Value e, size_t grain = 1) : m_begin(b), m_end(e), m_grain(grain ? grain : 1) {}
  Value begin() const { return m_begin; }
  Value end() const { return m_end; }
  size_t size() const { return size_t(m_end - m_begin); }
  size_t grainsize() const { return m_grain; }
  bool empty() const { return !(m_begin < m_end); }
  bool is_divisible() const { return m_grain < size(); }

 private:
  Value m_begin{}, m_end{};
  size_t m_grain = 1;
};

namespace shim {
// Splits [b, e) into at most 4*threads chunks no smaller than the grain and
// runs body on each; the caller participates.
template <typename Value, typename Body>
void for_chunks(Value b, Value e, size_t grain, const Body &body) {
  const size_t n = size_t(e - b);
  if (n == 0) return;
  if (serial()) {
    body(blocked_range<Value>(b, e, grain));
    return;
  }
  const size_t threads = (size_t)Pool::get().threads();
  size_t chunks = std::min(n / std::max<size_t>(grain, 1), threads * 4);
  if (chunks < 1) chunks = 1;
  const size_t step = (n + chunks - 1) / chunks;
  Pool::Group g;
  for (size_t c = 1; c < chunks; ++c) {
    Value cb = Value(b + c * step);
    if (!(cb < e)) break;
    Value ce = Value(std::min<size_t>(n, (c + 1) * step) + b);
    Pool::get().spawn(g, [=, &body] { body(blocked_range<Value>(cb, ce, grain)); });
  }
  body(blocked_range<Value>(b, Value(b + std::min(step, n)), grain));
  Pool::get().wait(g);
}
}  // namespace shim

// ---------------------------------------------------------------- parallel_for
template <typename Value, typename Body>
void parallel_for(const blocked_range<Value> &r, const Body &body) {
  shim::for_chunks(r.begin(), r.end(), r.grainsize(), body);
}
template <typename Value, typename Body, typename P>
void parallel_for(const blocked_range<Value> &r, const Body &body, P &&) {
  shim::for_chunks(r.begin(), r.end(), r.grainsize(), body);
}
template <typename Value, typename Body, typename P>
void parallel_for(const blocked_range<Value> &r, const Body &body, P &&, task_group_context &) {
  shim::for_chunks(r.begin(), r.end(), r.grainsize(), body);
}
template <typename Index, typename Func>
void parallel_for(Index first, Index last, Index step, const Func &f) {
  shim::for_chunks(first, last, 1, [&](const blocked_range<Index> &r) {
    for (Index i = r.begin(); i < r.end(); ++i)
      if (((i - first) % step) == 0) f(i);
  });
}
template <typename Index, typename Func>
void parallel_for(Index first, Index last, Index step, const Func &f, const simple_partitioner &) {
  ::tbb::parallel_for(first, last, step, f);
}
template <typename Index, typename Func>
void parallel_for(Index first, Index last, Index step, const Func &f, affinity_partitioner &) {
  ::tbb::parallel_for(first, last, step, f);
}
template <typename Index, typename Func, typename P>
void parallel_for(Index first, Index last, Index step, const Func &f, P &&, task_group_context &) {
  ::tbb::parallel_for(first, last, step, f);
}
template <typename Index, typename Func>
void parallel_for(Index first, Index last, Index step, const Func &f, task_group_context &) {
  ::tbb::parallel_for(first, last, step, f);
}

// ---------------------------------------------------------------- reduce
template <typename Value, typename T, typename Func, typename Red>
T parallel_reduce(const blocked_range<Value> &r, const T &identity, const Func &func, const Red &red) {
  if (shim::serial()) return func(r, identity);
  std::mutex m;
  std::vector<std::pair<size_t, T>> parts;
  shim::for_chunks(r.begin(), r.end(), r.grainsize(), [&](const blocked_range<Value> &sub) {
    T v = func(sub, identity);
    std::lock_guard<std::mutex> lk(m);
    parts.emplace_back(size_t(sub.begin() - r.begin()), v);
  });
  std::sort(parts.begin(), parts.end(),
            [](const std::pair<size_t, T> &a, const std::pair<size_t, T> &b) { return a.first < b.first; });
  T acc = identity;
  for (auto &p : parts) acc = red(acc, p.second);
  return acc;
}
template <typename Value, typename T, typename Func, typename Red>
T parallel_reduce(const blocked_range<Value> &r, const T &identity, const Func &func, const Red &red, task_group_context &) {
  return ::tbb::parallel_reduce(r, identity, func, red);
}

// ---------------------------------------------------------------- invoke
template <typename F0, typename F1>
void parallel_invoke(const F0 &f0, const F1 &f1) {
  if (shim::serial()) {
    f0();
    f1();
    return;
  }
  shim::Pool::Group g;
  shim::Pool::get().spawn(g, [&f1] { f1(); });
  f0();
  shim::Pool::get().wait(g);
}
template <typename F0, typename F1, typename F2>
void parallel_invoke(const F0 &f0, const F1 &f1, const F2 &f2) {
  ::tbb::parallel_invoke(f0, [&] { ::tbb::parallel_invoke(f1, f2); });
}

// ---------------------------------------------------------------- sort
template <typename It, typename Cmp>
void parallel_sort(It b, It e, const Cmp &cmp) {
  std::sort(b, e, cmp);
}
template <typename It>
void parallel_sort(It b, It e) {
  std::sort(b, e);
}

// ---------------------------------------------------------------- concurrent_vector
// Segmented storage: element addresses never move when the vector grows, as
// with oneTBB (the reference keeps references to nodes across growth).  Every
// segment is 64-byte aligned (the AVX2 code paths use aligned loads).
template <typename T>
class concurrent_vector {
  static constexpr size_t kFirst = 64;  // segment k holds kFirst << k elements
  static constexpr int kMaxSeg = 40;

  static int seg_of(size_t i, size_t &offset) {
    size_t q = i / kFirst + 1;
    int k = 63 - __builtin_clzll((unsigned long long)q);
    offset = i - kFirst * ((size_t(1) << k) - 1);
    return k;
  }

 public:
  typedef T value_type;
  typedef size_t size_type;
  typedef T &reference;
  typedef const T &const_reference;

  template <typename V, typename Owner>
  class iter {
   public:
    typedef std::random_access_iterator_tag iterator_category;
    typedef typename std::remove_const<V>::type value_type;
    typedef std::ptrdiff_t difference_type;
    typedef V *pointer;
    typedef V &reference;
    iter() = default;
    iter(Owner *o, size_t i) : m_o(o), m_i(i) {}
    template <typename V2, typename O2>
    iter(const iter<V2, O2> &o) : m_o(o.m_o), m_i(o.m_i) {}
    V &operator*() const { return (*m_o)[m_i]; }
    V *operator->() const { return &(*m_o)[m_i]; }
    V &operator[](difference_type d) const { return (*m_o)[m_i + d]; }
    iter &operator++() { ++m_i; return *this; }
    iter operator++(int) { iter t = *this; ++m_i; return t; }
    iter &operator--() { --m_i; return *this; }
    iter operator--(int) { iter t = *this; --m_i; return t; }
    iter &operator+=(difference_type d) { m_i += d; return *this; }
    iter &operator-=(difference_type d) { m_i -= d; return *this; }
    iter operator+(difference_type d) const { return iter(m_o, m_i + d); }
    iter operator-(difference_type d) const { return iter(m_o, m_i - d); }
    difference_type operator-(const iter &o) const { return difference_type(m_i) - difference_type(o.m_i); }
    bool operator==(const iter &o) const { return m_i == o.m_i; }
    bool operator!=(const iter &o) const { return m_i != o.m_i; }
    bool operator<(const iter &o) const { return m_i < o.m_i; }
    bool operator>(const iter &o) const { return m_i > o.m_i; }
    bool operator<=(const iter &o) const { return m_i <= o.m_i; }
    bool operator>=(const iter &o) const { return m_i >= o.m_i; }
    Owner *m_o = nullptr;
    size_t m_i = 0;
  };
  typedef iter<T, concurrent_vector> iterator;
  typedef iter<const T, const concurrent_vector> const_iterator;

  concurrent_vector() { for (auto &s : m_seg) s = nullptr; }
  concurrent_vector(const concurrent_vector &o) : concurrent_vector() { *this = o; }
  concurrent_vector &operator=(const concurrent_vector &o) {
    if (this == &o) return *this;
    clear();
    reserve(o.size());
    for (size_t i = 0; i < o.size(); ++i) new (slot(i)) T(o[i]);
    m_size.store(o.size());
    return *this;
  }
  ~concurrent_vector() {
    clear();
    for (auto &s : m_seg)
      if (s) { std::free(s); s = nullptr; }
  }

  size_t size() const { return m_size.load(); }
  bool empty() const { return size() == 0; }
  size_t capacity() const {
    size_t c = 0;
    for (int k = 0; k < kMaxSeg && m_seg[k]; ++k) c += kFirst << k;
    return c;
  }
  T &operator[](size_t i) { return *slot(i); }
  const T &operator[](size_t i) const { return *const_cast<concurrent_vector *>(this)->slot(i); }
  T &at(size_t i) { return (*this)[i]; }
  const T &at(size_t i) const { return (*this)[i]; }
  T &back() { return (*this)[size() - 1]; }

  iterator begin() { return iterator(this, 0); }
  iterator end() { return iterator(this, size()); }
  const_iterator begin() const { return const_iterator(this, 0); }
  const_iterator end() const { return const_iterator(this, size()); }

  void reserve(size_t n) {
    if (n == 0) return;
    size_t off;
    int k = seg_of(n - 1, off);
    std::lock_guard<std::mutex> lk(m_mutex);
    for (int s = 0; s <= k; ++s) ensure_locked(s);
  }

  iterator push_back(const T &v) {
    size_t i = m_size.fetch_add(1);
    new (slot_alloc(i)) T(v);
    return iterator(this, i);
  }
  template <typename... A>
  iterator emplace_back(A &&...a) {
    size_t i = m_size.fetch_add(1);
    new (slot_alloc(i)) T(std::forward<A>(a)...);
    return iterator(this, i);
  }
  iterator grow_by(size_t n) {
    size_t i = m_size.fetch_add(n);
    for (size_t j = 0; j < n; ++j) new (slot_alloc(i + j)) T();
    return iterator(this, i);
  }
  void resize(size_t n) {
    size_t s = size();
    if (n > s) {
      for (size_t j = s; j < n; ++j) new (slot_alloc(j)) T();
    } else {
      for (size_t j = n; j < s; ++j) slot(j)->~T();
    }
    m_size.store(n);
  }
  void clear() {
    size_t s = size();
    for (size_t j = 0; j < s; ++j) slot(j)->~T();
    m_size.store(0);
  }
  void shrink_to_fit() {}

 private:
  T *slot(size_t i) {
    size_t off;
    int k = seg_of(i, off);
    return reinterpret_cast<T *>(m_seg[k]) + off;
  }
  T *slot_alloc(size_t i) {
    size_t off;
    int k = seg_of(i, off);
    if (!m_seg[k]) {
      std::lock_guard<std::mutex> lk(m_mutex);
      ensure_locked(k);
    }
    return reinterpret_cast<T *>(m_seg[k]) + off;
  }
  void ensure_locked(int k) {
    if (m_seg[k]) return;
    size_t bytes = sizeof(T) * (kFirst << k);
    bytes = (bytes + 63) / 64 * 64;
    void *p = nullptr;
    if (posix_memalign(&p, 64, bytes) != 0 || !p) throw std::bad_alloc();
    m_seg[k] = p;
  }

  void *volatile m_seg[kMaxSeg];
  std::atomic<size_t> m_size{0};
  std::mutex m_mutex;
};

}  // namespace tbb
