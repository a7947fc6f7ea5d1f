/* Minimal std::thread stand-in for the parts of Intel TBB 2.2 that the
 * reference's VortonSim path uses (parallel_for / parallel_reduce over a
 * blocked_range, atomic<T>, tick_count, task_scheduler_init, parallel_invoke,
 * parallel_do).  TEST INFRASTRUCTURE ONLY: it lets the reference's own
 * USE_TBB=1 code run on all host cores as the CPU baseline.
 *
 * Scheduling: a persistent pool of (NUMBER_OF_PROCESSORS - 1) workers plus the
 * calling thread pull equal chunks of the range from an atomic counter.
 * parallel_reduce joins partial bodies in chunk order, so results do not
 * depend on thread timing.
 */
#pragma once
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <cstdlib>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>
#include <deque>
#include <type_traits>

namespace tbb {

struct split {};

template <typename Value>
class blocked_range {
 public:
  typedef Value const_iterator;
  typedef std::size_t size_type;
  blocked_range() : b_(), e_(), g_(1) {}
  blocked_range(Value b, Value e, size_type g = 1) : b_(b), e_(e), g_(g ? g : 1) {}
  blocked_range(blocked_range& r, split) : b_(), e_(r.e_), g_(r.g_) {
    Value mid = r.b_ + (r.e_ - r.b_) / 2;
    b_ = mid;
    r.e_ = mid;
  }
  Value begin() const { return b_; }
  Value end() const { return e_; }
  size_type size() const { return size_type(e_ - b_); }
  size_type grainsize() const { return g_; }
  bool empty() const { return !(b_ < e_); }
  bool is_divisible() const { return g_ < size(); }

 private:
  Value b_, e_;
  size_type g_;
};

namespace vgshim {

inline unsigned num_threads() {
  const char* s = std::getenv("NUMBER_OF_PROCESSORS");
  int n = s ? std::atoi(s) : 0;
  if (n <= 0) n = (int)std::thread::hardware_concurrency();
  return n > 0 ? (unsigned)n : 1u;
}

/* Persistent worker pool.  run(n, fn) calls fn(i) for i in [0, n) across the
 * pool and the caller, returning when every call has finished. */
class Pool {
 public:
  static Pool& get() {
    static Pool p;
    return p;
  }
  void run(std::size_t n, const std::function<void(std::size_t)>& fn) {
    if (n == 0) return;
    if (workers_.empty() || n == 1) {
      for (std::size_t i = 0; i < n; ++i) fn(i);
      return;
    }
    std::unique_lock<std::mutex> lk(run_mu_);  // one parallel region at a time
    {
      std::lock_guard<std::mutex> g(mu_);
      fn_ = &fn;
      n_ = n;
      next_.store(0);
      done_.store(0);
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> g(mu_);
    done_cv_.wait(g, [&] { return done_.load() == n_ && active_ == 0; });
    fn_ = nullptr;
  }

 private:
  Pool() {
    unsigned t = num_threads();
    for (unsigned i = 1; i < t; ++i) workers_.emplace_back([this] { loop(); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }
  void work() {
    for (;;) {
      std::size_t i = next_.fetch_add(1);
      if (i >= n_) break;
      (*fn_)(i);
      if (done_.fetch_add(1) + 1 == n_) {
        std::lock_guard<std::mutex> g(mu_);
        done_cv_.notify_all();
      }
    }
  }
  void loop() {
    unsigned long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        if (!fn_) continue;
        ++active_;
      }
      work();
      {
        std::lock_guard<std::mutex> g(mu_);
        --active_;
      }
      done_cv_.notify_all();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_, run_mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(std::size_t)>* fn_ = nullptr;
  std::size_t n_ = 0;
  std::atomic<std::size_t> next_{0}, done_{0};
  unsigned long gen_ = 0;
  unsigned active_ = 0;  // workers inside work() for the current region
  bool stop_ = false;
};

/* Split [b, e) into chunks no smaller than the grain, at most 4 per thread. */
template <typename Range>
std::vector<Range> chunks(const Range& r) {
  std::vector<Range> out;
  std::size_t n = r.size();
  if (n == 0) return out;
  std::size_t g = r.grainsize() ? r.grainsize() : 1;
  std::size_t maxc = 4 * (std::size_t)num_threads();
  std::size_t nc = (n + g - 1) / g;
  if (nc > maxc) nc = maxc;
  if (nc < 1) nc = 1;
  typedef decltype(r.begin()) V;
  for (std::size_t c = 0; c < nc; ++c) {
    V b = r.begin() + (V)(n * c / nc);
    V e = r.begin() + (V)(n * (c + 1) / nc);
    out.push_back(Range(b, e, g));
  }
  return out;
}

}  // namespace vgshim

template <typename Range, typename Body>
void parallel_for(const Range& range, const Body& body) {
  std::vector<Range> cs = vgshim::chunks(range);
  vgshim::Pool::get().run(cs.size(), [&](std::size_t i) { body(cs[i]); });
}

template <typename Range, typename Body>
void parallel_reduce(const Range& range, Body& body) {
  std::vector<Range> cs = vgshim::chunks(range);
  if (cs.empty()) return;
  std::vector<Body*> parts(cs.size(), nullptr);
  parts[0] = &body;
  for (std::size_t i = 1; i < cs.size(); ++i) parts[i] = new Body(body, split());
  vgshim::Pool::get().run(cs.size(), [&](std::size_t i) { (*parts[i])(cs[i]); });
  for (std::size_t i = 1; i < cs.size(); ++i) {
    body.join(*parts[i]);
    delete parts[i];
  }
}

template <typename F0, typename F1>
void parallel_invoke(const F0& f0, const F1& f1) { f0(); f1(); }
template <typename F0, typename F1, typename F2>
void parallel_invoke(const F0& f0, const F1& f1, const F2& f2) { f0(); f1(); f2(); }

template <typename Item>
class parallel_do_feeder {
 public:
  explicit parallel_do_feeder(std::deque<Item>& q) : q_(q) {}
  void add(const Item& it) { q_.push_back(it); }
 private:
  std::deque<Item>& q_;
};

/* Sequential work-list stand-in: the reference only uses it in particle
 * emission, which is not on the timed path. */
template <typename Iterator, typename Body>
void parallel_do(Iterator first, Iterator last, const Body& body) {
  typedef typename std::remove_cv<typename std::remove_reference<decltype(*first)>::type>::type Item;
  std::deque<Item> q;
  for (; first != last; ++first) q.push_back(*first);
  parallel_do_feeder<Item> feeder(q);
  while (!q.empty()) {
    Item it = q.front();
    q.pop_front();
    body(it, feeder);
  }
}

template <typename T>
struct atomic {
  T v;
  operator T() const { T r; __atomic_load(const_cast<T*>(&v), &r, __ATOMIC_SEQ_CST); return r; }
  atomic& operator=(T x) { __atomic_store(&v, &x, __ATOMIC_SEQ_CST); return *this; }
  T compare_and_swap(T value, T comparand) {
    T expected = comparand;
    __atomic_compare_exchange(&v, &expected, &value, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return expected;
  }
  T fetch_and_store(T value) {
    T old;
    __atomic_exchange(&v, &value, &old, __ATOMIC_SEQ_CST);
    return old;
  }
  T fetch_and_add(T d) { return __atomic_fetch_add(&v, d, __ATOMIC_SEQ_CST); }
  T operator++() { return fetch_and_add(1) + 1; }
  T operator--() { return fetch_and_add(T(-1)) - 1; }
  T operator++(int) { return fetch_and_add(1); }
  T operator--(int) { return fetch_and_add(T(-1)); }
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

class task_scheduler_init {
 public:
  static const int automatic = -1;
  static const int deferred = -2;
  explicit task_scheduler_init(int = automatic) {}
  void initialize(int = automatic) {}
  void terminate() {}
  static int default_num_threads() { return (int)vgshim::num_threads(); }
};

}  // namespace tbb
