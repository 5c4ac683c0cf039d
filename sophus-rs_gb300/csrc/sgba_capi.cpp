// sgba_capi.cpp -- host driver and C ABI of libsgba (include/sgba.h).
//
// Planning (once per problem): sort the cost terms as CostFn::sort does,
// reduce equal (point, pose) terms, assign free / marginalized block indices,
// build per-camera term lists, the reduced-camera-system block list and the
// observation pairs summed into each block.  Per LM iteration the whole step
// (linearize, Schur complement, factor + refine, back-substitute, update,
// trial cost, accept/reject) is one CUDA graph; termination is decided on the
// device, so optimize() enqueues num_iterations graph launches and
// synchronizes once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <pthread.h>
#include <functional>
#include <condition_variable>
#include <atomic>
#include <chrono>
#include <utility>
#include <mutex>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sgba.h"
#include "sgba_internal.h"

using sgba::Ctrl;
using sgba::Dev;
using sgba::Plan;
using sgba::Record;
using sgba::Sizes;
using sgba::kIntrMax;
using sgba::kIntrPart;
using sgba::kIntrScj;
using sgba::kIntrSum;
using sgba::kIntrZk;

namespace sgba {

cudaError_t raise_dynamic_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> granted;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& g = granted[std::make_pair(func, dev)];
  if (bytes <= g) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
  if (e == cudaSuccess) g = bytes;
  return e;
}

}  // namespace sgba

namespace {

thread_local std::string g_last_error;

int set_error(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

// (a failed call's error is also cleared from the thread's last-error slot, so
// that a later launch check of another problem on this thread does not see it)
#define SGBA_CK(expr)                                                                           \
  do {                                                                                          \
    cudaError_t e_ = (expr);                                                                    \
    if (e_ != cudaSuccess) {                                                                    \
      (void)cudaGetLastError();                                                                 \
      return set_error(e_ == cudaErrorMemoryAllocation ? SGBA_ERR_OUT_OF_MEMORY : SGBA_ERR_CUDA, \
                       "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__);   \
    }                                                                                           \
  } while (0)

// The kernels compare residual norms with the Huber threshold in float: a
// positive threshold must be a normal float (a smaller one would round to 0
// and silently drop the robust kernel).
bool huber_in_float_range(double h) { return !(h > 0.0) || (h >= 1.17549435e-38 && h <= 3.40282347e38); }

// CUDA events owned by one call: destroyed when the call returns, on every path.
struct EventSet {
  std::vector<cudaEvent_t> ev;
  EventSet() = default;
  EventSet(const EventSet&) = delete;
  EventSet& operator=(const EventSet&) = delete;
  ~EventSet() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
  cudaError_t create(cudaEvent_t* out) {
    cudaEvent_t e = nullptr;
    const cudaError_t r = cudaEventCreate(&e);
    if (r == cudaSuccess) ev.push_back(e);
    *out = e;
    return r;
  }
};

constexpr int kTile = 256;           // terms per camera tile (one CTA)
constexpr int64_t kSchurChunk = 256;  // observation pairs per warp in the Schur assembly
constexpr int32_t kMaxDenseFree = 4096;  // reduced-camera-system limit (6 * 4096 rows, stored dense in f64)

}  // namespace

struct sgba_problem {
  Plan plan;
  std::vector<double> cnt_f_base;  // damping counts of the free poses without pose priors
  int gauge_base = -1;             // gauge kind without pose priors (-1: not saved yet)
  int intr_free = 0;  // the camera params are a Free family (sgba_problem_create_ex)
  int camera_model = SGBA_CAMERA_PINHOLE;
  double eucm_ab[2] = {0.0, 0.0};  // EUCM alpha beta
  Sizes sz{};
  Dev d;
  int device = 0;
  cudaStream_t stream = nullptr;
  sgba_opt_params params{};
  bool inited = false;
  bool defer_sync = false;  // batch: init without a host synchronisation
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int iter_launches = 0;
  // profile
  bool profiling = false;
  sgba_profile prof{};
  void* flush_buf = nullptr;  // L2 flush target for benchmark hooks
  std::vector<void*> allocs;
  // Device memory comes from a stream-ordered pool (problem_pool) on the
  // problem's stream. Small device buffers are carved from chunks (fewer
  // allocations at create and destroy); large ones get their own allocation.
  cudaMemPool_t pool = nullptr;
  char* chunk_ptr = nullptr;
  size_t chunk_left = 0;
  size_t chunk_size = size_t(1) << 20;
  // covariance of the solution (sgba_covariance_prepare)
  sgba::CovBufs cov;
  bool pairs_built = true;  // the Schur pair lists exist (not for the tiled pass of nearly dense systems)
};

namespace {

// One stream-ordered memory pool per device for all problems: allocations are
// cudaMallocFromPoolAsync on the problem's stream and sgba_problem_destroy
// frees with cudaFreeAsync, so creating and destroying many small problems
// (local windows) costs no cudaMalloc / cudaFree (which synchronises the
// device). Freed memory stays cached for the next problem up to 1/16 of the
// device's memory; above that the pool returns it at synchronisation points.
cudaMemPool_t problem_pool(int dev) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(dev);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps pr{};
  pr.allocType = cudaMemAllocationTypePinned;
  pr.location.type = cudaMemLocationTypeDevice;
  pr.location.id = dev;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &pr) != cudaSuccess) return nullptr;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
    uint64_t keep = total_b / 16;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  pools[dev] = pool;
  return pool;
}

template <class V>
void release(V& v) {
  V().swap(v);
}

template <class T>
int dev_alloc(sgba_problem* p, T** ptr, size_t count) {
  *ptr = nullptr;
  if (count == 0) count = 1;
  const size_t bytes = (sizeof(T) * count + 255) & ~size_t(255);
  void* v = nullptr;
  if (bytes * 4 > p->chunk_size) {
    SGBA_CK(cudaMallocFromPoolAsync(&v, bytes, p->pool, p->stream));
    p->allocs.push_back(v);
  } else {
    if (bytes > p->chunk_left) {
      void* c = nullptr;
      SGBA_CK(cudaMallocFromPoolAsync(&c, p->chunk_size, p->pool, p->stream));
      p->allocs.push_back(c);
      p->chunk_ptr = static_cast<char*>(c);
      p->chunk_left = p->chunk_size;
    }
    v = p->chunk_ptr;
    p->chunk_ptr += bytes;
    p->chunk_left -= bytes;
  }
  *ptr = static_cast<T*>(v);
  return SGBA_OK;
}

// Device copy of a host vector, ordered on the problem's stream: `h` must stay
// alive until upload() synchronises the stream at its end.
template <class T, class A>
int dev_upload(sgba_problem* p, T** ptr, const std::vector<T, A>& h) {
  int st = dev_alloc(p, ptr, h.size());
  if (st) return st;
  if (!h.empty()) SGBA_CK(cudaMemcpyAsync(*ptr, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, p->stream));
  return SGBA_OK;
}

// Run f(begin, end) over [0, n) split across host threads (contiguous ranges,
// so per-range work that is itself ordered stays deterministic).
// Persistent host worker pool (the set-up loops of sgba_problem_create run on
// it; threads are created once per process).  run(n, f) calls f(k) for every
// k in [0, n) on the workers and the calling thread and returns when all have
// finished; a region started while another host thread's region runs is
// executed by its own caller, item by item.
// The set-up runs about a dozen short regions back to back, so a worker that
// finished a region watches for the next one for a while (kSpinNs) before it
// sleeps on the condition variable, and regions are entered and retired
// through atomics: a wake-up through the condition variable, or a convoy on
// one mutex, costs tens of microseconds per region.
//
// Retiring a region: the caller clears region_ once every item ran, then
// waits until no worker is inside_. A worker counts itself inside_ before it
// reads region_, so one that arrives after the caller saw inside_ == 0 reads
// the cleared pointer (sequentially consistent atomics).
class HostPool {
 public:
  static HostPool& get() {
    static HostPool pool;
    return pool;
  }
  int threads() const { return forked_child() ? 1 : nthreads_; }
  void run(int n, const std::function<void(int)>& f) {
    if (n <= 0) return;
    if (n == 1 || nthreads_ <= 1 || forked_child()) {  // a forked child has no workers
      for (int k = 0; k < n; ++k) f(k);
      return;
    }
    // Another host thread's region holds the workers (problems created
    // concurrently, e.g. many local windows): run the items here, in order,
    // instead of queueing behind it.  The items are the same either way, so
    // the results are too.
    std::unique_lock<std::mutex> region_lock(region_mu_, std::try_to_lock);
    if (!region_lock.owns_lock()) {
      for (int k = 0; k < n; ++k) f(k);
      return;
    }
    Region r;
    r.fn = &f;
    r.n = n;
    r.remaining.store(n);
    {
      std::lock_guard<std::mutex> lk(mu_);  // sleepers test gen_ under mu_
      region_.store(&r);
      gen_.fetch_add(1);
    }
    cv_.notify_all();
    drain(r);
    const auto t0 = std::chrono::steady_clock::now();
    for (int it = 0; r.remaining.load() != 0; ++it) {
      if ((it & 63) == 63 && std::chrono::steady_clock::now() - t0 > std::chrono::nanoseconds(kSpinNs)) {
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return r.remaining.load() == 0; });
        break;
      }
    }
    region_.store(nullptr);
    for (int it = 0; inside_.load() != 0; ++it)
      if ((it & 63) == 63) std::this_thread::yield();
  }

 private:
  static constexpr int64_t kSpinNs = 200000;
  struct Region {
    const std::function<void(int)>* fn = nullptr;
    int n = 0;
    std::atomic<int> next{0};
    std::atomic<int> remaining{0};
  };
  static bool& forked_child() {
    static bool forked = false;
    return forked;
  }
  static void on_fork_child() { forked_child() = true; }
  HostPool() {
    pthread_atfork(nullptr, nullptr, &HostPool::on_fork_child);
    int t = static_cast<int>(std::thread::hardware_concurrency());
    nthreads_ = std::max(1, std::min(t, 16));
    for (int k = 1; k < nthreads_; ++k) workers_.emplace_back([this] { loop(); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }
  void drain(Region& r) {
    for (;;) {
      const int k = r.next.fetch_add(1);
      if (k >= r.n) return;
      (*r.fn)(k);
      if (r.remaining.fetch_sub(1) == 1) {
        std::lock_guard<std::mutex> lk(mu_);
        done_cv_.notify_all();
      }
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      // watch for the next region before sleeping
      const auto t0 = std::chrono::steady_clock::now();
      for (int it = 0; gen_.load() == seen; ++it)
        if ((it & 63) == 63 && std::chrono::steady_clock::now() - t0 > std::chrono::nanoseconds(kSpinNs)) break;
      if (gen_.load() == seen) {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || gen_.load() != seen; });
        if (stop_) return;
      }
      seen = gen_.load();
      inside_.fetch_add(1);
      Region* r = region_.load();
      if (r) drain(*r);
      inside_.fetch_sub(1);
    }
  }
  int nthreads_ = 1;
  std::vector<std::thread> workers_;
  std::mutex region_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  std::atomic<Region*> region_{nullptr};
  std::atomic<uint64_t> gen_{0};
  std::atomic<int> inside_{0};
  bool stop_ = false;
};

// f(begin, end) over contiguous chunks of [0, n) on the host pool.
template <class F>
int par_chunks(int64_t n, int64_t min_per, F f) {
  const int64_t t = std::max<int64_t>(
      1, std::min<int64_t>(HostPool::get().threads(), (n + min_per - 1) / std::max<int64_t>(min_per, 1)));
  HostPool::get().run(static_cast<int>(t), [&](int k) { f(k, n * k / t, n * (k + 1) / t); });
  return static_cast<int>(t);
}

// Items per thread below which a loop is not split further (a fork-join of
// the pool costs a few microseconds while its workers are awake).
constexpr int64_t kMinPerThread = 8192;

template <class F>
void par_ranges(int64_t n, F f) {
  par_chunks(n, kMinPerThread, [&](int, int64_t b, int64_t e) { f(b, e); });
}

// f(begin, end) over ranges of points, whose work is their observations:
// chunks of at least 512 points.
template <class F>
void par_points(int64_t np, F f) {
  par_chunks(np, 512, [&](int, int64_t b, int64_t e) { f(b, e); });
}

bool finite_all(const double* v, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

// Rotation3 are_params_valid (crates/sophus_lie/src/groups/rotation3.rs:314-319).
bool quat_valid(const double* q) {
  double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  return std::fabs(n - 1.0) <= 1e-6;
}

int build_plan(const sgba_problem_desc* d, Plan* P) {
  if (d->n_cam < 1) return set_error(SGBA_ERR_INVALID_ARGUMENT, "n_cam must be >= 1 (got %d)", d->n_cam);
  if (d->n_pt < 0 || d->n_obs < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "negative n_pt or n_obs");
  if (!d->poses) return set_error(SGBA_ERR_INVALID_ARGUMENT, "poses is NULL");
  if (d->n_pt > 0 && !d->points) return set_error(SGBA_ERR_INVALID_ARGUMENT, "points is NULL");
  if (d->n_obs > 0 && (!d->obs_cam || !d->obs_pt || !d->obs_uv))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "observation arrays are NULL");
  if (d->n_obs >= (int64_t(1) << 31))
    return set_error(SGBA_ERR_UNSUPPORTED, "n_obs %lld exceeds the 2^31 term limit", (long long)d->n_obs);
  std::atomic<bool> finite_uv{true};
  par_ranges(2 * d->n_obs, [&](int64_t b, int64_t e) {
    if (!finite_all(d->obs_uv + b, e - b)) finite_uv = false;
  });
  if (!finite_all(d->poses, 7ll * d->n_cam) || !finite_all(d->points, 3ll * d->n_pt) || !finite_uv ||
      !finite_all(d->intrinsics, 4))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "non-finite input value");
  if (std::isnan(d->huber_delta) || !huber_in_float_range(d->huber_delta))
    return set_error(SGBA_ERR_INVALID_ARGUMENT,
                     "huber_delta %g: a positive threshold must lie in the normal float range [1.2e-38, 3.4e38]",
                     d->huber_delta);
  for (int j = 0; j < d->n_cam; ++j)
    if (!quat_valid(d->poses + 7 * j))
      return set_error(SGBA_ERR_INVALID_PARAMS, "pose %d: quaternion norm differs from 1 by more than 1e-6", j);
  const int nc = d->n_cam, np = d->n_pt;
  const int64_t no = d->n_obs;
  {
    // the first out-of-range observation, as a sequential scan reports it
    std::atomic<int64_t> first_bad{no};
    par_ranges(no, [&](int64_t b, int64_t e) {
      for (int64_t o = b; o < e; ++o) {
        if (static_cast<uint32_t>(d->obs_cam[o]) >= static_cast<uint32_t>(nc) ||
            static_cast<uint32_t>(d->obs_pt[o]) >= static_cast<uint32_t>(np)) {
          int64_t cur = first_bad.load();
          while (o < cur && !first_bad.compare_exchange_weak(cur, o)) {
          }
          return;
        }
      }
    });
    const int64_t o = first_bad.load();
    if (o < no) {
      const int32_t jc = d->obs_cam[o], ip = d->obs_pt[o];
      if (static_cast<uint32_t>(jc) >= static_cast<uint32_t>(nc))
        return set_error(SGBA_ERR_INVALID_ARGUMENT, "observation %lld: pose index %d out of range", (long long)o, jc);
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "observation %lld: point index %d out of range", (long long)o, ip);
    }
  }
  P->nc = nc;
  P->np = np;
  P->no = no;
  // Order (point, pose, original index): a stable counting sort by point, then
  // a stable sort by pose inside each point (points have few observations).
  // The counting sort runs on chunks of observations: per-chunk counts, then
  // each chunk's slots follow the earlier chunks' inside every point, so the
  // order is exactly the sequential stable one.
  sgba::RawVec<int64_t> ord(no);
  P->obs_pose.resize(no);  // the pose of every sorted observation, filled with ord
  int32_t* const opose = P->obs_pose.data();
  std::vector<int64_t> cp(np + 1, 0);
  {
    const int64_t T = std::max<int64_t>(1, std::min<int64_t>(HostPool::get().threads(), (no + kMinPerThread - 1) / kMinPerThread));
    std::vector<std::vector<int32_t>> cnt(T);
    HostPool::get().run(static_cast<int>(T), [&](int t) {
      cnt[t].assign(np, 0);
      for (int64_t o = no * t / T; o < no * (t + 1) / T; ++o) cnt[t][d->obs_pt[o]]++;
    });
    par_points(np, [&](int64_t i0, int64_t i1) {
      for (int64_t i = i0; i < i1; ++i) {
        int64_t run = 0;
        for (int64_t t = 0; t < T; ++t) run += cnt[t][i];
        cp[i + 1] = run;
      }
    });
    for (int i = 0; i < np; ++i) cp[i + 1] += cp[i];
    std::vector<std::vector<int64_t>> base(T);
    par_points(np, [&](int64_t i0, int64_t i1) {
      for (int64_t i = i0; i < i1; ++i) {
        int64_t run = cp[i];
        for (int64_t t = 0; t < T; ++t) {
          const int32_t c = cnt[t][i];
          cnt[t][i] = static_cast<int32_t>(run - cp[i]);  // chunk t's first slot inside point i
          run += c;
        }
      }
    });
    HostPool::get().run(static_cast<int>(T), [&](int t) {
      std::vector<int32_t>& slot = cnt[t];
      for (int64_t o = no * t / T; o < no * (t + 1) / T; ++o) {
        const int32_t i = d->obs_pt[o];
        const int64_t k = cp[i] + slot[i]++;
        ord[k] = o;
        opose[k] = d->obs_cam[o];
      }
    });
  }
  // groups (reduction ranges: equal non-conditioned arguments, cost_fn.rs:374-390):
  // runs of equal pose inside each point
  std::vector<int64_t> gcount(np + 1, 0);
  par_points(np, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      int64_t* a = ord.data() + cp[i];
      int32_t* kp = opose + cp[i];
      const int64_t n = cp[i + 1] - cp[i];
      for (int64_t k = 1; k < n; ++k) {  // insertion sort by pose, stable
        const int64_t v = a[k];
        const int32_t key = kp[k];
        int64_t m = k;
        while (m > 0 && kp[m - 1] > key) {
          a[m] = a[m - 1];
          kp[m] = kp[m - 1];
          --m;
        }
        a[m] = v;
        kp[m] = key;
      }
      int64_t runs = 0;
      for (int64_t k = 0; k < n; ++k)
        if (k == 0 || kp[k] != kp[k - 1]) ++runs;
      gcount[i + 1] = runs;
    }
  });
  for (int i = 0; i < np; ++i) gcount[i + 1] += gcount[i];
  P->ng = gcount[np];
  P->obs_pt.resize(no);
  P->g_begin.resize(P->ng + 1);
  P->g_pose.resize(P->ng);
  P->g_pt.resize(P->ng);
  par_points(np, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      int64_t g = gcount[i];
      for (int64_t k = cp[i]; k < cp[i + 1]; ++k) {
        const int32_t jc = opose[k];
        P->obs_pt[k] = static_cast<int32_t>(i);
        if (k == cp[i] || jc != opose[k - 1]) {
          P->g_begin[g] = k;
          P->g_pose[g] = jc;
          P->g_pt[g] = static_cast<int32_t>(i);
          ++g;
        }
      }
    }
  });
  P->g_begin[P->ng] = no;
  P->pt_g_begin.assign(gcount.begin(), gcount.end());
  P->ord = std::move(ord);
  // free / marginalized blocks (var_families.rs:60-113, var_family.rs:156-237)
  P->pose_fb.assign(nc, -1);
  P->fb_pose.clear();
  for (int j = 0; j < nc; ++j)
    if (!(d->pose_const && d->pose_const[j])) {
      P->pose_fb[j] = static_cast<int32_t>(P->fb_pose.size());
      P->fb_pose.push_back(j);
    }
  P->nf = static_cast<int32_t>(P->fb_pose.size());
  P->pt_mb.assign(np, -1);
  P->mb_pt.clear();
  for (int i = 0; i < np; ++i)
    if (!(d->point_const && d->point_const[i])) {
      P->pt_mb[i] = static_cast<int32_t>(P->mb_pt.size());
      P->mb_pt.push_back(i);
    }
  P->nm = static_cast<int32_t>(P->mb_pt.size());
  P->cnt_f.assign(P->nf, 0.0);
  P->cnt_m.assign(P->nm, 0.0);
  // per marginalized point: its reduced terms; per free pose: its terms,
  // counted on chunks of terms; the camera term lists fill stably the same way
  par_points(np, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i)
      if (P->pt_mb[i] >= 0) P->cnt_m[P->pt_mb[i]] = static_cast<double>(P->pt_g_begin[i + 1] - P->pt_g_begin[i]);
  });
  const int64_t TG = std::max<int64_t>(1, std::min<int64_t>(HostPool::get().threads(), (P->ng + kMinPerThread - 1) / kMinPerThread));
  std::vector<std::vector<int64_t>> fcnt(TG);
  std::vector<int64_t> hoff_part(TG, 0);
  HostPool::get().run(static_cast<int>(TG), [&](int t) {
    fcnt[t].assign(P->nf, 0);
    int64_t h = 0;
    for (int64_t g = P->ng * t / TG; g < P->ng * (t + 1) / TG; ++g) {
      const int fb = P->pose_fb[P->g_pose[g]];
      if (fb < 0) continue;
      fcnt[t][fb]++;
      if (P->pt_mb[P->g_pt[g]] >= 0) ++h;
    }
    hoff_part[t] = h;
  });
  int64_t h_off = 0;
  for (int64_t t = 0; t < TG; ++t) h_off += hoff_part[t];
  for (int f = 0; f < P->nf; ++f)
    for (int64_t t = 0; t < TG; ++t) P->cnt_f[f] += static_cast<double>(fcnt[t][f]);
  int64_t h_diag = 0;
  for (double c : P->cnt_f) h_diag += (c > 0);
  for (double c : P->cnt_m) h_diag += (c > 0);
  P->n_h_blocks = h_diag + h_off;
  // camera term lists and tiles
  P->cam_g_begin.assign(P->nf + 1, 0);
  for (int f = 0; f < P->nf; ++f) {
    int64_t run = 0;
    for (int64_t t = 0; t < TG; ++t) run += fcnt[t][f];
    P->cam_g_begin[f + 1] = P->cam_g_begin[f] + run;
  }
  P->cam_g.resize(P->cam_g_begin[P->nf]);
  for (int f = 0; f < P->nf; ++f) {
    int64_t run = P->cam_g_begin[f];
    for (int64_t t = 0; t < TG; ++t) {
      const int64_t c = fcnt[t][f];
      fcnt[t][f] = run;  // chunk t's first slot in camera f's list
      run += c;
    }
  }
  HostPool::get().run(static_cast<int>(TG), [&](int t) {
    std::vector<int64_t>& slot = fcnt[t];
    for (int64_t g = P->ng * t / TG; g < P->ng * (t + 1) / TG; ++g) {
      const int fb = P->pose_fb[P->g_pose[g]];
      if (fb >= 0) P->cam_g[slot[fb]++] = g;
    }
  });
  P->tile_fb.clear();
  P->tile_begin.clear();
  P->tile_end.clear();
  P->fb_tile_begin.assign(P->nf + 1, 0);
  for (int f = 0; f < P->nf; ++f) {
    P->fb_tile_begin[f] = static_cast<int64_t>(P->tile_fb.size());
    for (int64_t e = P->cam_g_begin[f]; e < P->cam_g_begin[f + 1]; e += kTile) {
      P->tile_fb.push_back(f);
      P->tile_begin.push_back(e);
      P->tile_end.push_back(std::min<int64_t>(e + kTile, P->cam_g_begin[f + 1]));
    }
  }
  P->fb_tile_begin[P->nf] = static_cast<int64_t>(P->tile_fb.size());
  // The reduced camera system pattern and its observation pairs are built on
  // the device in upload() (build_schur_pattern).
  P->sb_row.clear();
  P->sb_col.clear();
  P->sb_pair_begin.clear();
  P->chunk_begin.clear();
  P->block_chunk_begin.clear();
  // Gauge: scale about the common center of the constant poses, when no point
  // is constant and at least one pose is constant.
  P->gauge_kind = 0;
  bool any_const_pt = false;
  for (int i = 0; i < np; ++i) any_const_pt |= (d->point_const && d->point_const[i]);
  if (!any_const_pt && P->nf < nc && P->nm > 0) {
    const double* c0 = nullptr;
    bool same = true;
    for (int j = 0; j < nc; ++j) {
      if (P->pose_fb[j] >= 0) continue;
      const double* t = d->poses + 7 * j + 4;
      if (!c0) c0 = t;
      else same = same && t[0] == c0[0] && t[1] == c0[1] && t[2] == c0[2];
    }
    if (c0 && same) {
      P->gauge_kind = 1;
      P->gauge_center[0] = c0[0];
      P->gauge_center[1] = c0[1];
      P->gauge_center[2] = c0[2];
    }
  }
  return SGBA_OK;
}

// Pose-graph edges (PoseGraph3CostTerm): validated, sorted by (m, n) as
// CostFn::sort orders them, reduced into terms of equal (m, n); each term
// adds one damping count to each of its free poses (nu I once per reduced
// term, cost_system.rs:190-273); the per-free-block list of (term, side)
// records.  The edges fix the scale: no gauge projection.
int build_edges(const sgba_pose_graph* g, Plan* P) {
  if (!g || g->n_edge == 0) return SGBA_OK;
  const int32_t n = g->n_edge;
  if (n < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "negative edge count");
  if (!g->edge_pose || !g->edge_m_from_n) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL edge array");
  for (int32_t k = 0; k < n; ++k) {
    const int32_t m = g->edge_pose[2 * k], q = g->edge_pose[2 * k + 1];
    if (m < 0 || m >= P->nc || q < 0 || q >= P->nc || m == q)
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "edge %d: poses (%d, %d) out of range or equal", k, m, q);
    if (!finite_all(g->edge_m_from_n + 7 * k, 7))
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "edge %d: non-finite measurement", k);
    if (!quat_valid(g->edge_m_from_n + 7 * k))
      return set_error(SGBA_ERR_INVALID_PARAMS, "edge %d: invalid quaternion", k);
  }
  std::vector<int32_t> ord(n);
  for (int32_t k = 0; k < n; ++k) ord[k] = k;
  std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) {
    if (g->edge_pose[2 * a] != g->edge_pose[2 * b]) return g->edge_pose[2 * a] < g->edge_pose[2 * b];
    return g->edge_pose[2 * a + 1] < g->edge_pose[2 * b + 1];
  });
  P->edge_m.resize(n);
  P->edge_n.resize(n);
  P->edge_mn.resize(7 * static_cast<size_t>(n));
  P->eterm_begin.clear();
  P->eterm_fm.clear();
  P->eterm_fn.clear();
  for (int32_t k = 0; k < n; ++k) {
    const int32_t o = ord[k];
    P->edge_m[k] = g->edge_pose[2 * o];
    P->edge_n[k] = g->edge_pose[2 * o + 1];
    double* mn = &P->edge_mn[7 * static_cast<size_t>(k)];
    std::memcpy(mn, g->edge_m_from_n + 7 * o, sizeof(double) * 7);
    if (!(0.0 <= mn[0]))
      for (int q = 0; q < 4; ++q) mn[q] = -mn[q];
    if (k == 0 || P->edge_m[k] != P->edge_m[k - 1] || P->edge_n[k] != P->edge_n[k - 1]) {
      P->eterm_begin.push_back(k);
      P->eterm_fm.push_back(P->pose_fb[P->edge_m[k]]);
      P->eterm_fn.push_back(P->pose_fb[P->edge_n[k]]);
    }
  }
  const int32_t nt = static_cast<int32_t>(P->eterm_fm.size());
  P->eterm_begin.push_back(n);
  // per free block its records (term t side 0 -> slot 2t, side 1 -> 2t + 1), in term order
  P->efb_begin.assign(P->nf + 1, 0);
  for (int32_t t = 0; t < nt; ++t) {
    if (P->eterm_fm[t] >= 0) ++P->efb_begin[P->eterm_fm[t] + 1];
    if (P->eterm_fn[t] >= 0) ++P->efb_begin[P->eterm_fn[t] + 1];
  }
  for (int f = 0; f < P->nf; ++f) P->efb_begin[f + 1] += P->efb_begin[f];
  P->efb_slot.assign(P->efb_begin[P->nf], 0);
  std::vector<int32_t> fill(P->efb_begin.begin(), P->efb_begin.end() - 1);
  for (int32_t t = 0; t < nt; ++t) {
    if (P->eterm_fm[t] >= 0) P->efb_slot[fill[P->eterm_fm[t]]++] = 2 * t;
    if (P->eterm_fn[t] >= 0) P->efb_slot[fill[P->eterm_fn[t]]++] = 2 * t + 1;
    if (P->eterm_fm[t] >= 0) P->cnt_f[P->eterm_fm[t]] += 1.0;
    if (P->eterm_fn[t] >= 0) P->cnt_f[P->eterm_fn[t]] += 1.0;
  }
  P->gauge_kind = 0;
  return SGBA_OK;
}

// Reduced camera system: lower blocks (row >= col) of the Schur fill
// (crates/sophus_opt/src/nlls/damped_hessian.rs:261-325) and the observation
// pairs summed into each.  The pairs per block are counted on the device, the
// block pattern and offsets are formed here, and the pair list itself is
// written on the device in (block, point) order (sgba_plan.cu).
int build_schur_pattern(sgba_problem* p) {
  Plan& P = p->plan;
  Dev& d = p->d;
  const int nf = P.nf;
  if (!(nf > 0 && nf <= kMaxDenseFree)) return SGBA_OK;
  const int64_t nlow = static_cast<int64_t>(nf) * (nf + 1) / 2;
  auto lid = [](int64_t r, int64_t c) { return r * (r + 1) / 2 + c; };
  Sizes tmp_sizes = p->sz;
  tmp_sizes.np = P.np;
  int32_t* totals = nullptr;
  SGBA_CK(cudaMallocFromPoolAsync(&totals, sizeof(int32_t) * nlow, p->pool, p->stream));
  std::vector<int32_t> cnt(nlow, 0);
  cudaError_t e = cudaMemsetAsync(totals, 0, sizeof(int32_t) * nlow, p->stream);
  if (e == cudaSuccess) e = sgba::pair_totals(tmp_sizes, d, totals, p->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), totals, sizeof(int32_t) * nlow, cudaMemcpyDeviceToHost, p->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
  cudaFreeAsync(totals, p->stream);
  if (e != cudaSuccess) return set_error(SGBA_ERR_CUDA, "Schur pattern (counts): %s", cudaGetErrorString(e));
  std::vector<int32_t> bid(nlow, -1);
  int64_t nb = 0;
  // pose-graph terms between two free poses need their block even where no
  // point joins the two
  std::vector<char> eforce(P.eterm_fm.empty() ? 0 : nlow, 0);
  for (size_t t = 0; t < P.eterm_fm.size(); ++t)
    if (P.eterm_fm[t] >= 0 && P.eterm_fn[t] >= 0)
      eforce[lid(std::max(P.eterm_fm[t], P.eterm_fn[t]), std::min(P.eterm_fm[t], P.eterm_fn[t]))] = 1;
  for (int r = 0; r < nf; ++r)
    for (int c = 0; c <= r; ++c)
      if (cnt[lid(r, c)] > 0 || (r == c && P.cnt_f[r] > 0) || (!eforce.empty() && eforce[lid(r, c)])) {
        bid[lid(r, c)] = static_cast<int32_t>(nb++);
        P.sb_row.push_back(r);
        P.sb_col.push_back(c);
      }
  if (!P.eterm_fm.empty()) {
    // per block the terms landing there, in term order (bit 31: the block's
    // rows are pose n's, i.e. J_m^T J_n transposed)
    std::vector<std::vector<int32_t>> lists(nb);
    for (size_t t = 0; t < P.eterm_fm.size(); ++t) {
      const int fm = P.eterm_fm[t], fn = P.eterm_fn[t];
      if (fm < 0 || fn < 0) continue;
      const int32_t b = bid[lid(std::max(fm, fn), std::min(fm, fn))];
      lists[b].push_back(static_cast<int32_t>(t) | (fm > fn ? 0 : static_cast<int32_t>(0x80000000u)));
    }
    P.eblk_begin.assign(nb + 1, 0);
    P.eblk_term.clear();
    for (int64_t b = 0; b < nb; ++b) {
      P.eblk_term.insert(P.eblk_term.end(), lists[b].begin(), lists[b].end());
      P.eblk_begin[b + 1] = static_cast<int32_t>(P.eblk_term.size());
    }
  }
  P.sb_pair_begin.assign(nb + 1, 0);
  for (int64_t b = 0; b < nb; ++b) P.sb_pair_begin[b + 1] = P.sb_pair_begin[b] + cnt[lid(P.sb_row[b], P.sb_col[b])];
  const int64_t npairs = P.sb_pair_begin[nb];
  int st;
  // Nearly dense systems of the pinhole camera with fixed params and no
  // pose-graph edges take the tiled Schur pass (the selection in upload()),
  // which reads the term table: their pair lists are not built (a window of
  // 40 cameras and 4000 points has ~3M pairs).
  const bool tiled = p->camera_model == SGBA_CAMERA_PINHOLE && !p->intr_free && P.eterm_fm.empty() &&
                     10 * nb > 9 * nlow && 2 * P.ng >= static_cast<int64_t>(P.np) * nf;
  p->pairs_built = !tiled;
  if (tiled) return dev_alloc(p, &d.pairs, 0);
  if (npairs >= (int64_t(1) << 31))
    return set_error(SGBA_ERR_UNSUPPORTED, "%lld observation pairs exceed the 2^31 limit", (long long)npairs);
  // chunks of at most kSchurChunk pairs within one block (at least one per block)
  P.block_chunk_begin.assign(nb + 1, 0);
  for (int64_t b = 0; b < nb; ++b) {
    P.block_chunk_begin[b] = static_cast<int32_t>(P.chunk_begin.size());
    int64_t q = P.sb_pair_begin[b];
    do {
      P.chunk_begin.push_back(q);
      q += kSchurChunk;
    } while (q < P.sb_pair_begin[b + 1]);
  }
  P.block_chunk_begin[nb] = static_cast<int32_t>(P.chunk_begin.size());
  P.chunk_begin.push_back(npairs);
  if ((st = dev_alloc(p, &d.pairs, static_cast<size_t>(npairs)))) return st;
  if (npairs == 0) return SGBA_OK;
  // point chunks: as many as keep the (chunk x block) table near 64 Mi entries
  int64_t nch = (int64_t(64) << 20) / std::max<int64_t>(nb, 1);
  nch = std::max<int64_t>(1, std::min<int64_t>({nch, 512, static_cast<int64_t>(P.np)}));
  int32_t *bidmap = nullptr, *table = nullptr;
  int64_t* bbeg = nullptr;
  e = cudaMallocFromPoolAsync(&bidmap, sizeof(int32_t) * nlow, p->pool, p->stream);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&table, sizeof(int32_t) * nch * nb, p->pool, p->stream);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&bbeg, sizeof(int64_t) * (nb + 1), p->pool, p->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bidmap, bid.data(), sizeof(int32_t) * nlow, cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bbeg, P.sb_pair_begin.data(), sizeof(int64_t) * (nb + 1), cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(table, 0, sizeof(int32_t) * nch * nb, p->stream);
  if (e == cudaSuccess) e = sgba::pair_fill(tmp_sizes, d, bidmap, nb, bbeg, static_cast<int32_t>(nch), table, p->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
  if (bidmap) cudaFreeAsync(bidmap, p->stream);
  if (table) cudaFreeAsync(table, p->stream);
  if (bbeg) cudaFreeAsync(bbeg, p->stream);
  if (e != cudaSuccess)
    return set_error(e == cudaErrorMemoryAllocation ? SGBA_ERR_OUT_OF_MEMORY : SGBA_ERR_CUDA, "Schur pattern (pairs): %s",
                     cudaGetErrorString(e));
  return SGBA_OK;
}

int upload(sgba_problem* p, const sgba_problem_desc* desc) {
  Plan& P = p->plan;
  // chunk size for the small buffers: about 48 bytes per observation, 1-16 MiB
  p->chunk_size = std::min<size_t>(size_t(16) << 20, std::max<size_t>(size_t(1) << 20, 48 * static_cast<size_t>(P.no)));
  Dev& d = p->d;
  Sizes& s = p->sz;
  s.nc = P.nc;
  s.np = P.np;
  s.nf = P.nf;
  s.nm = P.nm;
  s.no = P.no;
  s.ng = P.ng;
  s.ntiles = static_cast<int64_t>(P.tile_fb.size());
  s.intr_free = p->intr_free;
  s.eucm = p->camera_model == SGBA_CAMERA_EUCM ? 1 : 0;
  s.intr_nk = s.eucm ? 6 : 4;
  s.n6 = 6 * P.nf + (p->intr_free ? 6 : 0);
  for (int k = 0; k < 4; ++k) s.intr[k] = desc->intrinsics[k];
  s.intr[4] = p->eucm_ab[0];
  s.intr[5] = p->eucm_ab[1];
  s.huber = desc->huber_delta;
  s.gauge_kind = P.gauge_kind;
  for (int k = 0; k < 3; ++k) s.gauge_center[k] = P.gauge_center[k];
  int st;
  // host staging of the copies below: alive until the stream is synchronised
  sgba::RawVec<double2> uv(P.no);
  std::vector<int32_t> cpt(1, 0);
  std::vector<double> poses(desc->poses, desc->poses + 7 * P.nc);
  std::vector<double> pts(desc->points, desc->points + 3 * P.np);
  par_ranges(P.no, [&](int64_t b, int64_t e) {
    for (int64_t k = b; k < e; ++k) uv[k] = make_double2(desc->obs_uv[2 * P.ord[k]], desc->obs_uv[2 * P.ord[k] + 1]);
  });
  if ((st = dev_upload(p, &d.obs_uv, uv))) return st;
  if ((st = dev_upload(p, &d.obs_pose, P.obs_pose))) return st;
  if ((st = dev_upload(p, &d.obs_pt, P.obs_pt))) return st;
  if ((st = dev_upload(p, &d.g_begin, P.g_begin))) return st;
  if ((st = dev_upload(p, &d.g_pose, P.g_pose))) return st;
  if ((st = dev_upload(p, &d.g_pt, P.g_pt))) return st;
  if ((st = dev_upload(p, &d.pt_g_begin, P.pt_g_begin))) return st;
  if ((st = dev_upload(p, &d.pose_fb, P.pose_fb))) return st;
  if ((st = dev_upload(p, &d.pt_mb, P.pt_mb))) return st;
  if ((st = dev_upload(p, &d.fb_pose, P.fb_pose))) return st;
  if ((st = dev_upload(p, &d.mb_pt, P.mb_pt))) return st;
  if ((st = dev_upload(p, &d.cnt_f, P.cnt_f))) return st;
  if ((st = dev_upload(p, &d.cnt_m, P.cnt_m))) return st;
  if ((st = dev_upload(p, &d.cam_g, P.cam_g))) return st;
  if ((st = dev_upload(p, &d.tile_fb, P.tile_fb))) return st;
  if ((st = dev_upload(p, &d.tile_begin, P.tile_begin))) return st;
  if ((st = dev_upload(p, &d.tile_end, P.tile_end))) return st;
  if ((st = dev_upload(p, &d.fb_tile_begin, P.fb_tile_begin))) return st;
  {
    // landmark point chunks: consecutive points, at most 256 terms and 256 points
    int64_t terms = 0, cap = 256;
    int npts = 0;
    for (int i = 0; i < P.np; ++i) {
      const int64_t L = P.pt_g_begin[i + 1] - P.pt_g_begin[i];
      cap = std::max(cap, L);
      if (npts > 0 && (terms + L > 256 || npts == 256)) {
        cpt.push_back(i);
        terms = 0;
        npts = 0;
      }
      terms += L;
      ++npts;
    }
    if (cpt.back() != P.np) cpt.push_back(P.np);
    s.nlchunk = static_cast<int32_t>(cpt.size()) - 1;
    s.lmk_cap = static_cast<int32_t>(cap);
    if (s.nlchunk > 0 && sgba::landmark_setup(s.lmk_cap) != 0) s.nlchunk = 0;  // fall back to the warp kernel
    if ((st = dev_upload(p, &d.lmk_chunk_pt, cpt))) return st;
    if ((st = dev_alloc(p, &d.slow_list, static_cast<size_t>(std::max(P.np, 1))))) return st;
    if ((st = dev_alloc(p, &d.slow_count, 1))) return st;
    SGBA_CK(cudaMemsetAsync(d.slow_count, 0, sizeof(int32_t), p->stream));
  }
  if ((st = build_schur_pattern(p))) return st;
  s.n_edge = static_cast<int>(P.edge_m.size());
  s.n_eterm = static_cast<int>(P.eterm_fm.size());
  if (s.n_edge > 0) {
    const size_t nt = static_cast<size_t>(s.n_eterm);
    if ((st = dev_upload(p, &d.edge_m, P.edge_m))) return st;
    if ((st = dev_upload(p, &d.edge_n, P.edge_n))) return st;
    if ((st = dev_upload(p, &d.edge_mn, P.edge_mn))) return st;
    if ((st = dev_upload(p, &d.eterm_begin, P.eterm_begin))) return st;
    if ((st = dev_upload(p, &d.eterm_fm, P.eterm_fm))) return st;
    if ((st = dev_upload(p, &d.eterm_fn, P.eterm_fn))) return st;
    if ((st = dev_alloc(p, &d.edge_out, 2 * nt * sgba::kPriorOut))) return st;
    if ((st = dev_alloc(p, &d.edge_hmn, 36 * nt))) return st;
    if ((st = dev_upload(p, &d.efb_begin, P.efb_begin))) return st;
    if ((st = dev_upload(p, &d.efb_slot, P.efb_slot))) return st;
    if ((st = dev_upload(p, &d.eblk_begin, P.eblk_begin))) return st;
    if ((st = dev_upload(p, &d.eblk_term, P.eblk_term))) return st;
  }
  s.nsb = static_cast<int64_t>(P.sb_row.size());
  s.nchunk = P.chunk_begin.empty() ? 0 : static_cast<int64_t>(P.chunk_begin.size()) - 1;
  if ((st = dev_upload(p, &d.sb_row, P.sb_row))) return st;
  if ((st = dev_upload(p, &d.sb_col, P.sb_col))) return st;
  if ((st = dev_upload(p, &d.sb_pair_begin, P.sb_pair_begin))) return st;
  if (s.nchunk > 0) {
    if ((st = dev_upload(p, &d.chunk_begin, P.chunk_begin))) return st;
    if ((st = dev_upload(p, &d.block_chunk_begin, P.block_chunk_begin))) return st;
    if ((st = dev_alloc(p, &d.schur_part, 36 * static_cast<size_t>(s.nchunk)))) return st;
  }
  // state (quaternions disambiguated to w >= 0 as from_params does)
  for (int j = 0; j < P.nc; ++j)
    if (!(0.0 <= poses[7 * j]))
      for (int k = 0; k < 4; ++k) poses[7 * j + k] = -poses[7 * j + k];
  {
    // camera params: current and trial, both from the descriptor and options
    std::vector<double> intr(2 * kIntrMax);
    for (int k = 0; k < kIntrMax; ++k) intr[k] = intr[kIntrMax + k] = s.intr[k];
    if ((st = dev_upload(p, &d.intr, intr))) return st;
    d.intr_t = d.intr + kIntrMax;
  }
  if ((st = dev_upload(p, &d.poses, poses))) return st;
  if ((st = dev_upload(p, &d.points, pts))) return st;
  if ((st = dev_alloc(p, &d.poses_t, 7 * static_cast<size_t>(P.nc)))) return st;
  if ((st = dev_alloc(p, &d.points_t, 3 * static_cast<size_t>(P.np)))) return st;
  if ((st = dev_alloc(p, &d.res, P.no))) return st;
  if ((st = dev_alloc(p, &d.res_t, P.no))) return st;
  if ((st = dev_alloc(p, &d.pose_f, 12 * static_cast<size_t>(P.nc)))) return st;
  if ((st = dev_alloc(p, &d.pose_dd, 24 * static_cast<size_t>(P.nc)))) return st;
  if ((st = dev_alloc(p, &d.zmat, 20 * static_cast<size_t>(P.ng)))) return st;
  if ((st = dev_alloc(p, &d.cinv, 12 * static_cast<size_t>(P.nm)))) return st;
  if ((st = dev_alloc(p, &d.cvec, 6 * static_cast<size_t>(P.nm)))) return st;
  if ((st = dev_alloc(p, &d.bm, 3 * static_cast<size_t>(P.nm)))) return st;
  if ((st = dev_alloc(p, &d.dm, 3 * static_cast<size_t>(P.nm)))) return st;
  if ((st = dev_alloc(p, &d.gauge_um, 3 * static_cast<size_t>(P.nm)))) return st;
  if (p->intr_free) {
    if ((st = dev_alloc(p, &d.intr_part, kIntrPart * static_cast<size_t>(std::max(P.np, 1))))) return st;
    if ((st = dev_alloc(p, &d.intr_zk, kIntrZk * static_cast<size_t>(std::max(P.nm, 1))))) return st;
    if ((st = dev_alloc(p, &d.intr_scj, kIntrScj * static_cast<size_t>(std::max(P.nf, 1))))) return st;
    if ((st = dev_alloc(p, &d.intr_sum, kIntrSum))) return st;
    SGBA_CK(cudaMemsetAsync(d.intr_sum, 0, sizeof(double) * kIntrSum, p->stream));
  }
  if ((st = dev_alloc(p, &d.bf, 6 * static_cast<size_t>(P.nf)))) return st;
  if ((st = dev_alloc(p, &d.rb, 6 * static_cast<size_t>(P.nf)))) return st;
  if ((st = dev_alloc(p, &d.ufull, 36 * static_cast<size_t>(P.nf)))) return st;
  if ((st = dev_alloc(p, &d.tile_part, 33 * static_cast<size_t>(s.ntiles)))) return st;
  const size_t n6 = static_cast<size_t>(s.n6);
  if ((st = dev_alloc(p, &d.S, n6 * n6))) return st;
  SGBA_CK(cudaMemsetAsync(d.S, 0, sizeof(double) * std::max<size_t>(n6 * n6, 1), p->stream));
  // single-launch cluster solver when the dense system fits one cluster's
  // distributed shared memory; it reads the float-float copy of S
  sgba::dense_cluster_setup(s.n6, &s.dense_c, &s.dense_smem);
  s.band_rows = s.band_w = s.band_c = s.band_ring = 0;
  s.band_nseg = 1;
  s.band_seg_rows = s.band_ring_c = 0;
  std::vector<int32_t> perm;  // staging of the dissection's permutation (alive until the set-up synchronises)
  int brows = 0, bw = 0;
  const bool banded = sgba::band_shape(P.nf, P.sb_row, P.sb_col, &brows, &bw) != 0;
  // loop-shaped: block bandwidth at most half the free poses (float-float
  // linearization and, even where the dense cluster solver would fit, the
  // float-float band solver: the FP32 factor with refinement leaves ~2e-6 in
  // the cost of a 100-camera loop).  A reduced system with (nearly) every
  // block present is dense, whatever split the band search finds (its border
  // can hold up to 24 pose blocks): local windows of 20-40 cameras that all
  // see the same points.
  const int64_t full_blocks = static_cast<int64_t>(P.nf) * (P.nf + 1) / 2;
  const bool nearly_dense = 10 * static_cast<int64_t>(P.sb_row.size()) > 9 * full_blocks;
  const bool loop_shaped = banded && 2 * (bw / 6) <= P.nf && !nearly_dense;
  if (loop_shaped && p->intr_free)
    return set_error(SGBA_ERR_UNSUPPORTED,
                     "free intrinsics on a loop-shaped problem (banded float-float solver) are not on this path");
  if (banded && !p->intr_free && (s.dense_c == 0 ? 4 * (bw / 6) <= P.nf : loop_shaped)) {
    // banded reduced system (sequential / loop problems): band + dense border solver
    int rows = brows, w = bw, c = 0, ring = 0, ring_c = 0;
    // Nested dissection of a loop: the band part is split into two arcs
    // around a separator one band width long; the arcs are independent bands
    // (the second in reverse order, so that both meet the separator at their
    // ends), factored and swept concurrently, and the separator joins the
    // loop closure in the corner.  Used when both arcs have at least 48 pose
    // blocks and the corner (at most 48 pose blocks) fits the factor kernel
    // as a dense band.
    const int rb = rows / 6, wb = w / 6, nbdb = P.nf - rb;
    const int m1 = (rb - wb) / 2, m2 = rb - wb - m1;
    int nseg = 1;
    if (loop_shaped && m1 >= 48 && m2 >= 48 && wb + nbdb <= 48 &&
        sgba::band_setup(s.n6, 6 * (rb - wb), w, 2, 6 * std::max(m1, m2), &c, &ring, &ring_c) > 0) {
      nseg = 2;
      rows = 6 * (rb - wb);
    } else if (sgba::band_setup(s.n6, rows, w, 1, rows, &c, &ring, &ring_c) <= 0) {
      c = 0;
    }
    if (c > 0) {
      s.band_rows = rows;
      s.band_w = w;
      s.band_c = c;
      s.band_ring = ring;
      s.band_nseg = nseg;
      s.band_seg_rows = nseg > 1 ? 6 * m1 : rows;
      s.band_ring_c = ring_c;
      s.dense_c = 0;
      const size_t nbd1 = n6 - static_cast<size_t>(rows) + 1;
      const size_t npan = (static_cast<size_t>(rows) + 23) / 24 + 1;  // panels of both segments
      if ((st = dev_alloc(p, &d.band_scl, n6))) return st;
      if ((st = dev_alloc(p, &d.band_L, static_cast<size_t>(rows) * w))) return st;
      if ((st = dev_alloc(p, &d.band_Xinv, npan * 24 * 24))) return st;
      if ((st = dev_alloc(p, &d.band_Mf, npan * 24 * static_cast<size_t>(w)))) return st;
      if ((st = dev_alloc(p, &d.band_Mb, npan * 24 * static_cast<size_t>(w)))) return st;
      if ((st = dev_alloc(p, &d.band_d, n6))) return st;
      if ((st = dev_alloc(p, &d.band_rd, n6))) return st;
      if ((st = dev_alloc(p, &d.band_P, static_cast<size_t>(w) * 24))) return st;
      if ((st = dev_alloc(p, &d.band_Z, nbd1 * rows))) return st;
      if ((st = dev_alloc(p, &d.band_Zd, nbd1 * rows))) return st;
      if ((st = dev_alloc(p, &d.band_E, nbd1 * nbd1))) return st;
      if ((st = dev_alloc(p, &d.band_xw, n6))) return st;
      if ((st = dev_alloc(p, &d.band_zlo, nbd1 * 2))) return st;
      if (nseg > 1) {
        // the permutation: arc 1 in order, arc 2 reversed, separator, closure
        std::vector<int32_t> blocks;
        blocks.reserve(P.nf);
        for (int b = 0; b < m1; ++b) blocks.push_back(b);
        for (int b = rb - 1; b >= m1 + wb; --b) blocks.push_back(b);
        for (int b = m1; b < m1 + wb; ++b) blocks.push_back(b);
        for (int b = rb; b < P.nf; ++b) blocks.push_back(b);
        perm.assign(n6, 0);
        for (size_t nb = 0; nb < blocks.size(); ++nb)
          for (int k = 0; k < 6; ++k) perm[6 * nb + k] = 6 * blocks[nb] + k;
        if ((st = dev_upload(p, &d.band_perm, perm))) return st;
        const size_t mc = nbd1 - 1, npc = (mc + 23) / 24;
        if ((st = dev_alloc(p, &d.band_Lc, mc * mc))) return st;
        if ((st = dev_alloc(p, &d.band_Xc, npc * 24 * 24))) return st;
        if ((st = dev_alloc(p, &d.band_Mfc, npc * 24 * mc))) return st;
        if ((st = dev_alloc(p, &d.band_Mbc, npc * 24 * mc))) return st;
        if ((st = dev_alloc(p, &d.band_Zcc, mc))) return st;
        if ((st = dev_alloc(p, &d.band_Zdc, mc))) return st;
        if ((st = dev_alloc(p, &d.band_zloc, 1))) return st;
      }
    }
  }
  // small systems that are not loop-shaped: the one-CTA float-float solver
  s.small_dense = 0;
  if (s.band_c == 0 && !loop_shaped && sgba::small_dense_setup(s.n6)) {
    s.small_dense = 1;
    s.dense_c = 0;
  }
  if (s.dense_c > 0 || s.small_dense) {
    if ((st = dev_alloc(p, &d.S2, n6 * n6))) return st;
    SGBA_CK(cudaMemsetAsync(d.S2, 0, sizeof(float2) * std::max<size_t>(n6 * n6, 1), p->stream));
  }
  // point blocks keep the FP32 Cholesky while no pivot loses more than three
  // digits; the others are redone in float-float by a 64-CTA pass
  s.lmk_well_tol = 1e-3f;
  s.lmk_list_grid = std::min(64, std::max(4, P.np / 256));  // grid-stride over the queued points: any grid gives the same results
  // Loop-shaped problems (block bandwidth of S at most half the free poses)
  // get the float-float linearization: their reduced systems cancel ~25x in
  // S = U - sum Z Z^T and their bending modes are weakly constrained, so FP32
  // Jacobian-side products move the step by percents (measured on 300- and
  // 1500-camera loops).  EUCM problems get it when their params are free:
  // fx, alpha and beta nearly trade off over a camera's field of view, so
  // their block of S is close to singular and FP32 Jacobian products move the
  // step by ~1e-6 relative (measured on the 10-camera circle and the 4-camera
  // example); and on the one-CTA solver (systems of at most 144 rows, bound
  // by launch latency, where float-float costs nothing measurable), where the
  // FP32 EUCM Jacobians left 7.6e-7 in the cost of the reference's
  // 10-camera benchmark scene.
  // Problems with pose-graph edges get it too: an edge's weight (residual in
  // radians and meters, unit weight) is ~1e-6 of a pixel term's, so the edges
  // hold the scale only weakly, and FP32 products in S (relative error ~1e-7)
  // moved the step along that direction by ~10 % (measured on an 8-camera
  // circle with odometry edges).
  s.lin_dd = (loop_shaped || (s.eucm && (p->intr_free || s.small_dense)) || s.n_edge > 0) ? 1 : 0;
  // S by tiles of pose blocks when nearly every block of S is present and a
  // point is seen by at least half the free poses on average (local windows):
  // each point's Z is then streamed once per tile instead of once per pair
  s.schur_dense = (!s.lin_dd && !p->intr_free && s.n_edge == 0 && nearly_dense &&
                   2 * P.ng >= static_cast<int64_t>(P.np) * static_cast<int64_t>(P.nf))
                      ? 1
                      : 0;
  if (!p->pairs_built && !s.schur_dense)
    return set_error(SGBA_ERR_UNSUPPORTED, "internal: no Schur pair lists for a system that needs them");
  if (s.schur_dense) {
    if ((st = dev_alloc(p, &d.zterm, static_cast<size_t>(P.np) * static_cast<size_t>(P.nf)))) return st;
    SGBA_CK(sgba::zterm_fill(s, d, d.zterm, p->stream));
  }
  s.lmk_dd_ok = (s.lin_dd && s.nlchunk > 0 && sgba::landmark_dd_setup(s.lmk_cap) == 0) ? 1 : 0;
  s.bsub_chunks_ok = (s.nlchunk > 0 && sgba::backsub_chunks_setup(s.lmk_cap) == 0) ? 1 : 0;
  if (s.lin_dd) {
    if ((st = dev_alloc(p, &d.res_lo, P.no))) return st;
    if ((st = dev_alloc(p, &d.res_lo_t, P.no))) return st;
  }
  // float-float Z: every term under the float-float linearization; otherwise
  // the terms of the points whose blocks are rebuilt in float-float (flagged
  // in zmat's padding)
  if ((st = dev_alloc(p, &d.zdd, static_cast<size_t>(sgba::kZddFloats) * static_cast<size_t>(std::max<int64_t>(P.ng, 1)))))
    return st;
  if (s.dense_c == 0 && s.band_c == 0) {
    // multi-launch dense solver
    if ((st = dev_alloc(p, &d.A, n6 * n6))) return st;
    if ((st = dev_alloc(p, &d.dpiv, n6))) return st;
    if ((st = dev_alloc(p, &d.wpanel, n6 * 48))) return st;
  }
  if ((st = dev_alloc(p, &d.x, n6))) return st;
  if ((st = dev_alloc(p, &d.xdd, 2 * n6))) return st;
  if ((st = dev_alloc(p, &d.r, n6))) return st;
  SGBA_CK(cudaMemsetAsync(d.x, 0, sizeof(double) * std::max<size_t>(n6, 1), p->stream));
  SGBA_CK(cudaMemsetAsync(d.dm, 0, sizeof(double) * std::max<size_t>(3 * P.nm, 1), p->stream));
  d.part_cap = sgba::cost_partials_needed(s);
  if ((st = dev_alloc(p, &d.part, static_cast<size_t>(d.part_cap)))) return st;
  if ((st = dev_alloc(p, &d.ctrl, 1))) return st;
  SGBA_CK(cudaMemsetAsync(d.ctrl, 0, sizeof(Ctrl), p->stream));
  if ((st = dev_alloc(p, &d.last_rec, 1))) return st;
  SGBA_CK(cudaStreamSynchronize(p->stream));
  // The per-observation host tables are on the device now; the host keeps
  // only what the queries after creation read (counts, block maps, the S
  // pattern). Releasing the rest lets the next problem's set-up reuse the
  // memory instead of faulting in fresh pages.
  release(P.ord);
  release(P.obs_pose);
  release(P.obs_pt);
  release(P.g_begin);
  release(P.g_pose);
  release(P.g_pt);
  release(P.pt_g_begin);
  release(P.fb_pose);
  release(P.mb_pt);
  release(P.cam_g_begin);
  release(P.cam_g);
  release(P.tile_fb);
  release(P.tile_begin);
  release(P.tile_end);
  release(P.fb_tile_begin);
  release(P.chunk_begin);
  release(P.block_chunk_begin);
  return SGBA_OK;
}

// One LM iteration (Optimizer::step for the NLLS strategy).
int enqueue_iteration(sgba_problem* p, cudaStream_t st) {
  int n = 0;
  n += sgba::launch_iteration_begin(p->sz, p->d, st);
  n += sgba::launch_linearize(p->sz, p->d, 0.0, false, st);
  n += sgba::launch_schur(p->sz, p->d, st);
  n += sgba::launch_factor_solve(p->sz, p->d, st);
  n += sgba::launch_update(p->sz, p->d, st);
  n += sgba::launch_decide(p->sz, p->d, st);
  return n;
}

int ensure_graph(sgba_problem* p) {
  if (p->graph_exec) return SGBA_OK;
  SGBA_CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
  int n = enqueue_iteration(p, p->stream);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(p->stream, &g);
  if (e != cudaSuccess)
    return set_error(SGBA_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
  p->graph = g;
  SGBA_CK(cudaGraphInstantiate(&p->graph_exec, g, 0));
  p->iter_launches = n;
  return SGBA_OK;
}

int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(SGBA_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  return SGBA_OK;
}

}  // namespace

extern "C" {

int32_t sgba_abi_version(void) { return SGBA_ABI_VERSION; }

size_t sgba_last_error(char* buf, size_t cap) {
  if (buf && cap > 0) {
    size_t n = std::min(cap - 1, g_last_error.size());
    std::memcpy(buf, g_last_error.data(), n);
    buf[n] = '\0';
  }
  return g_last_error.size();
}

int sgba_problem_create(const sgba_problem_desc* desc, int32_t device, sgba_problem** out) {
  return sgba_problem_create_ex(desc, nullptr, device, out);
}

int sgba_problem_create_ex(const sgba_problem_desc* desc, const sgba_problem_options* opts, int32_t device,
                           sgba_problem** out) {
  return sgba_problem_create_graph(desc, opts, nullptr, device, out);
}

int sgba_problem_create_graph(const sgba_problem_desc* desc, const sgba_problem_options* opts,
                              const sgba_pose_graph* graph, int32_t device, sgba_problem** out) {
  if (!out) return set_error(SGBA_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!desc) return set_error(SGBA_ERR_INVALID_ARGUMENT, "desc is NULL");
  if (opts && opts->camera_model != SGBA_CAMERA_PINHOLE && opts->camera_model != SGBA_CAMERA_EUCM)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "camera model %d: expected SGBA_CAMERA_PINHOLE or SGBA_CAMERA_EUCM",
                     opts->camera_model);
  if (opts && opts->intrinsics_free != 0 && opts->intrinsics_free != 1)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "intrinsics_free must be 0 or 1");
  const bool eucm = opts && opts->camera_model == SGBA_CAMERA_EUCM;
  if (eucm && !(std::isfinite(opts->eucm_alpha_beta[0]) && std::isfinite(opts->eucm_alpha_beta[1])))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "non-finite EUCM alpha / beta");
  if (opts && !eucm && (opts->eucm_alpha_beta[0] != 0.0 || opts->eucm_alpha_beta[1] != 0.0))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "eucm_alpha_beta must be zero for the pinhole camera");
  sgba_problem* p = new (std::nothrow) sgba_problem();
  if (!p) return set_error(SGBA_ERR_OUT_OF_MEMORY, "host allocation failed");
  p->intr_free = (opts && opts->intrinsics_free) ? 1 : 0;
  p->camera_model = eucm ? SGBA_CAMERA_EUCM : SGBA_CAMERA_PINHOLE;
  if (eucm) {
    p->eucm_ab[0] = opts->eucm_alpha_beta[0];
    p->eucm_ab[1] = opts->eucm_alpha_beta[1];
  }
  int st = build_plan(desc, &p->plan);
  if (st) { delete p; return st; }
  if (graph && graph->n_edge != 0 && p->intr_free) {
    delete p;
    return set_error(SGBA_ERR_UNSUPPORTED, "pose-graph edges with free camera params are not on this path");
  }
  st = build_edges(graph, &p->plan);
  if (st) { delete p; return st; }
  if (p->plan.nf > kMaxDenseFree) {
    const int nf = p->plan.nf;
    delete p;
    return set_error(SGBA_ERR_UNSUPPORTED, "%d free poses exceed the dense reduced-camera-system limit (%d)",
                     nf, kMaxDenseFree);
  }
  int dev = device;
  if (dev < 0) {
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { delete p; return set_error(SGBA_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e)); }
  }
  p->device = dev;
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) { delete p; return set_error(SGBA_ERR_CUDA, "cudaSetDevice(%d): %s", dev, cudaGetErrorString(e)); }
  e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete p; return set_error(SGBA_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
  p->pool = problem_pool(dev);
  if (!p->pool) { sgba_problem_destroy(p); return set_error(SGBA_ERR_CUDA, "device memory pool of device %d", dev); }
  st = upload(p, desc);
  if (st) { sgba_problem_destroy(p); return st; }
  *out = p;
  return SGBA_OK;
}

int sgba_problem_destroy(sgba_problem* p) {
  if (!p) return SGBA_OK;
  cudaSetDevice(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  for (void* v : p->cov.allocs) cudaFreeAsync(v, p->stream);
  for (void* v : p->allocs) cudaFreeAsync(v, p->stream);  // back to the pool, in stream order
  if (p->flush_buf) cudaFree(p->flush_buf);
  if (p->d.records) cudaFree(p->d.records);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return SGBA_OK;
}

int sgba_optimizer_init(sgba_problem* p, const sgba_opt_params* prm) {
  if (!p || !prm) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  SGBA_CK(cudaSetDevice(p->device));
  // validate_solver_config (crates/sophus_opt/src/nlls/optimizer.rs:649-717)
  if ((p->plan.nf == 0 && !p->intr_free) || p->plan.nm == 0)
    return set_error(SGBA_ERR_SCHUR_MISSING_FREE_OR_MARG,
                     "Schur solver needs free and marginalized variables (free scalars %d, marg scalars %d)",
                     6 * p->plan.nf + (p->intr_free ? p->sz.intr_nk : 0), 3 * p->plan.nm);
  if (!std::isfinite(prm->initial_lm_damping))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "initial_lm_damping is not finite");
  p->params = *prm;
  const int cap = std::max(1, prm->num_iterations);
  if (p->d.record_cap < cap) {
    if (p->d.records) cudaFree(p->d.records);
    p->d.records = nullptr;
    SGBA_CK(cudaMalloc(&p->d.records, sizeof(Record) * cap));
    p->d.record_cap = cap;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  }
  int gst = ensure_graph(p);  // capture before any work is queued on the stream
  if (gst) return gst;
  Ctrl c;
  std::memset(&c, 0, sizeof(c));
  c.nu = prm->initial_lm_damping;
  c.ftol = prm->function_tolerance;
  c.gtol = prm->gradient_tolerance;
  c.ptol = prm->parameter_tolerance;
  c.rejects = 0;
  c.max_rejects = prm->max_consecutive_rejects;
  c.step = 0;
  c.num_iterations = prm->num_iterations;
  c.record_cap = cap;
  c.n_eq = p->sz.n_eq;
  c.eq_lambda = p->d.eq_lambda;
  c.eq_dlam = p->d.eq_dlam;
  if (p->sz.n_eq > 0)  // EqSystem::new: zero multipliers
    SGBA_CK(cudaMemsetAsync(p->d.eq_lambda, 0, sizeof(double) * p->sz.n_eq, p->stream));
  SGBA_CK(cudaMemcpyAsync(p->d.ctrl, &c, sizeof(Ctrl), cudaMemcpyHostToDevice, p->stream));
  sgba::launch_init_merit(p->sz, p->d, p->stream);
  int st = check_launch();
  if (st) return st;
  if (!p->defer_sync) SGBA_CK(cudaStreamSynchronize(p->stream));
  p->inited = true;
  return SGBA_OK;
}

int sgba_optimizer_step(sgba_problem* p, sgba_iter_record* rec) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  if (!p->inited) return set_error(SGBA_ERR_STATE, "sgba_optimizer_step before sgba_optimizer_init");
  SGBA_CK(cudaSetDevice(p->device));
  // Optimizer::step always performs a step; the done flag only stops the
  // device-side loop of sgba_optimize.
  const int zero = 0;
  SGBA_CK(cudaMemcpyAsync(reinterpret_cast<char*>(p->d.ctrl) + offsetof(Ctrl, done), &zero, sizeof(int),
                          cudaMemcpyHostToDevice, p->stream));
  SGBA_CK(cudaGraphLaunch(p->graph_exec, p->stream));
  Record r;
  SGBA_CK(cudaMemcpyAsync(&r, p->d.last_rec, sizeof(Record), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  if (rec) std::memcpy(rec, &r, sizeof(Record));
  return SGBA_OK;
}

int sgba_optimize(sgba_problem* p, const sgba_opt_params* prm, sgba_iter_record* records, int32_t cap,
                  int32_t* n_records, int32_t* termination) {
  if (!p || !prm) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  EventSet events;  // every event below is destroyed on every return path
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  SGBA_CK(cudaSetDevice(p->device));
  SGBA_CK(events.create(&e0));
  SGBA_CK(events.create(&e1));
  int st = sgba_optimizer_init(p, prm);
  if (st) return st;
  SGBA_CK(cudaEventRecord(e0, p->stream));
  const int iters = std::max(1, prm->num_iterations);
  double ph[5] = {0, 0, 0, 0, 0};
  if (!p->profiling) {
    for (int it = 0; it < iters; ++it) SGBA_CK(cudaGraphLaunch(p->graph_exec, p->stream));
  } else {
    // Same kernels launched directly, with events between the phases.
    cudaEvent_t ev[6];
    for (auto& x : ev) SGBA_CK(events.create(&x));
    for (int it = 0; it < iters; ++it) {
      SGBA_CK(cudaEventRecord(ev[0], p->stream));
      sgba::launch_iteration_begin(p->sz, p->d, p->stream);
      sgba::launch_linearize(p->sz, p->d, 0.0, false, p->stream);
      SGBA_CK(cudaEventRecord(ev[1], p->stream));
      sgba::launch_schur(p->sz, p->d, p->stream);
      SGBA_CK(cudaEventRecord(ev[2], p->stream));
      sgba::launch_factor_solve(p->sz, p->d, p->stream);
      SGBA_CK(cudaEventRecord(ev[3], p->stream));
      sgba::launch_update(p->sz, p->d, p->stream);
      SGBA_CK(cudaEventRecord(ev[4], p->stream));
      sgba::launch_decide(p->sz, p->d, p->stream);
      SGBA_CK(cudaEventRecord(ev[5], p->stream));
      SGBA_CK(cudaEventSynchronize(ev[5]));
      for (int k = 0; k < 5; ++k) {
        float m = 0.f;
        cudaEventElapsedTime(&m, ev[k], ev[k + 1]);
        ph[k] += m;
      }
    }
  }
  // build_solution (optimizer.rs:609-646): final linearisation with zero
  // damping (or the current damping when skip_final_hessian is set).
  Ctrl c;
  SGBA_CK(cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  int final_launches = sgba::launch_linearize(p->sz, p->d, prm->skip_final_hessian ? c.nu : 0.0, true, p->stream);
  SGBA_CK(cudaEventRecord(e1, p->stream));
  st = check_launch();
  if (st) return st;
  SGBA_CK(cudaStreamSynchronize(p->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const int nrec = std::min(c.step, p->d.record_cap);
  if (records && cap > 0) {
    std::vector<Record> h(nrec);
    if (nrec > 0) SGBA_CK(cudaMemcpy(h.data(), p->d.records, sizeof(Record) * nrec, cudaMemcpyDeviceToHost));
    std::memcpy(records, h.data(), sizeof(Record) * std::min(nrec, cap));
  }
  if (n_records) *n_records = c.step;
  if (termination) *termination = c.termination;
  p->prof.kernel_launches = 3 + static_cast<int64_t>(iters) * p->iter_launches + final_launches;
  p->prof.ms_total = ms;
  p->prof.ms_linearize = ph[0];
  p->prof.ms_schur = ph[1];
  p->prof.ms_factor = ph[2];
  p->prof.ms_update = ph[3];
  p->prof.ms_cost = ph[4];
  return SGBA_OK;
}

int sgba_get_variables(sgba_problem* p, double* poses, double* points) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  SGBA_CK(cudaSetDevice(p->device));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  if (poses) SGBA_CK(cudaMemcpy(poses, p->d.poses, sizeof(double) * 7 * p->plan.nc, cudaMemcpyDeviceToHost));
  if (points && p->plan.np > 0)
    SGBA_CK(cudaMemcpy(points, p->d.points, sizeof(double) * 3 * p->plan.np, cudaMemcpyDeviceToHost));
  return SGBA_OK;
}

int sgba_set_pose_priors(sgba_problem* p, int32_t n, const int32_t* pose, const double* mean,
                         const double* precision) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  if (n < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "negative prior count");
  if (n > 0 && (!pose || !mean || !precision)) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (p->intr_free) return set_error(SGBA_ERR_UNSUPPORTED, "pose priors with free camera params are not on this path");
  const Plan& P = p->plan;
  for (int32_t k = 0; k < n; ++k) {
    if (pose[k] < 0 || pose[k] >= P.nc)
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "prior %d: pose index %d out of range", k, pose[k]);
    if (!finite_all(mean + 7 * k, 7) || !finite_all(precision + 36 * static_cast<int64_t>(k), 36))
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "prior %d: non-finite mean or precision", k);
    if (!quat_valid(mean + 7 * k)) return set_error(SGBA_ERR_INVALID_PARAMS, "prior %d: invalid quaternion", k);
  }
  SGBA_CK(cudaSetDevice(p->device));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  Dev& d = p->d;
  Sizes& s = p->sz;
  // CostFn::sort order: by pose, stable
  std::vector<int32_t> ord(n);
  for (int32_t k = 0; k < n; ++k) ord[k] = k;
  std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return pose[a] < pose[b]; });
  std::vector<int32_t> hp(n), hfb(n), beg(P.nf + 1, 0);
  std::vector<double> hm(7 * static_cast<size_t>(n)), hw(36 * static_cast<size_t>(n));
  for (int32_t k = 0; k < n; ++k) {
    const int32_t o = ord[k];
    hp[k] = pose[o];
    hfb[k] = P.pose_fb[pose[o]];
    std::memcpy(&hm[7 * k], mean + 7 * o, sizeof(double) * 7);
    if (!(0.0 <= hm[7 * k]))
      for (int q = 0; q < 4; ++q) hm[7 * k + q] = -hm[7 * k + q];
    std::memcpy(&hw[36 * static_cast<size_t>(k)], precision + 36 * static_cast<int64_t>(o), sizeof(double) * 36);
    if (hfb[k] >= 0) ++beg[hfb[k] + 1];
  }
  for (int f = 0; f < P.nf; ++f) beg[f + 1] += beg[f];
  // damping once per pose with a prior (one reduced term of the prior cost function)
  if (p->gauge_base < 0) {
    p->cnt_f_base = P.cnt_f;
    p->gauge_base = s.gauge_kind;
  }
  std::vector<double> cnt = p->cnt_f_base;
  for (int f = 0; f < P.nf; ++f)
    if (beg[f + 1] > beg[f]) cnt[f] += 1.0;
  int st;
  if (n > d.prior_cap) {
    if ((st = dev_alloc(p, &d.prior_pose, static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.prior_fb, static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.prior_mean, 7 * static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.prior_W, 36 * static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.prior_out, static_cast<size_t>(sgba::kPriorOut) * n))) return st;
    d.prior_cap = n;
  }
  if (!d.prior_fb_begin && (st = dev_alloc(p, &d.prior_fb_begin, static_cast<size_t>(P.nf) + 1))) return st;
  if (n > 0) {
    SGBA_CK(cudaMemcpyAsync(d.prior_pose, hp.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
    SGBA_CK(cudaMemcpyAsync(d.prior_fb, hfb.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
    SGBA_CK(cudaMemcpyAsync(d.prior_mean, hm.data(), sizeof(double) * hm.size(), cudaMemcpyHostToDevice, p->stream));
    SGBA_CK(cudaMemcpyAsync(d.prior_W, hw.data(), sizeof(double) * hw.size(), cudaMemcpyHostToDevice, p->stream));
  }
  SGBA_CK(cudaMemcpyAsync(d.prior_fb_begin, beg.data(), sizeof(int32_t) * beg.size(), cudaMemcpyHostToDevice,
                          p->stream));
  if (P.nf > 0)
    SGBA_CK(cudaMemcpyAsync(d.cnt_f, cnt.data(), sizeof(double) * P.nf, cudaMemcpyHostToDevice, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  p->plan.cnt_f = cnt;
  s.n_prior = n;
  // the priors hold the gauge: no projection along the scale direction
  s.gauge_kind = (n > 0 || s.n_eq > 0) ? 0 : p->gauge_base;
  // the iteration graph is captured again with the prior launches
  if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
  if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  p->inited = false;
  return SGBA_OK;
}

int sgba_set_eq_constraints(sgba_problem* p, int32_t n, const int32_t* pose, const double* radius) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  if (n < 0 || n > sgba::kMaxEq)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "%d constraints: expected 0 .. %d", n, sgba::kMaxEq);
  if (n > 0 && (!pose || !radius)) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  const Plan& P = p->plan;
  Sizes& s = p->sz;
  for (int32_t k = 0; k < n; ++k) {
    if (pose[k] < 0 || pose[k] >= P.nc)
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "constraint %d: pose index %d out of range", k, pose[k]);
    if (P.pose_fb[pose[k]] < 0)
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "constraint %d: pose %d is constant", k, pose[k]);
    if (!std::isfinite(radius[k])) return set_error(SGBA_ERR_INVALID_ARGUMENT, "constraint %d: radius", k);
  }
  if (n > 0 && s.pcg_mode)
    return set_error(SGBA_ERR_UNSUPPORTED, "equality constraints with the PCG solver are not on this path");
  if (n > 0 && !s.small_dense)
    return set_error(SGBA_ERR_UNSUPPORTED,
                     "equality constraints run on the one-CTA solver (reduced systems of at most 234 rows)");
  SGBA_CK(cudaSetDevice(p->device));
  if (n > 0 && !sgba::small_dense_setup_eq(s.n6, n))
    return set_error(SGBA_ERR_UNSUPPORTED, "%d constraints on a %d-row reduced system exceed the shared memory", n,
                     s.n6);
  SGBA_CK(cudaStreamSynchronize(p->stream));
  Dev& d = p->d;
  int st;
  if (n > d.eq_cap) {
    if ((st = dev_alloc(p, &d.eq_pose, static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.eq_fb, static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.eq_radius, static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.eq_c, static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.eq_jac, 3 * static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.eq_lambda, static_cast<size_t>(n)))) return st;
    if ((st = dev_alloc(p, &d.eq_dlam, static_cast<size_t>(n)))) return st;
    d.eq_cap = n;
  }
  if (n > 0) {
    std::vector<int32_t> fb(n);
    for (int32_t k = 0; k < n; ++k) fb[k] = P.pose_fb[pose[k]];
    SGBA_CK(cudaMemcpyAsync(d.eq_pose, pose, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
    SGBA_CK(cudaMemcpyAsync(d.eq_fb, fb.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
    SGBA_CK(cudaMemcpyAsync(d.eq_radius, radius, sizeof(double) * n, cudaMemcpyHostToDevice, p->stream));
    SGBA_CK(cudaMemsetAsync(d.eq_dlam, 0, sizeof(double) * n, p->stream));
    SGBA_CK(cudaStreamSynchronize(p->stream));
  }
  if (p->gauge_base < 0) {
    p->cnt_f_base = P.cnt_f;
    p->gauge_base = s.gauge_kind;
  }
  s.n_eq = n;
  // the constraints fix the scale: no gauge projection
  s.gauge_kind = (n > 0 || s.n_prior > 0) ? 0 : p->gauge_base;
  if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
  if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  p->inited = false;
  return SGBA_OK;
}

int sgba_set_variables(sgba_problem* p, const double* poses, const double* points) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  SGBA_CK(cudaSetDevice(p->device));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  if (poses) {
    std::vector<double> h(poses, poses + 7 * p->plan.nc);
    if (!finite_all(h.data(), static_cast<int64_t>(h.size())))
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "non-finite pose");
    for (int j = 0; j < p->plan.nc; ++j) {
      if (!quat_valid(&h[7 * j])) return set_error(SGBA_ERR_INVALID_PARAMS, "pose %d: invalid quaternion", j);
      if (!(0.0 <= h[7 * j]))
        for (int k = 0; k < 4; ++k) h[7 * j + k] = -h[7 * j + k];
    }
    SGBA_CK(cudaMemcpy(p->d.poses, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
  }
  if (points && p->plan.np > 0) {
    if (!finite_all(points, 3ll * p->plan.np)) return set_error(SGBA_ERR_INVALID_ARGUMENT, "non-finite point");
    SGBA_CK(cudaMemcpy(p->d.points, points, sizeof(double) * 3 * p->plan.np, cudaMemcpyHostToDevice));
  }
  p->inited = false;
  return SGBA_OK;
}

int sgba_get_intrinsics(sgba_problem* p, double* intrinsics) {
  if (!p || !intrinsics) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  SGBA_CK(cudaSetDevice(p->device));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  SGBA_CK(cudaMemcpy(intrinsics, p->d.intr, sizeof(double) * p->sz.intr_nk, cudaMemcpyDeviceToHost));
  return SGBA_OK;
}

int sgba_get_cost(sgba_problem* p, double* cost) {
  if (!p || !cost) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->inited) return set_error(SGBA_ERR_STATE, "no optimizer state (call sgba_optimizer_init)");
  SGBA_CK(cudaSetDevice(p->device));
  Ctrl c;
  SGBA_CK(cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  *cost = c.merit;
  return SGBA_OK;
}

int sgba_get_layout(sgba_problem* p, sgba_layout* out) {
  if (!p || !out) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  out->n_free_poses = p->plan.nf;
  out->n_marg_points = p->plan.nm;
  out->n_terms = p->plan.ng;
  out->n_h_blocks = p->plan.n_h_blocks;
  out->n_s_blocks = p->sz.nsb;
  out->intrinsics_rows = p->intr_free ? 6 : 0;
  if (p->intr_free) {
    // the intrinsics block, its coupling to every free pose and marg point with terms
    int64_t fh = 0, mh = 0;
    for (int f = 0; f < p->plan.nf; ++f) fh += p->plan.cnt_f[f] > 0;
    for (int m = 0; m < p->plan.nm; ++m) mh += p->plan.cnt_m[m] > 0;
    out->n_h_blocks += 1 + fh + mh;
    out->n_s_blocks += 1 + fh;
  }
  int64_t np = 0;
  if (!p->plan.sb_pair_begin.empty()) np = p->plan.sb_pair_begin.back();
  out->n_schur_pairs = np;
  out->solver = p->sz.small_dense   ? SGBA_SOLVER_DENSE_SMALL
                : p->sz.dense_c > 0 ? SGBA_SOLVER_DENSE_CLUSTER
                                    : (p->sz.band_c > 0 ? SGBA_SOLVER_BAND : SGBA_SOLVER_DENSE_PANELS);
  out->band_width = p->sz.band_c > 0 ? p->sz.band_w : 0;
  out->border_rows = p->sz.band_c > 0 ? p->sz.n6 - p->sz.band_rows : 0;
  out->float_float_lin = p->sz.lin_dd;
  return SGBA_OK;
}

int sgba_export_pattern(sgba_problem* p, int32_t* h_rows, int32_t* h_cols, int32_t* s_rows, int32_t* s_cols) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  const Plan& P = p->plan;
  if (h_rows && h_cols) {
    // the pose and point of every reduced term, read back from the device
    std::vector<int32_t> g_pose(P.ng), g_pt(P.ng);
    SGBA_CK(cudaSetDevice(p->device));
    if (P.ng > 0) {
      SGBA_CK(cudaMemcpy(g_pose.data(), p->d.g_pose, sizeof(int32_t) * P.ng, cudaMemcpyDeviceToHost));
      SGBA_CK(cudaMemcpy(g_pt.data(), p->d.g_pt, sizeof(int32_t) * P.ng, cudaMemcpyDeviceToHost));
    }
    // global block order: the intrinsics (when free), free poses, marg points
    const int o = p->intr_free ? 1 : 0;
    int64_t k = 0;
    if (o) { h_rows[k] = 0; h_cols[k] = 0; ++k; }
    for (int f = 0; f < P.nf; ++f)
      if (P.cnt_f[f] > 0) { h_rows[k] = o + f; h_cols[k] = o + f; ++k; }
    for (int m = 0; m < P.nm; ++m)
      if (P.cnt_m[m] > 0) { h_rows[k] = o + P.nf + m; h_cols[k] = o + P.nf + m; ++k; }
    for (int64_t g = 0; g < P.ng; ++g) {
      int fb = P.pose_fb[g_pose[g]], mb = P.pt_mb[g_pt[g]];
      if (fb >= 0 && mb >= 0) { h_rows[k] = o + P.nf + mb; h_cols[k] = o + fb; ++k; }
    }
    if (o) {
      for (int f = 0; f < P.nf; ++f)
        if (P.cnt_f[f] > 0) { h_rows[k] = 1 + f; h_cols[k] = 0; ++k; }
      for (int m = 0; m < P.nm; ++m)
        if (P.cnt_m[m] > 0) { h_rows[k] = 1 + P.nf + m; h_cols[k] = 0; ++k; }
    }
  }
  if (s_rows && s_cols) {
    const int o = p->intr_free ? 1 : 0;
    size_t k = 0;
    if (o) { s_rows[k] = 0; s_cols[k] = 0; ++k; }
    for (size_t b = 0; b < P.sb_row.size(); ++b, ++k) {
      s_rows[k] = o + P.sb_row[b];
      s_cols[k] = o + P.sb_col[b];
    }
    if (o)
      for (int f = 0; f < P.nf; ++f)
        if (P.cnt_f[f] > 0) { s_rows[k] = 1 + f; s_cols[k] = 0; ++k; }
  }
  return SGBA_OK;
}

int sgba_debug_last_system(sgba_problem* p, double* s_dense, double* rhs, double* delta) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  SGBA_CK(cudaSetDevice(p->device));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  const size_t n6 = static_cast<size_t>(p->sz.n6);
  if (s_dense) SGBA_CK(cudaMemcpy(s_dense, p->d.S, sizeof(double) * n6 * n6, cudaMemcpyDeviceToHost));
  if (rhs) SGBA_CK(cudaMemcpy(rhs, p->d.rb, sizeof(double) * n6, cudaMemcpyDeviceToHost));
  if (delta) {
    SGBA_CK(cudaMemcpy(delta, p->d.x, sizeof(double) * n6, cudaMemcpyDeviceToHost));
    if (p->plan.nm > 0)
      SGBA_CK(cudaMemcpy(delta + n6, p->d.dm, sizeof(double) * 3 * p->plan.nm, cudaMemcpyDeviceToHost));
  }
  if (p->intr_free) {
    // internally the intrinsics block is last; the reference's order puts it first
    const size_t kp = n6 - 6;
    auto perm = [kp](size_t i) { return i < 6 ? kp + i : i - 6; };  // exported index -> internal
    if (s_dense) {
      std::vector<double> t(s_dense, s_dense + n6 * n6);
      for (size_t i = 0; i < n6; ++i)
        for (size_t j = 0; j < n6; ++j) s_dense[i * n6 + j] = t[perm(i) * n6 + perm(j)];
    }
    if (rhs) {
      std::vector<double> t(rhs, rhs + n6);
      for (size_t i = 0; i < n6; ++i) rhs[i] = t[perm(i)];
    }
    if (delta) {
      std::vector<double> t(delta, delta + n6);
      for (size_t i = 0; i < n6; ++i) delta[i] = t[perm(i)];
    }
  }
  return SGBA_OK;
}

int sgba_debug_jacobians(sgba_problem* p, int64_t n, const int32_t* cam, const int32_t* pt, int32_t precision,
                         double* j_pose, double* j_point) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  if (n < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "negative term count");
  if (n > 0 && (!cam || !pt || !j_pose || !j_point)) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (precision != 0 && precision != 1) return set_error(SGBA_ERR_INVALID_ARGUMENT, "precision must be 0 or 1");
  for (int64_t i = 0; i < n; ++i) {
    if (cam[i] < 0 || cam[i] >= p->plan.nc || pt[i] < 0 || pt[i] >= p->plan.np)
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "term %lld: camera %d / point %d out of range",
                       static_cast<long long>(i), cam[i], pt[i]);
  }
  if (n == 0) return SGBA_OK;
  SGBA_CK(cudaSetDevice(p->device));
  // one pool allocation: cam, pt (int32) then J_pose, J_point (f64)
  const size_t idx_bytes = (sizeof(int32_t) * 2 * static_cast<size_t>(n) + 255) & ~size_t(255);
  const size_t bytes = idx_bytes + sizeof(double) * 18 * static_cast<size_t>(n);
  void* buf = nullptr;
  SGBA_CK(cudaMallocFromPoolAsync(&buf, bytes, p->pool, p->stream));
  int32_t* dcam = static_cast<int32_t*>(buf);
  int32_t* dpt = dcam + n;
  double* djp = reinterpret_cast<double*>(static_cast<char*>(buf) + idx_bytes);
  double* djm = djp + 12 * n;
  cudaError_t e = cudaMemcpyAsync(dcam, cam, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dpt, pt, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess) e = sgba::launch_debug_jacobians(p->sz, p->d, n, dcam, dpt, precision, djp, djm, p->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(j_pose, djp, sizeof(double) * 12 * n, cudaMemcpyDeviceToHost, p->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(j_point, djm, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, p->stream);
  cudaFreeAsync(buf, p->stream);
  const cudaError_t es = cudaStreamSynchronize(p->stream);
  if (e == cudaSuccess) e = es;
  if (e != cudaSuccess) return set_error(SGBA_ERR_CUDA, "sgba_debug_jacobians: %s", cudaGetErrorString(e));
  return SGBA_OK;
}

// State blob: magic, sizes, LM scalars, poses, points.
// ---------------------------------------------------------------------------
// Covariance and precision queries of the solution (sgba_cov.cu)
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

void cov_free(sgba_problem* p) {
  for (void* v : p->cov.allocs) cudaFreeAsync(v, p->stream);
  p->cov = sgba::CovBufs{};
}

template <class T>
int cov_alloc(sgba_problem* p, T** ptr, size_t count) {
  void* v = nullptr;
  SGBA_CK(cudaMallocFromPoolAsync(&v, sizeof(T) * std::max<size_t>(count, 1), p->pool, p->stream));
  p->cov.allocs.push_back(v);
  *ptr = static_cast<T*>(v);
  return SGBA_OK;
}

}  // namespace

extern "C" {

int sgba_covariance_release(sgba_problem* p) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  SGBA_CK(cudaSetDevice(p->device));
  cov_free(p);
  SGBA_CK(cudaStreamSynchronize(p->stream));
  return SGBA_OK;
}

int sgba_covariance_prepare(sgba_problem* p, sgba_cov_info* info) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  if (p->sz.n_eq > 0)
    return set_error(SGBA_ERR_UNSUPPORTED, "covariance queries with equality constraints are not on the GPU path");
  if (p->plan.nf > kMaxDenseFree)
    return set_error(SGBA_ERR_UNSUPPORTED, "covariance: %d free poses (at most %d)", p->plan.nf, kMaxDenseFree);
  SGBA_CK(cudaSetDevice(p->device));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  cov_free(p);
  const sgba::Sizes& s = p->sz;
  const sgba::Dev& d = p->d;
  sgba::CovBufs& c = p->cov;
  c.nci = p->intr_free ? 6 : 0;
  c.nk = p->intr_free ? s.intr_nk : 0;
  const int n = c.nci + 6 * p->plan.nf;
  const size_t nn = static_cast<size_t>(n) * n;
  c.n = n;
  int st;
  if (p->intr_free) {
    if ((st = cov_alloc(p, &c.crec, static_cast<size_t>(sgba::kCovCamRec) * std::max<int64_t>(s.ng, 1)))) return st;
    if ((st = cov_alloc(p, &c.wc, 18 * static_cast<size_t>(std::max(s.nm, 1))))) return st;
    if ((st = cov_alloc(p, &c.yc, 18 * static_cast<size_t>(std::max(s.nm, 1))))) return st;
    if ((st = cov_alloc(p, &c.hcc, 36))) return st;
    if ((st = cov_alloc(p, &c.hcp, 36 * static_cast<size_t>(std::max(s.nf, 1))))) return st;
  }
  if ((st = cov_alloc(p, &c.rec, static_cast<size_t>(sgba::kCovRec) * s.ng))) return st;
  if ((st = cov_alloc(p, &c.y, 18 * static_cast<size_t>(s.ng)))) return st;
  if ((st = cov_alloc(p, &c.vinv, 9 * static_cast<size_t>(s.nm)))) return st;
  if ((st = cov_alloc(p, &c.hdiag, 36 * static_cast<size_t>(s.nf)))) return st;
  if ((st = cov_alloc(p, &c.S, nn))) return st;
  if ((st = cov_alloc(p, &c.Z, nn))) return st;
  if ((st = cov_alloc(p, &c.ldiag, 6 * static_cast<size_t>(n)))) return st;
  if ((st = cov_alloc(p, &c.dpiv, static_cast<size_t>(n)))) return st;
  if ((st = cov_alloc(p, &c.work, sgba::cov_inverse_work(n)))) return st;
  if ((st = cov_alloc(p, &c.status, 2))) return st;
  cudaStream_t str = p->stream;
  EventSet evs;
  cudaEvent_t ev[4];
  for (cudaEvent_t& e : ev) SGBA_CK(evs.create(&e));
  SGBA_CK(cudaMemsetAsync(c.status, 0, 2 * sizeof(int), str));
  SGBA_CK(cudaMemsetAsync(c.y, 0, sizeof(double) * 18 * std::max<int64_t>(s.ng, 1), str));
  if (nn) SGBA_CK(cudaMemsetAsync(c.S, 0, sizeof(double) * nn, str));
  SGBA_CK(cudaEventRecord(ev[0], str));
  int launches = 0;
  // the pose-only cost functions' blocks at the current poses
  launches += sgba::launch_prior_eval(s, d, d.poses, 1, 0, nullptr, str);
  launches += sgba::launch_edge_eval(s, d, d.poses, 1, 0, nullptr, str);
  launches += sgba::launch_cov_assemble(s, d, c, str);
  SGBA_CK(cudaGetLastError());
  SGBA_CK(cudaEventRecord(ev[1], str));
  if (n > 0) launches += sgba::launch_cov_factor(n, c.S, c.ldiag, c.dpiv, c.status, str);
  SGBA_CK(cudaGetLastError());
  SGBA_CK(cudaEventRecord(ev[2], str));
  int hst[2] = {0, 0};
  std::vector<double> piv(n);
  SGBA_CK(cudaMemcpyAsync(hst, c.status, sizeof(hst), cudaMemcpyDeviceToHost, str));
  if (n > 0) SGBA_CK(cudaMemcpyAsync(piv.data(), c.dpiv, sizeof(double) * n, cudaMemcpyDeviceToHost, str));
  SGBA_CK(cudaStreamSynchronize(str));
  if (hst[1]) {
    cov_free(p);
    return set_error(SGBA_ERR_FACTORIZATION, "covariance: a marginalized point's H block is singular");
  }
  if (hst[0]) {
    cov_free(p);
    return set_error(SGBA_ERR_FACTORIZATION, "covariance: S could not be factored (%s)",
                     hst[0] == 1 ? "a non-finite pivot" : "an indefinite block");
  }
  std::vector<int32_t> J;
  for (int j = 0; j < n; ++j)
    if (piv[j] > 0.0) J.push_back(j);
  c.rank = static_cast<int>(J.size());
  if (n > 0) {
    if (c.rank == n) {
      launches += sgba::launch_cov_inverse(n, c.S, c.ldiag, c.dpiv, c.Z, c.work, str);
    } else {
      int g_ok = 1;
      SGBA_CK(sgba::cov_pinv(n, c.S, c.ldiag, c.dpiv, J, c.Z, p->pool, str, &g_ok));
      if (!g_ok) {
        cov_free(p);
        return set_error(SGBA_ERR_FACTORIZATION, "covariance: E^T E of the positive-pivot columns is singular");
      }
    }
  }
  SGBA_CK(cudaGetLastError());
  SGBA_CK(cudaEventRecord(ev[3], str));
  SGBA_CK(cudaStreamSynchronize(str));
  c.ready = 1;
  if (info) {
    info->n = n;
    info->rank = c.rank;
    info->kernel_launches = launches;
    info->pad = 0;
    float ms = 0.f;
    SGBA_CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    info->ms_assemble = ms;
    SGBA_CK(cudaEventElapsedTime(&ms, ev[1], ev[2]));
    info->ms_factor = ms;
    SGBA_CK(cudaEventElapsedTime(&ms, ev[2], ev[3]));
    info->ms_inverse = ms;
  }
  return SGBA_OK;
}

int sgba_covariance_blocks(sgba_problem* p, int32_t mode, int32_t n, const sgba_cov_query* queries, double* out,
                           int32_t* dims) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  if (mode != SGBA_QUERY_COVARIANCE && mode != SGBA_QUERY_PRECISION)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "unknown query mode %d", mode);
  if (n < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "negative query count");
  if (n > 0 && (!queries || !out || !dims)) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->cov.ready) return set_error(SGBA_ERR_STATE, "covariance queries need sgba_covariance_prepare first");
  for (int32_t i = 0; i < n; ++i) {
    const sgba_cov_query& q = queries[i];
    for (int32_t kind : {q.row_kind, q.col_kind})
      if (kind != SGBA_VAR_INTRINSICS && kind != SGBA_VAR_POSE && kind != SGBA_VAR_POINT)
        return set_error(SGBA_ERR_INVALID_ARGUMENT, "query %d: unknown variable kind %d", i, kind);
  }
  if (n == 0) return SGBA_OK;
  SGBA_CK(cudaSetDevice(p->device));
  const size_t qbytes = (sizeof(int32_t) * 4 * static_cast<size_t>(n) + 255) & ~size_t(255);
  const size_t obytes = sizeof(double) * 36 * static_cast<size_t>(n);
  void* buf = nullptr;
  SGBA_CK(cudaMallocFromPoolAsync(&buf, qbytes + obytes + sizeof(int32_t) * 2 * static_cast<size_t>(n), p->pool,
                                  p->stream));
  int32_t* dq = static_cast<int32_t*>(buf);
  double* dout = reinterpret_cast<double*>(static_cast<char*>(buf) + qbytes);
  int32_t* ddims = reinterpret_cast<int32_t*>(static_cast<char*>(buf) + qbytes + obytes);
  static_assert(sizeof(sgba_cov_query) == 4 * sizeof(int32_t), "query layout");
  cudaError_t e = cudaMemcpyAsync(dq, queries, sizeof(int32_t) * 4 * n, cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess) e = sgba::launch_cov_query(p->sz, p->d, p->cov, mode, n, dq, dout, ddims, p->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, obytes, cudaMemcpyDeviceToHost, p->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dims, ddims, sizeof(int32_t) * 2 * n, cudaMemcpyDeviceToHost, p->stream);
  const cudaError_t ef = cudaFreeAsync(buf, p->stream);
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
  SGBA_CK(e);
  return SGBA_OK;
}

int sgba_state_save(sgba_problem* p, void* buf, size_t* size) {
  if (!p || !size) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  const size_t need = 64 + sizeof(double) * (7 * static_cast<size_t>(p->plan.nc) + 3 * static_cast<size_t>(p->plan.np) + kIntrMax);
  if (!buf) { *size = need; return SGBA_OK; }
  if (*size < need) return set_error(SGBA_ERR_INVALID_ARGUMENT, "state buffer too small (%zu < %zu)", *size, need);
  if (!p->inited) return set_error(SGBA_ERR_STATE, "no optimizer state to save");
  SGBA_CK(cudaSetDevice(p->device));
  Ctrl c;
  SGBA_CK(cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  char* b = static_cast<char*>(buf);
  std::memset(b, 0, 64);
  const uint64_t magic = 0x5347424153544131ull;  // "SGBASTA1"
  std::memcpy(b, &magic, 8);
  int32_t nc = p->plan.nc, np = p->plan.np;
  std::memcpy(b + 8, &nc, 4);
  std::memcpy(b + 12, &np, 4);
  std::memcpy(b + 16, &c.nu, 8);
  std::memcpy(b + 24, &c.merit, 8);
  int64_t rej = c.rejects, stp = c.step;
  std::memcpy(b + 32, &rej, 8);
  std::memcpy(b + 40, &stp, 8);
  SGBA_CK(cudaMemcpy(b + 64, p->d.poses, sizeof(double) * 7 * nc, cudaMemcpyDeviceToHost));
  if (np > 0) SGBA_CK(cudaMemcpy(b + 64 + sizeof(double) * 7 * nc, p->d.points, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost));
  SGBA_CK(cudaMemcpy(b + need - sizeof(double) * kIntrMax, p->d.intr, sizeof(double) * kIntrMax,
                     cudaMemcpyDeviceToHost));
  *size = need;
  return SGBA_OK;
}

int sgba_state_load(sgba_problem* p, const void* buf, size_t size) {
  if (!p || !buf) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->inited) return set_error(SGBA_ERR_STATE, "call sgba_optimizer_init before sgba_state_load");
  const char* b = static_cast<const char*>(buf);
  const size_t need = 64 + sizeof(double) * (7 * static_cast<size_t>(p->plan.nc) + 3 * static_cast<size_t>(p->plan.np) + kIntrMax);
  uint64_t magic;
  int32_t nc, np;
  if (size < need) return set_error(SGBA_ERR_INVALID_ARGUMENT, "state blob too small");
  std::memcpy(&magic, b, 8);
  std::memcpy(&nc, b + 8, 4);
  std::memcpy(&np, b + 12, 4);
  if (magic != 0x5347424153544131ull || nc != p->plan.nc || np != p->plan.np)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "state blob does not match this problem");
  SGBA_CK(cudaSetDevice(p->device));
  Ctrl c;
  SGBA_CK(cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  int64_t rej, stp;
  std::memcpy(&c.nu, b + 16, 8);
  std::memcpy(&c.merit, b + 24, 8);
  std::memcpy(&rej, b + 32, 8);
  std::memcpy(&stp, b + 40, 8);
  c.rejects = rej;
  c.step = static_cast<int>(stp);
  c.done = 0;
  SGBA_CK(cudaMemcpy(p->d.poses, b + 64, sizeof(double) * 7 * nc, cudaMemcpyHostToDevice));
  if (np > 0) SGBA_CK(cudaMemcpy(p->d.points, b + 64 + sizeof(double) * 7 * nc, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
  SGBA_CK(cudaMemcpy(p->d.intr, b + need - sizeof(double) * kIntrMax, sizeof(double) * kIntrMax,
                     cudaMemcpyHostToDevice));
  SGBA_CK(cudaMemcpy(p->d.intr_t, b + need - sizeof(double) * kIntrMax, sizeof(double) * kIntrMax,
                     cudaMemcpyHostToDevice));
  SGBA_CK(cudaMemcpy(p->d.ctrl, &c, sizeof(Ctrl), cudaMemcpyHostToDevice));
  // residuals of the loaded state
  sgba::launch_init_merit(p->sz, p->d, p->stream);
  SGBA_CK(cudaMemcpyAsync(reinterpret_cast<char*>(p->d.ctrl) + offsetof(Ctrl, merit), b + 24, 8,
                          cudaMemcpyHostToDevice, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  return check_launch();
}

static int bench_prepare(sgba_problem* p, bool flush) {
  if (!p->inited) return set_error(SGBA_ERR_STATE, "benchmark hooks need sgba_optimizer_init");
  SGBA_CK(cudaSetDevice(p->device));
  if (flush && !p->flush_buf) SGBA_CK(cudaMalloc(&p->flush_buf, size_t(256) << 20));
  // clear done / skip so the kernels do their work
  const int zero[2] = {0, 0};
  SGBA_CK(cudaMemcpyAsync(reinterpret_cast<char*>(p->d.ctrl) + offsetof(Ctrl, done), zero, 2 * sizeof(int),
                          cudaMemcpyHostToDevice, p->stream));
  return SGBA_OK;
}

int sgba_bench_iterations(sgba_problem* p, int32_t iters, int32_t flush_l2, double* ms_sum, int64_t* launches) {
  if (!p || !ms_sum) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  int st = bench_prepare(p, flush_l2 != 0);
  if (st) return st;
  EventSet events;
  cudaEvent_t a, b;
  SGBA_CK(events.create(&a));
  SGBA_CK(events.create(&b));
  double total = 0.0;
  for (int i = 0; i < iters; ++i) {
    if (flush_l2) SGBA_CK(cudaMemsetAsync(p->flush_buf, i & 0xff, size_t(256) << 20, p->stream));
    SGBA_CK(cudaEventRecord(a, p->stream));
    SGBA_CK(cudaGraphLaunch(p->graph_exec, p->stream));
    SGBA_CK(cudaEventRecord(b, p->stream));
    SGBA_CK(cudaEventSynchronize(b));
    float ms = 0.f;
    SGBA_CK(cudaEventElapsedTime(&ms, a, b));
    total += ms;
  }
  *ms_sum = total;
  if (launches) *launches = static_cast<int64_t>(iters) * p->iter_launches;
  return SGBA_OK;
}

int sgba_bench_kernel(sgba_problem* p, int32_t kernel, int32_t reps, int32_t flush_l2, double* ms_avg) {
  if (!p || !ms_avg || reps < 1) return set_error(SGBA_ERR_INVALID_ARGUMENT, "bad argument");
  int st = bench_prepare(p, flush_l2 != 0);
  if (st) return st;
  EventSet events;
  cudaEvent_t a, b;
  SGBA_CK(events.create(&a));
  SGBA_CK(events.create(&b));
  double total = 0.0;
  for (int i = 0; i < reps; ++i) {
    if (flush_l2) SGBA_CK(cudaMemsetAsync(p->flush_buf, i & 0xff, size_t(256) << 20, p->stream));
    SGBA_CK(cudaEventRecord(a, p->stream));
    if (kernel == SGBA_KERNEL_ITERATION) SGBA_CK(cudaGraphLaunch(p->graph_exec, p->stream));
    else sgba::launch_single(p->sz, p->d, kernel, p->stream);
    SGBA_CK(cudaEventRecord(b, p->stream));
    SGBA_CK(cudaEventSynchronize(b));
    float ms = 0.f;
    SGBA_CK(cudaEventElapsedTime(&ms, a, b));
    total += ms;
  }
  st = check_launch();
  if (st) return st;
  *ms_avg = total / reps;
  return SGBA_OK;
}

int sgba_get_profile(sgba_problem* p, sgba_profile* out) {
  if (!p || !out) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = p->prof;
  return SGBA_OK;
}

int sgba_set_profiling(sgba_problem* p, int32_t enabled) {
  if (!p) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL problem");
  p->profiling = enabled != 0;
  return SGBA_OK;
}

int sgba_total_cost_noalloc(int32_t n_cam, const double* poses, int32_t n_pt, const double* points, int64_t n_obs,
                            const int32_t* obs_cam, const int32_t* obs_pt, const double* obs_uv,
                            const double* intrinsics, double huber_delta, double* cost, void* stream) {
  // Host-side checks only: no CUDA call before the arguments are known good.
  const int max_cams = sgba::noalloc_max_cams();
  if (n_cam < 1 || n_cam > max_cams)
    return set_error(SGBA_ERR_INVALID_ARGUMENT,
                     "sgba_total_cost_noalloc: n_cam %d outside [1, %d] (the static scratch holds %d cameras)",
                     n_cam, max_cams, max_cams);
  if (n_pt < 0 || n_obs < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "sgba_total_cost_noalloc: negative n_pt or n_obs");
  if (!poses || !cost || !intrinsics || (n_pt > 0 && !points) || (n_obs > 0 && (!obs_cam || !obs_pt || !obs_uv)))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "sgba_total_cost_noalloc: NULL argument");
  for (int i = 0; i < 4; ++i)
    if (!std::isfinite(intrinsics[i]))
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "sgba_total_cost_noalloc: non-finite intrinsics");
  if (!std::isfinite(huber_delta))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "sgba_total_cost_noalloc: non-finite huber_delta");
  if (!huber_in_float_range(huber_delta))
    return set_error(SGBA_ERR_INVALID_ARGUMENT,
                     "sgba_total_cost_noalloc: huber_delta %g outside the float range the kernels compare in", huber_delta);
  // the kernels load obs_uv as 16-byte pairs and the other arrays as whole elements
  auto misaligned = [](const void* q, uintptr_t a) { return q && (reinterpret_cast<uintptr_t>(q) % a) != 0; };
  if (misaligned(obs_uv, 16) || misaligned(poses, 8) || misaligned(points, 8) || misaligned(cost, 8) ||
      misaligned(obs_cam, 4) || misaligned(obs_pt, 4))
    return set_error(SGBA_ERR_INVALID_ARGUMENT,
                     "sgba_total_cost_noalloc: misaligned device pointer (obs_uv needs 16 bytes, doubles 8, indices 4)");
  cudaError_t e = sgba::launch_total_cost_noalloc(n_cam, poses, n_pt, points, n_obs, obs_cam, obs_pt, obs_uv,
                                                  intrinsics, huber_delta, cost, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess)
    return set_error(SGBA_ERR_CUDA, "sgba_total_cost_noalloc: %s", cudaGetErrorString(e));
  return SGBA_OK;
}

// ---- iterative solve of the reduced camera system ------------------------

namespace {

// Full block rows of S (both triangles) from the lower block list, columns
// ascending in every row; diag[j] = lower block id of block (j, j).
void pcg_structure(const Plan& P, std::vector<int32_t>* rowptr, std::vector<int32_t>* cols,
                   std::vector<int32_t>* blks, std::vector<int32_t>* diag) {
  const int nf = P.nf;
  std::vector<std::vector<std::pair<int32_t, int32_t>>> rows(nf);
  diag->assign(nf, -1);
  for (size_t b = 0; b < P.sb_row.size(); ++b) {
    const int j = P.sb_row[b], k = P.sb_col[b];
    rows[j].push_back({k, static_cast<int32_t>(b)});
    if (j != k) rows[k].push_back({j, static_cast<int32_t>(b) | static_cast<int32_t>(0x80000000u)});
    else (*diag)[j] = static_cast<int32_t>(b);
  }
  rowptr->assign(nf + 1, 0);
  cols->clear();
  blks->clear();
  for (int j = 0; j < nf; ++j) {
    std::sort(rows[j].begin(), rows[j].end());
    for (const auto& e : rows[j]) {
      cols->push_back(e.first);
      blks->push_back(e.second);
    }
    (*rowptr)[j + 1] = static_cast<int32_t>(cols->size());
  }
}

int pcg_alloc(sgba_problem* p) {
  Dev& d = p->d;
  if (d.pcg_rowptr) return SGBA_OK;
  Sizes& s = p->sz;
  std::vector<int32_t> rowptr, cols, blks, diag;
  pcg_structure(p->plan, &rowptr, &cols, &blks, &diag);
  for (int j = 0; j < s.nf; ++j)
    if (diag[j] < 0) return set_error(SGBA_ERR_STATE, "free pose block %d has no diagonal block in S", j);
  int st;
  const size_t nf = static_cast<size_t>(s.nf), n6 = static_cast<size_t>(s.n6);
  if ((st = dev_upload(p, &d.pcg_rowptr, rowptr))) return st;
  if ((st = dev_upload(p, &d.pcg_cols, cols))) return st;
  if ((st = dev_upload(p, &d.pcg_blks, blks))) return st;
  if ((st = dev_upload(p, &d.pcg_diag, diag))) return st;
  if ((st = dev_alloc(p, &d.pcg_S, 36 * static_cast<size_t>(s.nsb)))) return st;
  if ((st = dev_alloc(p, &d.pcg_scl, n6))) return st;
  if ((st = dev_alloc(p, &d.pcg_P, 36 * nf))) return st;
  if ((st = dev_alloc(p, &d.pcg_Cinv, 36 * nf))) return st;
  if ((st = dev_alloc(p, &d.pcg_vec, 6 * n6))) return st;
  if ((st = dev_alloc(p, &d.pcg_S2, 36 * static_cast<size_t>(s.nsb)))) return st;
  if ((st = dev_alloc(p, &d.pcg_bar, 4))) return st;
  if ((st = dev_alloc(p, &d.pcg_part, 4 * static_cast<size_t>(sgba::kPcgMaxGrid)))) return st;
  if ((st = dev_alloc(p, &d.pcg_feat, nf * sgba::kPcgFeat))) return st;
  if ((st = dev_alloc(p, &d.pcg_ew, cols.size()))) return st;
  if ((st = dev_alloc(p, &d.pcg_h, 2 * nf * sgba::kPcgHidden))) return st;
  if ((st = dev_alloc(p, &d.pcg_msg, nf * sgba::kPcgHidden))) return st;
  if ((st = dev_alloc(p, &d.pcg_L, nf * sgba::kPcgOut))) return st;
  s.pcg_nnzb = static_cast<int64_t>(cols.size());
  SGBA_CK(cudaStreamSynchronize(p->stream));  // the host vectors above go out of scope
  return SGBA_OK;
}

uint16_t f32_to_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even
  return static_cast<uint16_t>(u >> 16);
}

int model_upload(sgba::PcgModel& m, const std::vector<float>& w) {
  std::vector<uint16_t> b(w.size());
  for (size_t i = 0; i < w.size(); ++i) b[i] = f32_to_bf16(w[i]);
  SGBA_CK(cudaSetDevice(m.device));
  SGBA_CK(cudaMemcpy(m.w32, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice));
  SGBA_CK(cudaMemcpy(m.wbf, b.data(), sizeof(uint16_t) * b.size(), cudaMemcpyHostToDevice));
  return SGBA_OK;
}

}  // namespace

struct sgba_pcg_model {
  sgba::PcgModel m;
};

int32_t sgba_pcg_num_params(void) { return sgba::kPcgParams; }

int sgba_pcg_model_create(int32_t device, uint64_t seed, sgba_pcg_model** out) {
  if (!out) return set_error(SGBA_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int dev = device;
  if (dev < 0) SGBA_CK(cudaGetDevice(&dev));
  SGBA_CK(cudaSetDevice(dev));
  std::unique_ptr<sgba_pcg_model> h(new (std::nothrow) sgba_pcg_model());
  if (!h) return set_error(SGBA_ERR_OUT_OF_MEMORY, "host allocation failed");
  sgba::PcgModel& m = h->m;
  m.device = dev;
  const size_t n = sgba::kPcgParams;
  auto fail = [&](cudaError_t e) {
    cudaFree(m.w32); cudaFree(m.wbf); cudaFree(m.m1); cudaFree(m.m2); cudaFree(m.grad);
    return set_error(SGBA_ERR_OUT_OF_MEMORY, "model allocation: %s", cudaGetErrorString(e));
  };
  cudaError_t e;
  if ((e = cudaMalloc(&m.w32, sizeof(float) * n)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&m.wbf, sizeof(uint16_t) * n)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&m.m1, sizeof(float) * n)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&m.m2, sizeof(float) * n)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&m.grad, sizeof(float) * n)) != cudaSuccess) return fail(e);
  cudaMemset(m.m1, 0, sizeof(float) * n);
  cudaMemset(m.m2, 0, sizeof(float) * n);
  cudaMemset(m.grad, 0, sizeof(float) * n);
  // Glorot-uniform hidden weights from a SplitMix64 stream; the output head
  // starts at L = 0.1 I (P = 1.01 x block-Jacobi: the gradient of L L^T
  // vanishes at L = 0) with small random weights
  std::vector<float> w(n, 0.0f);
  uint64_t st = seed;
  auto uni = [&st]() {
    uint64_t z = (st += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  const int H = sgba::kPcgHidden, F = sgba::kPcgFeat;
  const double a_in = std::sqrt(6.0 / (F + H)), a_h = 0.5 * std::sqrt(6.0 / (2.0 * H));
  for (int i = 0; i < H * F; ++i) w[i] = static_cast<float>(a_in * uni());
  size_t off = static_cast<size_t>(H) * F + H;
  for (int l = 0; l < sgba::kPcgLayers; ++l) {
    for (int i = 0; i < 2 * H * H; ++i) w[off + i] = static_cast<float>(a_h * uni());
    off += 2 * static_cast<size_t>(H) * H + H;
  }
  for (int i = 0; i < sgba::kPcgOut * H; ++i) w[off + i] = static_cast<float>(0.01 * uni());
  off += static_cast<size_t>(sgba::kPcgOut) * H;
  for (int r = 0, t = 0; r < 6; ++r)
    for (int c = 0; c <= r; ++c, ++t) w[off + t] = (r == c) ? 0.1f : 0.0f;
  int rc = model_upload(m, w);
  if (rc) { fail(cudaSuccess); return rc; }
  *out = h.release();
  return SGBA_OK;
}

int sgba_pcg_model_destroy(sgba_pcg_model* h) {
  if (!h) return SGBA_OK;
  cudaSetDevice(h->m.device);
  cudaFree(h->m.w32);
  cudaFree(h->m.wbf);
  cudaFree(h->m.m1);
  cudaFree(h->m.m2);
  cudaFree(h->m.grad);
  delete h;
  return SGBA_OK;
}

int sgba_pcg_model_set_params(sgba_pcg_model* h, const float* params, int32_t n) {
  if (!h || !params) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n != sgba::kPcgParams) return set_error(SGBA_ERR_INVALID_ARGUMENT, "%d parameters (expected %d)", n, sgba::kPcgParams);
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(params[i])) return set_error(SGBA_ERR_INVALID_ARGUMENT, "parameter %d is not finite", i);
  std::vector<float> w(params, params + n);
  int rc = model_upload(h->m, w);
  if (rc) return rc;
  SGBA_CK(cudaMemset(h->m.m1, 0, sizeof(float) * n));
  SGBA_CK(cudaMemset(h->m.m2, 0, sizeof(float) * n));
  h->m.step = 0;
  return SGBA_OK;
}

int sgba_pcg_model_get_params(const sgba_pcg_model* h, float* params, int32_t n) {
  if (!h || !params) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n != sgba::kPcgParams) return set_error(SGBA_ERR_INVALID_ARGUMENT, "%d parameters (expected %d)", n, sgba::kPcgParams);
  SGBA_CK(cudaSetDevice(h->m.device));
  SGBA_CK(cudaMemcpy(params, h->m.w32, sizeof(float) * n, cudaMemcpyDeviceToHost));
  return SGBA_OK;
}

int sgba_set_linear_solver(sgba_problem* p, const sgba_linear_solver* cfg, const sgba_pcg_model* model) {
  if (!p || !cfg) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (cfg->mode < SGBA_LINSOLVE_EXACT || cfg->mode > SGBA_LINSOLVE_PCG_LEARNED)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "unknown linear solver mode %d", cfg->mode);
  if (cfg->mode == SGBA_LINSOLVE_PCG_LEARNED && !model)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "the learned preconditioner needs a model");
  if (cfg->mode != SGBA_LINSOLVE_EXACT) {
    if (!(cfg->max_iterations >= 1) || !(cfg->tolerance > 0.0) || !std::isfinite(cfg->tolerance))
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "PCG needs max_iterations >= 1 and a finite tolerance > 0");
    if (p->plan.nf < 1) return set_error(SGBA_ERR_SCHUR_MISSING_FREE_OR_MARG, "no free pose: nothing to solve");
    if (p->intr_free) return set_error(SGBA_ERR_UNSUPPORTED, "PCG with free intrinsics is not on this path");
    if (p->sz.n_eq > 0) return set_error(SGBA_ERR_UNSUPPORTED, "PCG with equality constraints is not on this path");
    if (model && model->m.device != p->device)
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "model on device %d, problem on device %d", model->m.device,
                       p->device);
  }
  SGBA_CK(cudaSetDevice(p->device));
  if (cfg->mode != SGBA_LINSOLVE_EXACT) {
    int st = pcg_alloc(p);
    if (st) return st;
    int grid = 0;
    if (sgba::pcg_setup(p->plan.nf, &grid) != 0 || grid < 1)
      return set_error(SGBA_ERR_UNSUPPORTED, "cooperative launch of the PCG kernel is not available");
    if (cfg->mode == SGBA_LINSOLVE_PCG_LEARNED && sgba::pcg_net_setup() != 0)
      return set_error(SGBA_ERR_CUDA, "could not raise the shared memory limit of the network kernels");
    p->sz.pcg_grid = grid;
  }
  p->sz.pcg_mode = cfg->mode;
  p->sz.pcg_max_iters = cfg->max_iterations;
  p->sz.pcg_tol = cfg->tolerance;
  p->d.pcg_w = (cfg->mode == SGBA_LINSOLVE_PCG_LEARNED) ? model->m.wbf : nullptr;
  // the iteration graph is captured again with the new solver chain
  SGBA_CK(cudaStreamSynchronize(p->stream));
  if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
  if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  const int zero = 0;
  SGBA_CK(cudaMemcpy(reinterpret_cast<char*>(p->d.ctrl) + offsetof(Ctrl, pcg_done), &zero, sizeof(int),
                     cudaMemcpyHostToDevice));
  return SGBA_OK;
}

int sgba_get_pcg_stats(sgba_problem* p, sgba_pcg_stats* out) {
  if (!p || !out) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  SGBA_CK(cudaSetDevice(p->device));
  Ctrl c;
  SGBA_CK(cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  out->solves = c.pcg_solves;
  out->fallbacks = c.pcg_fallbacks;
  out->iterations = c.pcg_total_iters;
  out->last_iterations = c.pcg_iters;
  out->last_status = c.pcg_status;
  out->last_relative_residual = c.pcg_relres;
  return SGBA_OK;
}

// ---- training the learned preconditioner ----------------------------------

struct sgba_pcg_trainset {
  sgba::PcgTrainSet t;
  cudaStream_t stream = nullptr;
};

namespace {

// Device copy of one system; blocks64 / b / xs are device or host pointers
// (kind = the cudaMemcpy direction from them).
int trainset_append(sgba_pcg_trainset* h, const Plan* plan, int nf, const std::vector<int32_t>& sb_row,
                    const std::vector<int32_t>& sb_col, const double* blocks64, const double* b, const double* xs,
                    cudaMemcpyKind kind) {
  sgba::PcgSystem s;
  s.nf = nf;
  s.nsb = static_cast<int64_t>(sb_row.size());
  Plan tmp;
  tmp.nf = nf;
  tmp.sb_row = sb_row;
  tmp.sb_col = sb_col;
  std::vector<int32_t> rowptr, cols, blks, diag;
  pcg_structure(plan ? *plan : tmp, &rowptr, &cols, &blks, &diag);
  for (int j = 0; j < nf; ++j)
    if (diag[j] < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "block row %d has no diagonal block", j);
  s.nnzb = static_cast<int64_t>(cols.size());
  const size_t n6 = 6 * static_cast<size_t>(nf), nb = 36 * static_cast<size_t>(s.nsb);
  auto fail = [&](cudaError_t e) {
    cudaFree(s.rowptr); cudaFree(s.cols); cudaFree(s.blks); cudaFree(s.diag);
    cudaFree(s.Sb); cudaFree(s.Sb2); cudaFree(s.b); cudaFree(s.xs);
    return set_error(e == cudaErrorMemoryAllocation ? SGBA_ERR_OUT_OF_MEMORY : SGBA_ERR_CUDA, "training set: %s",
                     cudaGetErrorString(e));
  };
  cudaError_t e;
  if ((e = cudaMalloc(&s.rowptr, sizeof(int32_t) * rowptr.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&s.cols, sizeof(int32_t) * std::max<size_t>(cols.size(), 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&s.blks, sizeof(int32_t) * std::max<size_t>(blks.size(), 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&s.diag, sizeof(int32_t) * diag.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&s.Sb, sizeof(double) * nb)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&s.Sb2, sizeof(float2) * nb)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&s.b, sizeof(double) * n6)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&s.xs, sizeof(double) * n6)) != cudaSuccess) return fail(e);
  e = cudaMemcpy(s.rowptr, rowptr.data(), sizeof(int32_t) * rowptr.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s.cols, cols.data(), sizeof(int32_t) * cols.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s.blks, blks.data(), sizeof(int32_t) * blks.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s.diag, diag.data(), sizeof(int32_t) * diag.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s.Sb, blocks64, sizeof(double) * nb, kind);
  if (e == cudaSuccess) e = cudaMemcpy(s.b, b, sizeof(double) * n6, kind);
  if (e == cudaSuccess) e = cudaMemcpy(s.xs, xs, sizeof(double) * n6, kind);
  if (e != cudaSuccess) return fail(e);
  // float-float copy of the blocks and den = x* . b on the host
  std::vector<double> hb(nb), hbv(n6), hx(n6);
  e = cudaMemcpy(hb.data(), s.Sb, sizeof(double) * nb, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hbv.data(), s.b, sizeof(double) * n6, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hx.data(), s.xs, sizeof(double) * n6, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(e);
  std::vector<float2> h2(nb);
  for (size_t i = 0; i < nb; ++i) {
    if (!std::isfinite(hb[i])) { fail(cudaSuccess); return set_error(SGBA_ERR_INVALID_ARGUMENT, "non-finite block entry"); }
    const float hi = static_cast<float>(hb[i]);
    h2[i] = make_float2(hi, static_cast<float>(hb[i] - static_cast<double>(hi)));
  }
  if ((e = cudaMemcpy(s.Sb2, h2.data(), sizeof(float2) * nb, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
  double den = 0.0;
  for (size_t i = 0; i < n6; ++i) den += hx[i] * hbv[i];
  if (!(den > 0.0) || !std::isfinite(den)) {
    fail(cudaSuccess);
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "x* . b = %g: not a positive definite system's solution", den);
  }
  s.den = den;
  h->t.sys.push_back(s);
  return SGBA_OK;
}

}  // namespace

int sgba_pcg_trainset_create(int32_t device, sgba_pcg_trainset** out) {
  if (!out) return set_error(SGBA_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int dev = device;
  if (dev < 0) SGBA_CK(cudaGetDevice(&dev));
  SGBA_CK(cudaSetDevice(dev));
  std::unique_ptr<sgba_pcg_trainset> h(new (std::nothrow) sgba_pcg_trainset());
  if (!h) return set_error(SGBA_ERR_OUT_OF_MEMORY, "host allocation failed");
  h->t.device = dev;
  SGBA_CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  *out = h.release();
  return SGBA_OK;
}

int sgba_pcg_trainset_destroy(sgba_pcg_trainset* h) {
  if (!h) return SGBA_OK;
  cudaSetDevice(h->t.device);
  if (h->stream) {
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  delete h;
  return SGBA_OK;
}

int32_t sgba_pcg_trainset_size(const sgba_pcg_trainset* h) { return h ? static_cast<int32_t>(h->t.sys.size()) : 0; }

int sgba_pcg_trainset_add(sgba_pcg_trainset* h, int32_t nf, int64_t n_blocks, const int32_t* s_rows,
                          const int32_t* s_cols, const double* blocks, const double* b, const double* x) {
  if (!h || !s_rows || !s_cols || !blocks || !b || !x) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (nf < 1 || n_blocks < nf) return set_error(SGBA_ERR_INVALID_ARGUMENT, "bad system size");
  std::vector<int32_t> r(s_rows, s_rows + n_blocks), c(s_cols, s_cols + n_blocks);
  for (int64_t k = 0; k < n_blocks; ++k)
    if (r[k] < 0 || r[k] >= nf || c[k] < 0 || c[k] > r[k])
      return set_error(SGBA_ERR_INVALID_ARGUMENT, "block %lld: (%d, %d) is not a lower block of a %d-row system",
                       static_cast<long long>(k), r[k], c[k], nf);
  SGBA_CK(cudaSetDevice(h->t.device));
  return trainset_append(h, nullptr, nf, r, c, blocks, b, x, cudaMemcpyHostToDevice);
}

int sgba_pcg_collect(sgba_problem* p, sgba_pcg_trainset* h) {
  if (!p || !h) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->inited) return set_error(SGBA_ERR_STATE, "sgba_pcg_collect before sgba_optimizer_init");
  if (h->t.device != p->device) return set_error(SGBA_ERR_INVALID_ARGUMENT, "training set on another device");
  SGBA_CK(cudaSetDevice(p->device));
  int st = pcg_alloc(p);
  if (st) return st;
  // the reduced system of the latest linearisation: its scaled blocks and
  // its exact solution (the factorization, not the gauge-projected step)
  const Ctrl* cz = nullptr;
  (void)cz;
  Ctrl c;
  SGBA_CK(cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  if (c.step < 1) return set_error(SGBA_ERR_STATE, "sgba_pcg_collect needs a step first");
  Ctrl saved = c;
  c.done = 0;
  c.skip = 0;
  c.pcg_done = 0;
  SGBA_CK(cudaMemcpyAsync(p->d.ctrl, &c, sizeof(Ctrl), cudaMemcpyHostToDevice, p->stream));
  sgba::Sizes z = p->sz;
  z.pcg_mode = 0;
  sgba::launch_pcg_blocks_only(z, p->d, p->stream);
  sgba::launch_exact_solve(z, p->d, p->stream);
  SGBA_CK(cudaGetLastError());
  Ctrl after;
  SGBA_CK(cudaMemcpyAsync(&after, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream));
  SGBA_CK(cudaStreamSynchronize(p->stream));
  SGBA_CK(cudaMemcpy(p->d.ctrl, &saved, sizeof(Ctrl), cudaMemcpyHostToDevice));
  if (after.skip != 0) return set_error(SGBA_ERR_STATE, "the exact factorization failed on this system");
  const size_t n6 = static_cast<size_t>(p->sz.n6);
  std::vector<double> scl(n6), rb(n6), x(n6);
  SGBA_CK(cudaMemcpy(scl.data(), p->d.pcg_scl, sizeof(double) * n6, cudaMemcpyDeviceToHost));
  SGBA_CK(cudaMemcpy(rb.data(), p->d.rb, sizeof(double) * n6, cudaMemcpyDeviceToHost));
  SGBA_CK(cudaMemcpy(x.data(), p->d.x, sizeof(double) * n6, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < n6; ++i) {
    rb[i] *= scl[i];  // b~ = D^-1/2 b
    x[i] /= scl[i];   // x~ = D^1/2 x
  }
  std::vector<double> blocks(36 * static_cast<size_t>(p->sz.nsb));
  SGBA_CK(cudaMemcpy(blocks.data(), p->d.pcg_S, sizeof(double) * blocks.size(), cudaMemcpyDeviceToHost));
  SGBA_CK(cudaSetDevice(h->t.device));
  return trainset_append(h, &p->plan, p->plan.nf, p->plan.sb_row, p->plan.sb_col, blocks.data(), rb.data(), x.data(),
                         cudaMemcpyHostToDevice);
}

int sgba_pcg_loss_grad(sgba_pcg_model* m, sgba_pcg_trainset* h, int32_t index, double* loss, float* grad,
                       int32_t n_grad) {
  if (!m || !h || !loss) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (index < 0 || index >= static_cast<int32_t>(h->t.sys.size()))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "system %d of %zu", index, h->t.sys.size());
  if (grad && n_grad != sgba::kPcgParams)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "%d gradient entries (expected %d)", n_grad, sgba::kPcgParams);
  if (m->m.device != h->t.device) return set_error(SGBA_ERR_INVALID_ARGUMENT, "model and training set on different devices");
  SGBA_CK(cudaSetDevice(h->t.device));
  SGBA_CK(cudaMemsetAsync(m->m.grad, 0, sizeof(float) * sgba::kPcgParams, h->stream));
  SGBA_CK(sgba::pcg_loss_grad(m->m, h->t, index, grad != nullptr, loss, h->stream));
  if (grad) {
    SGBA_CK(cudaMemcpyAsync(grad, m->m.grad, sizeof(float) * sgba::kPcgParams, cudaMemcpyDeviceToHost, h->stream));
    SGBA_CK(cudaMemsetAsync(m->m.grad, 0, sizeof(float) * sgba::kPcgParams, h->stream));
    SGBA_CK(cudaStreamSynchronize(h->stream));
  }
  return SGBA_OK;
}

int sgba_pcg_train(sgba_pcg_model* m, sgba_pcg_trainset* h, const sgba_pcg_train_params* tp, double* epoch_loss) {
  if (!m || !h || !tp) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  const int n = static_cast<int>(h->t.sys.size());
  if (n < 1) return set_error(SGBA_ERR_INVALID_ARGUMENT, "empty training set");
  if (tp->epochs < 1 || tp->batch < 1 || !(tp->learning_rate > 0.0))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "epochs, batch and learning_rate must be positive");
  if (m->m.device != h->t.device) return set_error(SGBA_ERR_INVALID_ARGUMENT, "model and training set on different devices");
  SGBA_CK(cudaSetDevice(h->t.device));
  SGBA_CK(cudaMemsetAsync(m->m.grad, 0, sizeof(float) * sgba::kPcgParams, h->stream));
  std::vector<int> order(n);
  uint64_t rng = tp->seed;
  auto next = [&rng]() {
    uint64_t z = (rng += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  };
  for (int ep = 0; ep < tp->epochs; ++ep) {
    for (int i = 0; i < n; ++i) order[i] = i;
    for (int i = n - 1; i > 0; --i) std::swap(order[i], order[static_cast<int>(next() % (uint64_t)(i + 1))]);
    double tot = 0.0;
    int in_batch = 0;
    for (int i = 0; i < n; ++i) {
      double l = 0.0;
      SGBA_CK(sgba::pcg_loss_grad(m->m, h->t, order[i], true, &l, h->stream));
      tot += l;
      if (++in_batch == tp->batch || i == n - 1) {
        SGBA_CK(sgba::pcg_adam(m->m, 1.0f / static_cast<float>(in_batch), static_cast<float>(tp->learning_rate),
                               0.9f, 0.999f, 1e-8f, h->stream));
        in_batch = 0;
      }
    }
    if (epoch_loss) epoch_loss[ep] = tot / n;
  }
  SGBA_CK(cudaStreamSynchronize(h->stream));
  return SGBA_OK;
}

int sgba_pcg_evaluate(const sgba_pcg_model* m, sgba_pcg_trainset* h, int32_t index, int32_t mode,
                      int32_t max_iterations, double tolerance, int32_t* iterations, double* relative_residual,
                      int32_t* status) {
  if (!h || !iterations || !relative_residual || !status) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (index < 0 || index >= static_cast<int32_t>(h->t.sys.size()))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "system %d of %zu", index, h->t.sys.size());
  if (mode != SGBA_LINSOLVE_PCG_BLOCK_JACOBI && mode != SGBA_LINSOLVE_PCG_LEARNED)
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "mode must be 1 or 2");
  if (mode == SGBA_LINSOLVE_PCG_LEARNED && !m) return set_error(SGBA_ERR_INVALID_ARGUMENT, "mode 2 needs a model");
  if (max_iterations < 1 || !(tolerance > 0.0)) return set_error(SGBA_ERR_INVALID_ARGUMENT, "bad iteration cap or tolerance");
  SGBA_CK(cudaSetDevice(h->t.device));
  int it = 0, stt = 0;
  double rr = 0.0;
  SGBA_CK(sgba::pcg_evaluate(m ? &m->m : nullptr, h->t, index, mode, max_iterations, tolerance, &it, &rr, &stt,
                             h->stream));
  *iterations = it;
  *relative_residual = rr;
  *status = stt;
  return SGBA_OK;
}

}  // extern "C"

namespace {

// ---------------------------------------------------------------------------
// Batched windows.  The eligible windows of a batch are split into groups;
// each group's LM iteration is one CUDA graph of batched launches (every
// kernel once for all windows of the group) on its own stream.  The schedule
// -- how many groups, and whether windows are ordered by decreasing work --
// changes only which CTAs run side by side, never what a window computes, so
// the autotuner below may pick it from timings: on the first calls for a
// shape (window count and observation count, rounded to powers of two) it
// times one LM iteration with each candidate schedule (iterations are
// identical work for every schedule), then keeps the fastest for that shape.
// SGBA_BATCH_SCHEDULE=<index> forces a candidate.
// ---------------------------------------------------------------------------
struct BatchSched {
  int groups;
  int order;  // 1: decreasing work, 0: as given
};
constexpr BatchSched kSched[] = {{1, 1}, {2, 1}, {4, 1}, {1, 0}};
constexpr int kNSched = 4;

struct TuneState {
  double ms[kNSched] = {0, 0, 0, 0};
  int samples[kNSched] = {0, 0, 0, 0};
  int best = -1;
};
std::mutex g_tune_mu;
std::map<std::pair<int, int>, TuneState> g_tune;

std::mutex g_batch_stats_mu;
sgba_batch_stats g_batch_stats{};

// Streams of the batched path on one device (created once, kept).
struct BatchCtx {
  std::mutex mu;  // one batched run at a time per device
  cudaStream_t main = nullptr;
  cudaStream_t side[4] = {nullptr, nullptr, nullptr, nullptr};
};
BatchCtx* batch_ctx(int dev) {
  static std::mutex mu;
  static std::map<int, std::unique_ptr<BatchCtx>> ctxs;
  std::lock_guard<std::mutex> lk(mu);
  auto& c = ctxs[dev];
  if (!c) {
    std::unique_ptr<BatchCtx> b(new BatchCtx());
    if (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    for (auto& x : b->side)
      if (cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    c = std::move(b);
  }
  return c.get();
}

int ceil_log2(int64_t v) {
  int k = 0;
  while ((int64_t(1) << k) < v && k < 62) ++k;
  return k;
}

// sgba_optimizer_init's checks and record buffers for a window that the
// batched launches run (its control block is written by the batch).
int batch_window_prepare(sgba_problem* p, const sgba_opt_params* prm) {
  SGBA_CK(cudaSetDevice(p->device));
  if ((p->plan.nf == 0 && !p->intr_free) || p->plan.nm == 0)
    return set_error(SGBA_ERR_SCHUR_MISSING_FREE_OR_MARG,
                     "Schur solver needs free and marginalized variables (free scalars %d, marg scalars %d)",
                     6 * p->plan.nf + (p->intr_free ? p->sz.intr_nk : 0), 3 * p->plan.nm);
  if (!std::isfinite(prm->initial_lm_damping))
    return set_error(SGBA_ERR_INVALID_ARGUMENT, "initial_lm_damping is not finite");
  p->params = *prm;
  const int cap = std::max(1, prm->num_iterations);
  if (p->d.record_cap < cap) {
    if (p->d.records) cudaFree(p->d.records);
    p->d.records = nullptr;
    SGBA_CK(cudaMalloc(&p->d.records, sizeof(Record) * cap));
    p->d.record_cap = cap;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  }
  // the batch reads and writes the window's buffers on its own streams
  SGBA_CK(cudaStreamSynchronize(p->stream));
  return SGBA_OK;
}

struct BatchRun {
  std::vector<size_t> index;  // window -> row of ctrl / recs
  std::vector<Ctrl> ctrl;
  std::vector<Record> recs;   // rows x cap
  float ms = 0.f;
};

// One schedule's groups: tables and the captured iteration graph of each.
struct SchedGroups {
  int sched = -1;
  std::vector<std::vector<int>> wins;  // per group: windows (indices into the batch list)
  std::vector<sgba::BatchTables*> tabs;
  std::vector<cudaGraphExec_t> graphs;
  std::vector<int> iter_launches;
};

void sched_destroy(SchedGroups& g, cudaStream_t st) {
  for (auto x : g.graphs)
    if (x) cudaGraphExecDestroy(x);
  for (auto t : g.tabs) sgba::batch_tables_destroy(t, st);
  g.graphs.clear();
  g.tabs.clear();
}

int sched_build(sgba_problem* const* problems, const std::vector<int>& batched, const std::vector<int>& by_work,
                int sc, int skip_final, BatchCtx* bc, SchedGroups* out) {
  const BatchSched S = kSched[sc];
  out->sched = sc;
  out->wins.assign(S.groups, {});
  const std::vector<int>& ord = by_work;
  // decreasing work dealt round robin (similar mixes per group); or as given
  for (size_t k = 0; k < ord.size(); ++k) {
    const int item = S.order ? ord[k] : static_cast<int>(k);
    out->wins[k % S.groups].push_back(item);
  }
  for (int g = 0; g < S.groups; ++g) {
    cudaStream_t st = g == 0 ? bc->main : bc->side[g];
    std::vector<sgba::BatchWin> bw;
    for (int item : out->wins[g]) {
      const sgba_problem* p = problems[batched[item]];
      bw.push_back(sgba::BatchWin{&p->sz, &p->d});
    }
    cudaError_t e = cudaSuccess;
    sgba::BatchTables* t = bw.empty() ? nullptr : sgba::batch_tables_create(bw, skip_final, st, &e);
    out->tabs.push_back(t);
    out->graphs.push_back(nullptr);
    out->iter_launches.push_back(0);
    if (!bw.empty() && !t)
      return set_error(SGBA_ERR_CUDA, "batch tables: %s", cudaGetErrorString(e));
    if (!t) continue;
    cudaGraph_t graph = nullptr;
    SGBA_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int nl = sgba::batch_launch_iteration(t, st);
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess) return set_error(SGBA_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&out->graphs[g], graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return set_error(SGBA_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(ce));
    out->iter_launches[g] = nl;
  }
  return SGBA_OK;
}

int batch_run(sgba_problem* const* problems, const std::vector<int>& batched, const sgba_opt_params* prm, int iters,
              int cap, BatchRun* run) {
  const int nb = static_cast<int>(batched.size());
  const int dev = problems[batched[0]]->device;
  SGBA_CK(cudaSetDevice(dev));
  BatchCtx* bc = batch_ctx(dev);
  if (!bc) return set_error(SGBA_ERR_CUDA, "batch streams could not be created");
  std::lock_guard<std::mutex> lk(bc->mu);
  // shape key and the schedule of every iteration
  int64_t obs = 0;
  std::vector<int64_t> work(nb);
  for (int k = 0; k < nb; ++k) {
    const Sizes& s = problems[batched[k]]->sz;
    obs += s.no;
    work[k] = s.no + 128 * s.nchunk;
  }
  std::vector<int> by_work(nb);
  for (int k = 0; k < nb; ++k) by_work[k] = k;
  std::stable_sort(by_work.begin(), by_work.end(), [&](int a, int b) { return work[a] > work[b]; });
  const std::pair<int, int> key(ceil_log2(nb), ceil_log2(std::max<int64_t>(obs, 1)));
  int forced = -1;
  if (const char* env = std::getenv("SGBA_BATCH_SCHEDULE")) {
    forced = std::atoi(env);
    if (forced < 0 || forced >= kNSched) forced = -1;
  }
  std::vector<int> plan(iters, 0);
  std::vector<int> timed(iters, 0);
  {
    std::lock_guard<std::mutex> tl(g_tune_mu);
    TuneState& ts = g_tune[key];
    if (forced >= 0) {
      std::fill(plan.begin(), plan.end(), forced);
    } else if (ts.best >= 0) {
      std::fill(plan.begin(), plan.end(), ts.best);
    } else {
      // iteration 0 untimed; then one timed iteration per unmeasured
      // candidate; then the best candidate measured before this call
      // (candidate 0 when none was)
      std::vector<int> todo;
      int best = 0;
      double bm = 1e300;
      for (int c = 0; c < kNSched; ++c) {
        if (ts.samples[c] == 0) todo.push_back(c);
        else if (ts.ms[c] / ts.samples[c] < bm) { bm = ts.ms[c] / ts.samples[c]; best = c; }
      }
      plan[0] = todo.empty() ? best : todo[0];
      size_t t = 0;
      for (int it = 1; it < iters; ++it) {
        if (t < todo.size()) { plan[it] = todo[t++]; timed[it] = 1; }
        else plan[it] = best;
      }
    }
  }
  // build the schedules this call uses; on every return path the main
  // stream (which joins every group's stream) is drained before the graphs
  // and tables go
  struct Schedules {
    SchedGroups g[kNSched];
    cudaStream_t main;
    ~Schedules() {
      cudaStreamSynchronize(main);
      for (auto& x : g) sched_destroy(x, main);
    }
  } schedules;
  schedules.main = bc->main;
  SchedGroups* sg = schedules.g;
  int st = SGBA_OK;
  for (int it = 0; it < iters && st == SGBA_OK; ++it)
    if (sg[plan[it]].sched < 0)
      st = sched_build(problems, batched, by_work, plan[it], prm->skip_final_hessian, bc, &sg[plan[it]]);
  if (st) return st;
  Ctrl init;
  std::memset(&init, 0, sizeof(init));
  init.nu = prm->initial_lm_damping;
  init.ftol = prm->function_tolerance;
  init.gtol = prm->gradient_tolerance;
  init.ptol = prm->parameter_tolerance;
  init.max_rejects = prm->max_consecutive_rejects;
  init.num_iterations = prm->num_iterations;
  init.record_cap = iters;
  EventSet events;
  cudaEvent_t ev0, ev1, fork;
  cudaEvent_t join[4];
  SGBA_CK(events.create(&ev0));
  SGBA_CK(events.create(&ev1));
  SGBA_CK(events.create(&fork));
  for (auto& j : join) SGBA_CK(events.create(&j));
  std::vector<cudaEvent_t> itev(iters + 1, nullptr);
  for (int it = 0; it <= iters; ++it)
    if ((it < iters && timed[it]) || (it > 0 && timed[it - 1])) SGBA_CK(events.create(&itev[it]));
  int64_t launches = 0;
  // fork the groups of schedule sc from the main stream, run fn per group, join
  auto across = [&](SchedGroups& G, const std::function<int(sgba::BatchTables*, int, cudaStream_t)>& fn) -> cudaError_t {
    const int ng = static_cast<int>(G.tabs.size());
    cudaError_t e = cudaEventRecord(fork, bc->main);
    for (int g = 1; g < ng && e == cudaSuccess; ++g) e = cudaStreamWaitEvent(bc->side[g], fork, 0);
    for (int g = 0; g < ng && e == cudaSuccess; ++g) {
      if (!G.tabs[g]) continue;
      launches += fn(G.tabs[g], g, g == 0 ? bc->main : bc->side[g]);
      e = cudaGetLastError();
    }
    for (int g = 1; g < ng && e == cudaSuccess; ++g) {
      e = cudaEventRecord(join[g], bc->side[g]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(bc->main, join[g], 0);
    }
    return e;
  };
  cudaError_t e = cudaEventRecord(ev0, bc->main);
  SchedGroups& first = sg[plan[0]];
  if (e == cudaSuccess)
    e = across(first, [&](sgba::BatchTables* t, int, cudaStream_t s) { return sgba::batch_launch_init(t, init, s); });
  for (int it = 0; it < iters && e == cudaSuccess; ++it) {
    if (itev[it]) e = cudaEventRecord(itev[it], bc->main);
    SchedGroups& G = sg[plan[it]];
    if (e == cudaSuccess)
      e = across(G, [&](sgba::BatchTables*, int g, cudaStream_t s) {
        return cudaGraphLaunch(G.graphs[g], s) == cudaSuccess ? G.iter_launches[g] : 0;
      });
    if (e == cudaSuccess && itev[it + 1] && (timed[it])) e = cudaEventRecord(itev[it + 1], bc->main);
  }
  SchedGroups& last = sg[plan[iters - 1]];
  const size_t rows = static_cast<size_t>(nb);
  const size_t rcap = static_cast<size_t>(std::max(1, cap));
  Ctrl* d_ctrl = nullptr;
  Record* d_rec = nullptr;
  if (e == cudaSuccess)
    e = across(last, [&](sgba::BatchTables* t, int, cudaStream_t s) { return sgba::batch_launch_final(t, s); });
  if (e == cudaSuccess) e = cudaEventRecord(ev1, bc->main);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_ctrl, sizeof(Ctrl) * rows, bc->main);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_rec, sizeof(Record) * rows * rcap, bc->main);
  // rows: the last schedule's groups in order
  run->index.assign(static_cast<size_t>(*std::max_element(batched.begin(), batched.end())) + 1, 0);
  size_t row0 = 0;
  std::vector<size_t> grow(last.tabs.size(), 0);
  for (size_t g = 0; g < last.tabs.size(); ++g) {
    grow[g] = row0;
    for (size_t k = 0; k < last.wins[g].size(); ++k) run->index[batched[last.wins[g][k]]] = row0 + k;
    row0 += last.wins[g].size();
  }
  if (e == cudaSuccess)
    e = across(last, [&](sgba::BatchTables* t, int g, cudaStream_t s) {
      return sgba::batch_launch_collect(t, d_ctrl + grow[g], d_rec + grow[g] * rcap, static_cast<int>(rcap), s);
    });
  run->ctrl.resize(rows);
  run->recs.resize(rows * rcap);
  if (e == cudaSuccess) e = cudaMemcpyAsync(run->ctrl.data(), d_ctrl, sizeof(Ctrl) * rows, cudaMemcpyDeviceToHost, bc->main);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(run->recs.data(), d_rec, sizeof(Record) * rows * rcap, cudaMemcpyDeviceToHost, bc->main);
  if (d_ctrl) cudaFreeAsync(d_ctrl, bc->main);
  if (d_rec) cudaFreeAsync(d_rec, bc->main);
  if (e == cudaSuccess) e = cudaStreamSynchronize(bc->main);
  if (e != cudaSuccess) return set_error(SGBA_ERR_CUDA, "batched windows: %s", cudaGetErrorString(e));
  cudaEventElapsedTime(&run->ms, ev0, ev1);
  // autotuner: the timed iterations
  sgba_batch_stats bs{};
  {
    std::lock_guard<std::mutex> tl(g_tune_mu);
    TuneState& ts = g_tune[key];
    for (int it = 0; it < iters; ++it) {
      if (!timed[it]) continue;
      float m = 0.f;
      if (cudaEventElapsedTime(&m, itev[it], itev[it + 1]) == cudaSuccess) {
        ts.ms[plan[it]] += m;
        ts.samples[plan[it]] += 1;
      }
    }
    bool all = true;
    int best = -1;
    double bm = 1e300;
    for (int c = 0; c < kNSched; ++c) {
      if (ts.samples[c] == 0) { all = false; continue; }
      const double v = ts.ms[c] / ts.samples[c];
      bs.schedule_ms[c] = static_cast<float>(v);
      if (v < bm) { bm = v; best = c; }
    }
    if (all && ts.best < 0) ts.best = best;
    bs.tuned = ts.best >= 0 ? 1 : 0;
  }
  bs.batched_windows = nb;
  bs.schedule = plan[iters - 1];
  bs.groups = kSched[plan[iters - 1]].groups;
  bs.order = kSched[plan[iters - 1]].order;
  bs.kernel_launches = launches;
  bs.ms = run->ms;
  {
    std::lock_guard<std::mutex> sl(g_batch_stats_mu);
    g_batch_stats = bs;
  }
  return SGBA_OK;
}

}  // namespace

extern "C" {

int sgba_batch_optimize(sgba_problem* const* problems, int32_t n, const sgba_opt_params* prm,
                        sgba_iter_record* records, int32_t cap, sgba_window_result* results) {
  if (!prm || (n > 0 && (!problems || !results))) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n < 0) return set_error(SGBA_ERR_INVALID_ARGUMENT, "negative window count");
  const int iters = std::max(1, prm->num_iterations);
  std::vector<cudaEvent_t> e0(n, nullptr), e1(n, nullptr);
  std::vector<int> live(n, 0);
  std::vector<int> batched;  // windows run by the batched launches
  int dev0 = -1;
  // 0. validation; the windows that the batched launches can run
  for (int w = 0; w < n; ++w) {
    sgba_window_result& r = results[w];
    std::memset(&r, 0, sizeof(r));
    sgba_problem* p = problems[w];
    if (!p) { r.status = set_error(SGBA_ERR_INVALID_ARGUMENT, "window %d: NULL problem", w); continue; }
    if (dev0 < 0) dev0 = p->device;
    if (p->device == dev0 && !p->profiling && sgba::batch_eligible(p->sz)) {
      const int st = batch_window_prepare(p, prm);
      if (st) { r.status = st; continue; }
      batched.push_back(w);
      live[w] = 2;
    }
  }
  // 1. the other windows: init and all iterations, each on its own stream
  for (int w = 0; w < n; ++w) {
    sgba_window_result& r = results[w];
    sgba_problem* p = problems[w];
    if (!p || live[w] == 2 || r.status) continue;
    if (cudaSetDevice(p->device) != cudaSuccess || cudaEventCreate(&e0[w]) != cudaSuccess ||
        cudaEventCreate(&e1[w]) != cudaSuccess) {
      r.status = set_error(SGBA_ERR_CUDA, "window %d: event creation failed", w);
      continue;
    }
    p->defer_sync = true;
    const int st = sgba_optimizer_init(p, prm);
    p->defer_sync = false;
    if (st) { r.status = st; continue; }
    cudaError_t e = cudaEventRecord(e0[w], p->stream);
    for (int it = 0; it < iters && e == cudaSuccess; ++it) e = cudaGraphLaunch(p->graph_exec, p->stream);
    if (e != cudaSuccess) { r.status = set_error(SGBA_ERR_CUDA, "window %d: %s", w, cudaGetErrorString(e)); continue; }
    live[w] = 1;
  }
  // 2. the batched windows: every kernel of an iteration once for all of them
  BatchRun run;
  if (!batched.empty()) {
    const int st = batch_run(problems, batched, prm, iters, cap, &run);
    for (int w : batched) {
      if (st) { results[w].status = st; live[w] = 0; }
    }
  }
  // 3. the other windows: the final linearisation of build_solution
  for (int w = 0; w < n; ++w) {
    if (live[w] != 1) continue;
    sgba_problem* p = problems[w];
    cudaSetDevice(p->device);
    double nu = 0.0;
    if (prm->skip_final_hessian) {
      Ctrl c;
      if (cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream) != cudaSuccess ||
          cudaStreamSynchronize(p->stream) != cudaSuccess) {
        results[w].status = set_error(SGBA_ERR_CUDA, "window %d: state readback failed", w);
        live[w] = 0;
        continue;
      }
      nu = c.nu;
    }
    const int final_launches = sgba::launch_linearize(p->sz, p->d, nu, true, p->stream);
    p->prof.kernel_launches = 3 + static_cast<int64_t>(iters) * p->iter_launches + final_launches;
    cudaEventRecord(e1[w], p->stream);
  }
  // 4. collect
  for (int w = 0; w < n; ++w) {
    sgba_window_result& r = results[w];
    if (live[w] == 1) {
      sgba_problem* p = problems[w];
      cudaSetDevice(p->device);
      Ctrl c;
      cudaError_t e = cudaMemcpyAsync(&c, p->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, p->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
      if (e != cudaSuccess) {
        r.status = set_error(SGBA_ERR_CUDA, "window %d: %s", w, cudaGetErrorString(e));
      } else {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0[w], e1[w]);
        r.status = SGBA_OK;
        r.termination = c.termination;
        r.n_records = c.step;
        r.ms = ms;
        r.final_cost = c.merit;
        if (records && cap > 0) {
          const int nrec = std::min(std::min(c.step, p->d.record_cap), cap);
          if (nrec > 0 && cudaMemcpy(records + static_cast<int64_t>(w) * cap, p->d.records, sizeof(Record) * nrec,
                                     cudaMemcpyDeviceToHost) != cudaSuccess)
            r.status = set_error(SGBA_ERR_CUDA, "window %d: record readback failed", w);
        }
      }
    } else if (live[w] == 2) {
      const size_t k = run.index[w];
      const Ctrl& c = run.ctrl[k];
      sgba_problem* p = problems[w];
      r.status = SGBA_OK;
      r.termination = c.termination;
      r.n_records = c.step;
      r.ms = run.ms;
      r.final_cost = c.merit;
      if (records && cap > 0) {
        const int nrec = std::min(std::min(c.step, p->d.record_cap), cap);
        if (nrec > 0)
          std::memcpy(records + static_cast<int64_t>(w) * cap, run.recs.data() + k * static_cast<size_t>(cap),
                      sizeof(Record) * nrec);
      }
      p->prof.kernel_launches = 0;  // counted for the whole batch (sgba_batch_last_stats)
      p->inited = true;
    }
    if (e0[w]) cudaEventDestroy(e0[w]);
    if (e1[w]) cudaEventDestroy(e1[w]);
  }
  return SGBA_OK;
}

int sgba_batch_last_stats(sgba_batch_stats* out) {
  if (!out) return set_error(SGBA_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(g_batch_stats_mu);
  *out = g_batch_stats;
  return SGBA_OK;
}

}  // extern "C"
