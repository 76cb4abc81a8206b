// gba_plan.cu -- host side of libgba.so: builds the device layout of a batch
// of problems (point-major keys, per-image key lists, reduced-system block
// structure with its pair lists, work chunks), owns the device buffers and
// drives the Levenberg-Marquardt iterations, and implements the C ABI of
// include/gba.h.
//
// The LM decisions are taken on the device (gba_kernels.cu, k_ctrl_*), so a
// whole solve is a fixed sequence of launches with no host synchronization;
// that sequence is captured once into a CUDA graph and replayed.
#include "gba_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <unistd.h>
#include <condition_variable>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <cstdlib>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

namespace gba {

namespace {

std::atomic<long long> g_launches{0};

#define GBA_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      std::fprintf(stderr, "gba: %s failed: %s (%s:%d)\n", #call,          \
                   cudaGetErrorString(e_), __FILE__, __LINE__);             \
      throw ::gba::CudaError{e_ == cudaErrorMemoryAllocation ? GBA_ERR_OOM         \
                                                      : GBA_ERR_CUDA};      \
    }                                                                       \
  } while (0)

// Worker threads kept for the host build: a job f(t), t = 1 .. n-1, runs on
// the workers while the caller runs t = 0, so a parallel phase costs a wake-up
// instead of thread creation.  One job at a time; a caller that finds the
// pool busy (another plan building on another thread) gets false and runs
// the job on fresh threads instead.
class HostPool {
 public:
  static HostPool& get() {
    static HostPool pool;
    return pool;
  }
  bool run(int n, const std::function<void(int)>& f) {
    if (getpid() != pid_) return false;   // a forked child has no workers
    std::unique_lock<std::mutex> busy(busy_, std::try_to_lock);
    if (!busy.owns_lock() || n - 1 > int(workers_.size())) return false;
    {
      std::lock_guard<std::mutex> lk(m_);
      job_ = &f;
      njob_ = n;
      pending_ = n - 1;
      ++gen_;
    }
    cv_.notify_all();
    f(0);
    std::unique_lock<std::mutex> lk(m_);
    done_.wait(lk, [&] { return pending_ == 0; });
    job_ = nullptr;
    return true;
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  HostPool() : pid_(getpid()) {
    const unsigned hw = std::thread::hardware_concurrency();
    const int n = int(std::max(1u, std::min(hw, 16u))) - 1;
    for (int w = 0; w < n; ++w) workers_.emplace_back([this, w] { loop(w + 1); });
  }
  void loop(int t) {
    long long seen = 0;
    for (;;) {
      const std::function<void(int)>* f = nullptr;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        if (t < njob_) f = job_;
      }
      if (!f) continue;
      (*f)(t);
      std::lock_guard<std::mutex> lk(m_);
      if (--pending_ == 0) done_.notify_one();
    }
  }
  const pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex m_, busy_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int njob_ = 0, pending_ = 0;
  long long gen_ = 0;
  bool stop_ = false;
};

// Runs f(begin, end, t) over [0, n) split into contiguous pieces, piece t
// in thread t (piece 0 in the calling thread).  cuts, if given, are the
// piece boundaries; otherwise the pieces are equal.
template <typename F>
void host_parallel(int64_t n, int threads, F f, const std::vector<int64_t>* cuts = nullptr) {
  if (threads <= 1 || n <= 1) {
    f(int64_t(0), n, 0);
    return;
  }
  auto lo = [&](int t) { return cuts ? (*cuts)[t] : n * t / threads; };
  const std::function<void(int)> piece = [&](int t) { f(lo(t), lo(t + 1), t); };
  if (HostPool::get().run(threads, piece)) return;
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back([&, t] { piece(t); });
  piece(0);
  for (auto& th : pool) th.join();
}

// Stable counting sort of the indices [0, n) by key(i) in [0, nb): off
// [nb + 1] gets each key's first slot and out[off[b] ..] its indices in
// ascending order.  Pieces of the index range count in parallel; the slots of
// a key go to the pieces in index order, so the result is the serial one.
template <typename KeyF>
void counting_sort(int64_t n, int nb, int threads, KeyF key, std::vector<int>& off,
                   std::vector<int>& out) {
  threads = int(std::max<int64_t>(1, std::min<int64_t>(threads, n / 65536)));
  std::vector<std::vector<int>> hist(threads, std::vector<int>(size_t(nb), 0));
  host_parallel(n, threads, [&](int64_t i0, int64_t i1, int t) {
    int* h = hist[t].data();
    for (int64_t i = i0; i < i1; ++i) h[key(i)]++;
  });
  off.assign(size_t(nb) + 1, 0);
  int run = 0;
  for (int b = 0; b < nb; ++b) {
    off[b] = run;
    for (int t = 0; t < threads; ++t) {
      const int c = hist[t][b];
      hist[t][b] = run;
      run += c;
    }
  }
  off[nb] = run;
  out.resize(size_t(n));
  host_parallel(n, threads, [&](int64_t i0, int64_t i1, int t) {
    int* h = hist[t].data();
    for (int64_t i = i0; i < i1; ++i) out[h[key(i)]++] = int(i);
  });
}

int host_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return int(std::max(1u, std::min(hw, 16u)));
}

int64_t params_per_camera(uint32_t m) {
  return ((m & GBA_COMPUTE_RADIAL_DISTORTION) ? 3 : 0) +
         ((m & GBA_COMPUTE_DECENTERING_DISTORTION) ? 2 : 0) +
         ((m & GBA_COMPUTE_INTRINSIC_PARAMS) ? 5 : 0);
}

// Full 10-parameter camera [k1 k2 k3 d1 d2 f s cx cy a] from the masked one.
void expand_camera(uint32_t mask, const double* c, double out[10]) {
  const double ident[10] = {0, 0, 0, 0, 0, 1, 0, 0, 0, 1};
  std::memcpy(out, ident, sizeof(ident));
  int o = 0;
  if (mask & GBA_COMPUTE_RADIAL_DISTORTION) {
    out[0] = c[0]; out[1] = c[1]; out[2] = c[2];
    o += 3;
  }
  if (mask & GBA_COMPUTE_DECENTERING_DISTORTION) {
    out[3] = c[o]; out[4] = c[o + 1];
    o += 2;
  }
  if (mask & GBA_COMPUTE_INTRINSIC_PARAMS) {
    for (int j = 0; j < 5; ++j) out[5 + j] = c[o + j];
  }
}

// Column of the full ten holding a camera's computed parameter m.
int camera_full_column(uint32_t mask, int m) {
  if (mask & GBA_COMPUTE_RADIAL_DISTORTION) {
    if (m < 3) return m;
    m -= 3;
  }
  if (mask & GBA_COMPUTE_DECENTERING_DISTORTION) {
    if (m < 2) return 3 + m;
    m -= 2;
  }
  return 5 + m;
}

// Whether a problem's shared cameras are unknowns of the device path.
bool cameras_free(const gba_problem& p) {
  return !(p.fix_mask & GBA_FIX_CAMERAS) && p.number_of_cameras > 0 &&
         params_per_camera(p.intrinsic_computations_mask) > 0;
}

// Page-locked host memory, pooled.  Page-locking is costly, so released
// buffers are kept (at most kPinnedKeepBuffers of them and kPinnedKeepBytes
// in all, the smallest dropped first) and handed to later requests that
// fit; a request that cannot be page-locked gets nullptr (the caller then
// uses pageable memory).
class PinnedPool {
 public:
  static void* take(size_t bytes, size_t* cap) {
    {
      std::lock_guard<std::mutex> g(mu());
      auto& fl = list();
      size_t best = fl.size();
      for (size_t i = 0; i < fl.size(); ++i)   // the smallest buffer that fits
        if (fl[i].second >= bytes && (best == fl.size() || fl[i].second < fl[best].second)) best = i;
      if (best < fl.size()) {
        void* p = fl[best].first;
        *cap = fl[best].second;
        fl.erase(fl.begin() + long(best));
        return p;
      }
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    *cap = bytes;
    return p;
  }
  static void give(void* p, size_t cap) {
    if (!p) return;
    std::lock_guard<std::mutex> g(mu());
    auto& fl = list();
    fl.emplace_back(p, cap);
    for (;;) {
      size_t total = 0, m = 0;
      for (size_t i = 0; i < fl.size(); ++i) {
        total += fl[i].second;
        if (fl[i].second < fl[m].second) m = i;
      }
      if (fl.size() <= kPinnedKeepBuffers && total <= kPinnedKeepBytes) break;
      cudaFreeHost(fl[m].first);
      fl.erase(fl.begin() + long(m));
    }
  }

 private:
  static constexpr size_t kPinnedKeepBuffers = 16;
  static constexpr size_t kPinnedKeepBytes = size_t(4) << 30;
  static std::mutex& mu() {
    static std::mutex m;
    return m;
  }
  static std::vector<std::pair<void*, size_t>>& list() {
    static auto* fl = new std::vector<std::pair<void*, size_t>>();   // outlives static destruction
    return *fl;
  }
};

// A host array whose elements start uninitialized: the builders write every
// entry, so the pages are first touched by their parallel loops instead of
// by a serial zero fill.  Arrays of a megabyte or more live in pooled
// page-locked memory, so their uploads run at the copy engines' rate.
template <typename T>
class HostBuf {
 public:
  HostBuf() = default;
  explicit HostBuf(size_t count) : n_(count) {
    if (!count) return;
    if (count * sizeof(T) >= (size_t(1) << 20)) p_ = static_cast<T*>(PinnedPool::take(count * sizeof(T), &cap_));
    if (!p_) {
      own_.reset(new T[count]);
      p_ = own_.get();
      cap_ = 0;
    }
  }
  ~HostBuf() {
    if (cap_) PinnedPool::give(p_, cap_);
  }
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
  T& operator[](size_t i) { return p_[i]; }
  const T& operator[](size_t i) const { return p_[i]; }
  T* data() { return p_; }
  const T* data() const { return p_; }
  size_t size() const { return n_; }
  bool empty() const { return n_ == 0; }

 private:
  size_t n_ = 0;
  T* p_ = nullptr;
  size_t cap_ = 0;   // page-locked capacity in bytes (0: owned pageable memory)
  std::unique_ptr<T[]> own_;
};

// Device buffer registry.  Allocations are stream-ordered on the plan's
// stream (cudaMallocAsync / cudaFreeAsync from the device's default pool), so
// creating or destroying a plan never synchronizes other plans' streams.
struct DeviceArena {
  std::vector<void*> ptrs;
  cudaStream_t stream = nullptr;
  size_t bytes = 0;
  long long uploaded = 0;
  template <typename T>
  T* alloc(size_t count) {
    if (count == 0) count = 1;
    void* p = nullptr;
    GBA_CUDA(cudaMallocAsync(&p, count * sizeof(T), stream));
    ptrs.push_back(p);
    bytes += count * sizeof(T);
    return static_cast<T*>(p);
  }
  template <typename T>
  T* upload(const T* h, size_t n) {
    T* p = alloc<T>(n);
    if (n) GBA_CUDA(cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, stream));
    uploaded += (long long)(n * sizeof(T));
    return p;
  }
  template <typename T>
  T* upload(const std::vector<T>& h) {
    return upload(h.data(), h.size());
  }
  template <typename T>
  T* upload(const HostBuf<T>& h) {
    return upload(h.data(), h.size());
  }
  void release() {
    for (void* p : ptrs) cudaFreeAsync(p, stream);
    ptrs.clear();
  }
};

}  // namespace

void count_launches(long long n) { g_launches += n; }

// ---------------------------------------------------------------------------
// Plan
// ---------------------------------------------------------------------------
struct Plan {
  gba_options opt{};
  int B = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  DeviceArena arena;
  DevPlan d{};
  // host layout
  std::vector<ProbInfo> prob;
  std::vector<std::vector<int32_t>> key_sorted_to_orig;  // per problem
  std::vector<int64_t> x_size;
  // values of fixed points / images per problem (empty when free); the
  // caller's x holds only the free groups: [points][images][cameras]
  std::vector<std::vector<double>> fix_pt_vals, fix_img_vals;
  int64_t x_img_off(int q) const { return prob[q].fix & 1 ? 0 : 3LL * prob[q].num_points; }
  int64_t x_cam_off(int q) const {
    return x_img_off(q) + (prob[q].fix & 2 ? 0 : 6LL * prob[q].num_images);
  }
  // the problem's full points / images from the caller's x
  const double* pts_of(int q, const double* x) const {
    return prob[q].fix & 1 ? fix_pt_vals[q].data() : x;
  }
  const double* imgs_of(int q, const double* x) const {
    return prob[q].fix & 2 ? fix_img_vals[q].data() : x + x_img_off(q);
  }
  // run state
  cudaGraphExec_t graph_exec = nullptr;
  cudaGraphExec_t iter_exec = nullptr;   // one LM iteration (one-shot solves)
  long long iter_launches = 0, graph_launches = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // the device-side PCG loop: the stream its body is captured on and the
  // passes it ran beyond the first of each loop (read back after each run)
  cudaStream_t pcg_stream = nullptr;
  unsigned long long* h_pcg_extra = nullptr;
  // the second stream of an iteration's fork (image sums beside the point
  // Schur and the assembly) and its fork / join events
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  unsigned long long pcg_extra_seen = 0;
  bool ran = false;
  long long launches_last_run = 0;
  double setup_ms = 0;
  long long h2d_bytes = 0, d2h_bytes = 0;
  // profiling: per stage event pairs per iteration
  std::vector<cudaEvent_t> prof_events;
  std::vector<int> prof_stage;
  double stage_ms[GBA_NUM_STAGES] = {};
  int stage_launches[GBA_NUM_STAGES] = {};
  double* d_rmse_scratch = nullptr;
  std::string trace_path;
  long long n_pairs = 0;           // key pairs of the Schur assembly (all problems)
  double z_density = 0.0;          // mean share of an image's keys in a block's pairs

  // Task timeline of the last dataflow factorization as CSV:
  // cta,mode,i,j,k0,count,wait_ns,select_ns,end_ns (times from the first wait).
  void write_trace() {
    const size_t nent = size_t(d.df_grid) * kDfTraceCap;
    std::vector<unsigned long long> h(nent * 4);
    GBA_CUDA(cudaMemcpy(h.data(), d.df_trace, h.size() * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost));
    unsigned long long t0 = ~0ull;
    for (size_t e = 0; e < nent; ++e)
      if (h[4 * e + 3]) t0 = std::min(t0, h[4 * e + 1]);
    FILE* f = std::fopen(trace_path.c_str(), "w");
    if (!f) return;
    std::fprintf(f, "cta,mode,i,j,k0,count,wait_ns,select_ns,end_ns\n");
    for (size_t e = 0; e < nent; ++e) {
      const unsigned long long* r = &h[4 * e];
      if (!r[3]) continue;
      std::fprintf(f, "%zu,%llu,%llu,%llu,%llu,%llu,%llu,%llu,%llu\n", e / kDfTraceCap, r[0] >> 56,
                   (r[0] >> 40) & 0xffff, (r[0] >> 24) & 0xffff, (r[0] >> 8) & 0xffff, r[0] & 0xff,
                   r[1] - t0, r[2] - t0, r[3] - t0);
    }
    std::fclose(f);
  }

  ~Plan() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (iter_exec) cudaGraphExecDestroy(iter_exec);
    for (cudaEvent_t e : prof_events) cudaEventDestroy(e);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    arena.release();
    if (stream) cudaStreamDestroy(stream);
    if (pcg_stream) cudaStreamDestroy(pcg_stream);
    if (side_stream) cudaStreamDestroy(side_stream);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (h_pcg_extra) cudaFreeHost(h_pcg_extra);
  }

  int build(const gba_problem* problems, const double* const* near_ys, int nprob,
            const gba_options* options);
  // parts of the launch sequence: everything, the prologue (initial cost
  // and linearization) or one LM iteration
  // kIteration starts with the previous linearization's image sums and
  // control (beside the point Schur and the assembly, which do not need
  // them); kEpilogue runs them for the last iteration
  enum Part { kAll, kPrologue, kIteration, kEpilogue };
  void enqueue(bool profile, Part part = kAll);
  int run();
  int sync();
};

namespace {

// Validates a problem for the device path: points and images free, the
// shared cameras fixed or (dense solver) free, soft constraints on any free
// group.
int validate(const gba_problem& p, bool pcg, int threads) {
  if (p.number_of_points < 0 || p.number_of_images < 0 || p.number_of_cameras < 0 ||
      p.number_of_keys < 0)
    return GBA_ERR_INVALID;
  if (p.number_of_keys > 0 && !p.feature_maps) return GBA_ERR_INVALID;
  if (p.number_of_images > 0 && !p.image_camera_map) return GBA_ERR_INVALID;
  // every combination of fixed groups but all three (nothing to solve)
  if (p.fix_mask > (GBA_FIX_POINTS | GBA_FIX_IMAGES | GBA_FIX_CAMERAS)) return GBA_ERR_INVALID;
  if (p.fix_mask == (GBA_FIX_POINTS | GBA_FIX_IMAGES | GBA_FIX_CAMERAS)) return GBA_ERR_UNSUPPORTED;
  const bool fixP = p.fix_mask & GBA_FIX_POINTS, fixI = p.fix_mask & GBA_FIX_IMAGES;
  const int64_t cps = params_per_camera(p.intrinsic_computations_mask);
  const bool free_cams = cameras_free(p);
  if ((p.fix_mask & GBA_FIX_CAMERAS) && p.number_of_cameras > 0 && cps > 0 && !p.fix_cameras)
    return GBA_ERR_INVALID;
  if (fixP && p.number_of_points > 0 && !p.fix_points) return GBA_ERR_INVALID;
  if (fixI && p.number_of_images > 0 && !p.fix_images) return GBA_ERR_INVALID;
  // point priors weigh free points (ba_gcp_constrained_vector_function.hpp:60-110)
  if (fixP && p.number_of_point_priors > 0) return GBA_ERR_INVALID;
  if (!(p.fix_mask & GBA_FIX_CAMERAS)) {
    if ((p.number_of_camera_constraints > 0 && !p.camera_constraints) ||
        p.number_of_camera_constraints < 0)
      return GBA_ERR_INVALID;
    const uint32_t m = p.intrinsic_computations_mask;
    for (int64_t c = 0; c < p.number_of_camera_constraints; ++c) {
      const gba_camera_constraint& cc = p.camera_constraints[c];
      if (cc.camera_id < 0 || cc.camera_id >= p.number_of_cameras) return GBA_ERR_BAD_INDEX;
      // a constraint on a group that is not computed fails
      // (camera_shared_vector_function.hpp:549-557)
      if ((cc.radial_mask && !(m & GBA_COMPUTE_RADIAL_DISTORTION)) ||
          (cc.decentering_mask && !(m & GBA_COMPUTE_DECENTERING_DISTORTION)) ||
          (cc.intrinsic_mask && !(m & GBA_COMPUTE_INTRINSIC_PARAMS)))
        return GBA_ERR;
    }
  }
  if ((p.number_of_point_constraints > 0 && !p.point_constraints) ||
      (p.number_of_image_constraints > 0 && !p.image_constraints) ||
      p.number_of_point_constraints < 0 || p.number_of_image_constraints < 0)
    return GBA_ERR_INVALID;
  // constraints on a fixed group have no rows (camera_shared_vector_function.hpp:483-629)
  for (int64_t c = 0; c < (fixP ? 0 : p.number_of_point_constraints); ++c)
    if (p.point_constraints[c].point_id < 0 || p.point_constraints[c].point_id >= p.number_of_points)
      return GBA_ERR_BAD_INDEX;
  for (int64_t c = 0; c < (fixI ? 0 : p.number_of_image_constraints); ++c)
    if (p.image_constraints[c].image_id < 0 || p.image_constraints[c].image_id >= p.number_of_images)
      return GBA_ERR_BAD_INDEX;
  if (p.number_of_point_priors < 0 || (p.number_of_point_priors > 0 && !p.point_prior_ids))
    return GBA_ERR_INVALID;
  for (int64_t i = 0; i < p.number_of_point_priors; ++i)
    if (p.point_prior_ids[i] < 0 || p.point_prior_ids[i] >= p.number_of_points) return GBA_ERR_BAD_INDEX;
  if (p.number_of_points > INT32_MAX / 4 || p.number_of_keys > INT32_MAX / 4)
    return GBA_ERR_INVALID;
  // the dense reduced system of one problem is at most 12288^2 doubles
  // (2048 reduced-system images: the images and the cameras' 6-wide parts)
  const int64_t n_ext = p.number_of_images + (free_cams ? p.number_of_cameras * ((cps + 5) / 6) : 0);
  if (!pcg && n_ext > 2048) return GBA_ERR_UNSUPPORTED;
  for (int64_t i = 0; i < p.number_of_images; ++i) {
    int64_t c = p.image_camera_map[i];
    if (c < 0 || c >= p.number_of_cameras) return GBA_ERR_BAD_INDEX;
  }
  // key indices, in parallel pieces for large problems
  const int64_t nk = p.number_of_keys;
  const int nth = nk > 200000 ? threads : 1;
  std::vector<char> bad(size_t(nth), 0);
  host_parallel(nk, nth, [&](int64_t k0, int64_t k1, int t) {
    for (int64_t k = k0; k < k1; ++k) {
      const int64_t im = p.feature_maps[2 * k], pt = p.feature_maps[2 * k + 1];
      if (im < 0 || im >= p.number_of_images || pt < 0 || pt >= p.number_of_points) bad[t] = 1;
    }
  });
  for (char v : bad)
    if (v) return GBA_ERR_BAD_INDEX;
  return GBA_OK;
}

}  // namespace

int Plan::build(const gba_problem* problems, const double* const* near_ys, int nprob,
                const gba_options* options) {
  auto t0 = std::chrono::steady_clock::now();
  // GBA_BUILD_TIMING=1 prints the host build's phases to stderr
  const bool timing = std::getenv("GBA_BUILD_TIMING") != nullptr;
  std::vector<std::pair<const char*, double>> phases;
  auto phase = [&](const char* name) {
    if (timing)
      phases.emplace_back(name, std::chrono::duration<double, std::milli>(
                                    std::chrono::steady_clock::now() - t0).count());
  };
  opt = *options;
  B = nprob;
  device = opt.device;
  GBA_CUDA(cudaSetDevice(device));
  GBA_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  arena.stream = stream;
  {
    // keep freed plan memory in the pool instead of returning it each time
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  GBA_CUDA(cudaEventCreate(&ev0));
  GBA_CUDA(cudaEventCreate(&ev1));
  const bool mixed = opt.precision == GBA_PRECISION_MIXED;
  const size_t tsz = mixed ? sizeof(float) : sizeof(double);
  const bool pcg = opt.linear_solver == GBA_LINEAR_PCG;

  if (!near_ys) return GBA_ERR_INVALID;
  for (int q = 0; q < nprob; ++q)
    if (!near_ys[q]) return GBA_ERR_INVALID;
  if (nprob == 1) {
    if (int err = validate(problems[0], pcg, host_threads())) return err;
  } else {   // problems in parallel; the first failing problem's status, as in order
    std::vector<int> errs(nprob, GBA_OK);
    const int nth = std::min(host_threads(), nprob);
    std::atomic<int> next{0};
    host_parallel(nth, nth, [&](int64_t, int64_t, int) {
      for (int q = next++; q < nprob; q = next++) errs[q] = validate(problems[q], pcg, 1);
    });
    for (int e : errs)
      if (e) return e;
  }
  phase("validate");
  // ---- global sizes
  int64_t P = 0, I = 0, K = 0, C = 0;
  for (int q = 0; q < nprob; ++q) {
    P += problems[q].number_of_points;
    I += problems[q].number_of_images;
    K += problems[q].number_of_keys;
    C += problems[q].number_of_cameras;
  }
  if (P > INT32_MAX / 4 || K > INT32_MAX / 4 || I > INT32_MAX / 64) return GBA_ERR_INVALID;
  // The iteration's fork (image sums beside the point Schur and the
  // assembly) pays where one plan's stages leave the GPU partly idle; small
  // plans (a server's micro-batches, several in flight) lose more to the
  // fork's setup and joins than they gain.  GBA_ONE_STREAM=1: never fork;
  // GBA_FORK=1: always.
  {
    const bool fork = std::getenv("GBA_ONE_STREAM") == nullptr &&
                      (K >= kForkMinKeys || std::getenv("GBA_FORK") != nullptr);
    if (fork) {
      GBA_CUDA(cudaStreamCreateWithFlags(&side_stream, cudaStreamNonBlocking));
      GBA_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
      GBA_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    }
  }

  HostBuf<int> key_img(K), key_pt(K), img_keys(K);
  HostBuf<double2> key_obs(K);
  bool any_weights = false;
  for (int q = 0; q < nprob; ++q) any_weights |= problems[q].key_covariance_inverse != nullptr;
  HostBuf<double> key_wl(any_weights ? 3 * K : 0);
  // per point (page-locked above 1 MB: uploaded without staging); every
  // entry is written below (entry 0 with the problems' first entries)
  HostBuf<int> pt_key_off(P + 1), pt_prob(P);
  std::vector<int> img_key_off(I + 1, 0), img_prob(I), img_cam(I);
  std::vector<double> cam64(10 * std::max<int64_t>(C, 1), 0.0);
  std::vector<float> cam32(cam64.size(), 0.0f);
  std::vector<int2> pairs;
  std::vector<int4> items;
  std::vector<int2> blk_ij;
  std::vector<int> blk_item_off(1, 0);
  std::vector<int> blk_map;
  std::vector<long long> blk_map_off(nprob, 0);
  std::vector<Chunk> key_chunks, pt_chunks, img_chunks;
  std::vector<int4> img_items;
  std::vector<int> img_item_off(1, 0);
  std::vector<int> prob_key_chunk_off(1, 0), prob_pt_chunk_off(1, 0), prob_img_chunk_off(1, 0);
  std::vector<int4> cons;          // (group 0 point / 1 image / 2 camera, global index, parameter, problem)
  std::vector<double2> cons_yw;    // (observed value, weight)
  std::vector<int> prob_cons_off(1, 0);
  std::vector<int> prior_pt, prob_prior_off(1, 0);
  std::vector<double> prior_y, prior_info;
  prob.resize(nprob);
  key_sorted_to_orig.resize(nprob);
  x_size.resize(nprob);
  fix_pt_vals.assign(nprob, {});
  fix_img_vals.assign(nprob, {});

  // ---- per-problem bases
  std::vector<int64_t> pbase(nprob + 1, 0), ibase(nprob + 1, 0), kbase(nprob + 1, 0),
      cbase(nprob + 1, 0);
  long long s_off = 0;
  int max_n = 0, max_nt = 0;
  int64_t I_ext = 0;
  bool any_free = false;
  for (int q = 0; q < nprob; ++q) {
    const gba_problem& p = problems[q];
    const int np = int(p.number_of_points), ni = int(p.number_of_images), nk = int(p.number_of_keys);
    const bool fc = cameras_free(p);
    const int cps = int(params_per_camera(p.intrinsic_computations_mask));
    ProbInfo& pi = prob[q];
    pi.point_begin = int(pbase[q]);
    pi.num_points = np;
    pi.image_begin = int(ibase[q]);
    pi.num_images = ni;
    pi.key_begin = int(kbase[q]);
    pi.num_keys = nk;
    pi.cam_begin = int(cbase[q]);
    pi.num_cams = int(p.number_of_cameras);
    pi.cps = fc ? cps : 0;
    pi.nc = fc ? (cps + 5) / 6 : 0;
    pi.ext_begin = int(I_ext);
    pi.num_ext = ni + pi.num_cams * pi.nc;
    any_free |= fc;
    pi.n = 6 * pi.num_ext;
    pi.nt = (pi.n + kTile - 1) / kTile;
    pi.s_off = s_off;
    if (!pcg) s_off += (long long)pi.n * pi.n;   // the dense system only for the factorization
    max_n = std::max(max_n, pi.n);
    max_nt = std::max(max_nt, pi.nt);
    pi.fix = (p.fix_mask & GBA_FIX_POINTS ? 1 : 0) | (p.fix_mask & GBA_FIX_IMAGES ? 2 : 0);
    pi.pad_ = 0;
    if (pi.fix & 1) fix_pt_vals[q].assign(p.fix_points, p.fix_points + 3LL * np);
    if (pi.fix & 2) fix_img_vals[q].assign(p.fix_images, p.fix_images + 6LL * ni);
    x_size[q] = (pi.fix & 1 ? 0 : 3LL * np) + (pi.fix & 2 ? 0 : 6LL * ni) +
                (p.fix_mask & GBA_FIX_CAMERAS ? 0 : int64_t(cps) * pi.num_cams);
    pbase[q + 1] = pbase[q] + np;
    ibase[q + 1] = ibase[q] + ni;
    kbase[q + 1] = kbase[q] + nk;
    cbase[q + 1] = cbase[q] + p.number_of_cameras;
    I_ext += pi.num_ext;
  }
  if (I_ext > INT32_MAX / 64) return GBA_ERR_INVALID;

  // ---- each problem's structure: the per-key, per-point and per-image
  // arrays are written in place (disjoint ranges), the appended lists go to
  // a piece per problem; problems are built in parallel, or one problem's
  // points in parallel when there is only one
  struct Piece {
    int err = GBA_OK;
    std::vector<int4> img_items;       // image reduction items, image order
    std::vector<int> img_item_cnt;     // items per image
    std::vector<int2> pairs;           // key pairs of every block, block order
    std::vector<int2> blk_ij;          // (i, j) local image ids, i <= j
    std::vector<long long> blk_off;    // [nblk + 1] first pair of each block
    std::vector<int> blk_map;          // [ni * ni] local block id or -1 (dense solver)
    std::vector<int4> cons;
    std::vector<double2> cons_yw;
    std::vector<int> pt_rec_off;       // [np + 1] camera records of each point (free cameras)
    std::vector<int> rec_ext;          // local reduced-system image of each camera record
    std::vector<int> prior_pt;         // point priors: global point, observed y, information
    std::vector<double> prior_y, prior_info;
    long long n_pairs = 0;             // key pairs (blocks built on the device)
  };
  // work-item sizes of the Schur assembly and the image reduction
  const int pair_item = opt.pair_item > 0 ? opt.pair_item : kPairItem;
  const int image_item = opt.image_item > 0 ? opt.image_item : kImageItem;
  const int key_item = opt.key_item > 0 ? opt.key_item : kKeyChunk;
  // plans without free cameras count, number and place their key pairs on
  // the device (GBA_HOST_PAIRS=1 keeps the host build, for comparison); the
  // per-code tables take 12 bytes per (image, image) entry of every problem
  long long codes = 0;
  for (int q = 0; q < nprob; ++q) codes += (long long)prob[q].num_ext * prob[q].num_ext;
  const bool dev_blocks = !any_free && nprob <= 65535 && codes <= (1LL << 26) &&
                          std::getenv("GBA_HOST_PAIRS") == nullptr;
  std::vector<Piece> pieces(nprob);
  // fine phases of a single problem's build (GBA_BUILD_TIMING)
  auto sub = [&](const char* name) {
    if (timing && nprob == 1) phase(name);
  };
  auto build_one = [&](int q, int inner) {
    Piece& out = pieces[q];
    const gba_problem& p = problems[q];
    const int np = int(p.number_of_points), ni = int(p.number_of_images), nk = int(p.number_of_keys);
    const int64_t cps = params_per_camera(p.intrinsic_computations_mask);
    const int64_t pb = pbase[q], ib = ibase[q], kb = kbase[q], cb = cbase[q];
    const bool fc = cameras_free(p);
    const int Ie = prob[q].num_ext, ncp = prob[q].nc;
    // cameras (free ones are written on the device from x)
    for (int64_t c = 0; c < p.number_of_cameras; ++c) {
      double full[10] = {0, 0, 0, 0, 0, 1, 0, 0, 0, 1};
      if (!fc) expand_camera(p.intrinsic_computations_mask, p.fix_cameras + cps * c, full);
      for (int j = 0; j < 10; ++j) {
        cam64[10 * (cb + c) + j] = full[j];
        cam32[10 * (cb + c) + j] = float(full[j]);
      }
    }
    for (int i = 0; i < ni; ++i) {
      img_cam[ib + i] = int(cb + p.image_camera_map[i]);
      img_prob[ib + i] = q;
    }
    // point-major order: counting sort by point, then image within point
    const int nth0 = nk > 200000 ? inner : 1;
    std::vector<int> cnt, order;
    // keys that already come point-major (by point, then image, no repeats --
    // the usual track layout) need no sort: the order is the identity and
    // each point's first key is found where the point id steps
    const int64_t* fm = p.feature_maps;
    std::vector<char> unsorted(nth0, 0);
    host_parallel(nk, nth0, [&](int64_t k0, int64_t k1, int t) {
      for (int64_t k = std::max<int64_t>(k0, 1); k < k1; ++k) {
        const int64_t dp = fm[2 * k + 1] - fm[2 * k - 1];
        if (dp < 0 || (dp == 0 && fm[2 * k] <= fm[2 * k - 2])) {
          unsorted[t] = 1;
          break;
        }
      }
    });
    const bool presorted = std::find(unsorted.begin(), unsorted.end(), char(1)) == unsorted.end();
    if (presorted) {
      cnt.assign(size_t(np) + 1, nk);
      order.resize(size_t(nk));
      host_parallel(nk, nth0, [&](int64_t k0, int64_t k1, int) {
        for (int64_t k = k0; k < k1; ++k) {
          order[k] = int(k);
          // points prev+1 .. this one start at key k (points without keys too)
          const int64_t prev = k == 0 ? -1 : fm[2 * k - 1];
          for (int64_t i = prev + 1; i <= fm[2 * k + 1]; ++i) cnt[i] = int(k);
        }
      });
    } else {
      counting_sort(nk, np, nth0, [&](int64_t k) { return int(p.feature_maps[2 * k + 1]); }, cnt,
                    order);
    }
    if (!presorted) {
      std::vector<char> dup(nth0, 0);
      host_parallel(np, nth0, [&](int64_t i0, int64_t i1, int t) {
        constexpr int kShort = 32;   // tracks this long sort in registers
        int64_t im[kShort];
        int ix[kShort];
        for (int64_t i = i0; i < i1; ++i) {
          const int b0 = cnt[i], n = cnt[i + 1] - b0;
          if (n <= 1) continue;
          if (n <= kShort) {   // insertion sort of (image, key) (a repeated image is an error)
            for (int u = 0; u < n; ++u) {
              const int k = order[b0 + u];
              const int64_t v = fm[2 * k];
              int j = u - 1;
              while (j >= 0 && im[j] > v) {
                im[j + 1] = im[j];
                ix[j + 1] = ix[j];
                --j;
              }
              im[j + 1] = v;
              ix[j + 1] = k;
            }
            for (int u = 0; u < n; ++u) {
              order[b0 + u] = ix[u];
              if (u && im[u] == im[u - 1]) dup[t] = 1;
            }
            continue;
          }
          std::sort(order.begin() + b0, order.begin() + b0 + n, [&](int a, int b) { return fm[2 * a] < fm[2 * b]; });
          for (int u = b0 + 1; u < b0 + n; ++u)
            if (fm[2 * order[u]] == fm[2 * order[u - 1]]) dup[t] = 1;
        }
      });
      for (char v : dup)
        if (v) {
          out.err = GBA_ERR_DUPLICATE;
          return;
        }
    }
    const double* y = near_ys[q];
    {
      std::vector<char> bad(nth0, 0);
      host_parallel(nk, nth0, [&](int64_t t0_, int64_t t1_, int th) {
        for (int64_t t = t0_; t < t1_; ++t) {
          const int k = order[t];
          key_img[kb + t] = int(ib + p.feature_maps[2 * k]);
          key_pt[kb + t] = int(pb + p.feature_maps[2 * k + 1]);
          key_obs[kb + t] = make_double2(y[2 * k], y[2 * k + 1]);
          if (any_weights) {
            double l00 = 1, l10 = 0, l11 = 1;
            if (p.key_covariance_inverse) {
              const double* L = p.key_covariance_inverse + 4 * k;
              double a = L[0], bb = 0.5 * (L[1] + L[2]), dd = L[3];
              if (!(a > 0)) { bad[th] = 1; continue; }
              l00 = std::sqrt(a);
              l10 = bb / l00;
              double r = dd - l10 * l10;
              if (!(r > 0)) { bad[th] = 1; continue; }
              l11 = std::sqrt(r);
            }
            key_wl[3 * (kb + t)] = l00;
            key_wl[3 * (kb + t) + 1] = l10;
            key_wl[3 * (kb + t) + 2] = l11;
          }
        }
      });
      for (char v : bad)
        if (v) {
          out.err = GBA_ERR_INVALID;
          return;
        }
    }
    sub("  keys sorted");
    key_sorted_to_orig[q] = std::move(order);
    for (int i = 0; i < np; ++i) {   // entry pb is set by the caller
      pt_key_off[pb + i + 1] = int(kb + cnt[i + 1]);
      pt_prob[pb + i] = q;
    }
    // per-image key lists (by point, since keys are point-major)
    {
      std::vector<int> ic, lst;
      counting_sort(nk, ni, nth0, [&](int64_t t) { return key_img[kb + t] - int(ib); }, ic, lst);
      host_parallel(nk, nth0, [&](int64_t t0_, int64_t t1_, int) {
        for (int64_t t = t0_; t < t1_; ++t) img_keys[kb + t] = int(kb + lst[t]);
      });
      for (int i = 1; i <= ni; ++i) img_key_off[ib + i] = int(kb + ic[i]);   // entry ib: the caller
      out.img_item_cnt.assign(ni, 0);
      for (int i = 0; i < ni; ++i) {
        const int q0 = int(kb + ic[i]), q1 = int(kb + ic[i + 1]);
        for (int qq = q0; qq < q1; qq += image_item) {
          out.img_items.push_back(make_int4(int(ib + i), qq, std::min(q1, qq + image_item), q));
          out.img_item_cnt[i]++;
        }
      }
    }
    sub("  image lists");
    // free cameras: each point has nc camera records (one per 6-wide part)
    // for every distinct camera among its keys, ascending
    if (fc) {
      out.pt_rec_off.assign(np + 1, 0);
      auto point_cams = [&](int64_t i, std::vector<int>& cams) {
        cams.clear();
        for (int a = cnt[i]; a < cnt[i + 1]; ++a) cams.push_back(img_cam[key_img[kb + a]] - int(cb));
        std::sort(cams.begin(), cams.end());
        cams.erase(std::unique(cams.begin(), cams.end()), cams.end());
      };
      host_parallel(np, nth0, [&](int64_t i0, int64_t i1, int) {
        std::vector<int> cams;
        for (int64_t i = i0; i < i1; ++i) {
          point_cams(i, cams);
          out.pt_rec_off[i + 1] = int(cams.size()) * ncp;
        }
      });
      for (int i = 0; i < np; ++i) out.pt_rec_off[i + 1] += out.pt_rec_off[i];
      out.rec_ext.resize(out.pt_rec_off[np]);
      host_parallel(np, nth0, [&](int64_t i0, int64_t i1, int) {
        std::vector<int> cams;
        for (int64_t i = i0; i < i1; ++i) {
          point_cams(i, cams);
          int o = out.pt_rec_off[i];
          for (int c : cams)
            for (int h = 0; h < ncp; ++h) out.rec_ext[o++] = ni + c * ncp + h;
        }
      });
    }
    // The Z records of point i with their reduced-system images, ascending:
    // its keys (the key index), then its camera records (-(local record + 1)).
    auto point_records = [&](int64_t i, std::vector<int2>& rec) {
      rec.clear();
      for (int a = cnt[i]; a < cnt[i + 1]; ++a) rec.push_back(make_int2(key_img[kb + a] - int(ib), int(kb + a)));
      if (fc)
        for (int r = out.pt_rec_off[i]; r < out.pt_rec_off[i + 1]; ++r)
          rec.push_back(make_int2(out.rec_ext[r], -(r + 1)));
    };
    sub("  records");
    // plans that build their blocks on the device (after this phase) only
    // need the pair count here
    if (dev_blocks) {
      long long t = 0;
      for (int i = 0; i < np; ++i) {
        const long long k = cnt[i + 1] - cnt[i];
        t += k * (k + 1) / 2;
      }
      out.n_pairs = t;
    }
    // reduced-system blocks: (i <= j) with their record pairs, point order.
    // Pairs are counted and placed by point ranges in parallel: each piece
    // counts its pairs per image pair, a piece's pairs of a block follow
    // those of the pieces before it, so every block lists its pairs in
    // point order whatever the number of pieces.
    if (!dev_blocks) {
      const size_t nn = (size_t)Ie * Ie;
      int nth = nth0;
      while (nth > 1 && nn * size_t(nth) * sizeof(int) > (size_t(256) << 20)) --nth;
      std::vector<int64_t> cuts(nth + 1, np);
      for (int t = 0; t < nth; ++t)   // pieces of about equal key counts
        cuts[t] = std::lower_bound(cnt.begin(), cnt.end() - 1, int((int64_t)nk * t / nth)) - cnt.begin();
      cuts[0] = 0;
      std::vector<std::vector<int>> cnt_t(nth, std::vector<int>(nn, 0));
      host_parallel(np, nth, [&](int64_t i0, int64_t i1, int t) {
        int* bc = cnt_t[t].data();
        std::vector<int2> rec;
        for (int64_t i = i0; i < i1; ++i) {
          if (!fc) {   // keys only: straight from the point's key range
            const int b0 = cnt[i], b1 = cnt[i + 1];
            for (int a = b0; a < b1; ++a) {
              const size_t row = (size_t)(key_img[kb + a] - int(ib)) * Ie;
              for (int c = a; c < b1; ++c) bc[row + key_img[kb + c] - int(ib)]++;
            }
            continue;
          }
          point_records(i, rec);
          const int nr = int(rec.size());
          for (int a = 0; a < nr; ++a) {
            const size_t row = (size_t)rec[a].x * Ie;
            for (int c = a; c < nr; ++c) bc[row + rec[c].x]++;
          }
        }
      }, &cuts);
      std::vector<long long> bcount(nn, 0);
      for (int t = 0; t < nth; ++t)
        for (size_t e = 0; e < nn; ++e) bcount[e] += cnt_t[t][e];
      // every reduced-system image gets a diagonal block (so S keeps U_i + mu I
      // even for an image without keys)
      std::vector<int> bid(nn, -1);
      long long acc = 0;
      for (int a = 0; a < Ie; ++a)
        for (int c = a; c < Ie; ++c) {
          const long long n_ = bcount[(size_t)a * Ie + c];
          if (n_ == 0 && a != c) continue;
          bid[(size_t)a * Ie + c] = int(out.blk_ij.size());
          out.blk_ij.push_back(make_int2(a, c));
          out.blk_off.push_back(acc);
          acc += n_;
        }
      out.blk_off.push_back(acc);
      if (acc > INT32_MAX) {
        out.err = GBA_ERR_INVALID;
        return;
      }
      {
        // cnt_t[t][e] becomes piece t's first slot in block e
        for (size_t e = 0; e < nn; ++e) {
          if (bid[e] < 0) continue;
          long long o = out.blk_off[bid[e]];
          for (int t = 0; t < nth; ++t) {
            const int c_ = cnt_t[t][e];
            cnt_t[t][e] = int(o);
            o += c_;
          }
        }
        sub("  pair counts");
        out.pairs.resize(acc);
        host_parallel(np, nth, [&](int64_t i0, int64_t i1, int t) {
          int* slot = cnt_t[t].data();
          std::vector<int2> rec;
          for (int64_t i = i0; i < i1; ++i) {
            if (!fc) {
              const int b0 = cnt[i], b1 = cnt[i + 1];
              for (int a = b0; a < b1; ++a) {
                const size_t row = (size_t)(key_img[kb + a] - int(ib)) * Ie;
                for (int c = a; c < b1; ++c)
                  out.pairs[slot[row + key_img[kb + c] - int(ib)]++] =
                      make_int2(int(kb + a), a == c ? int(pb + i) : int(kb + c));
              }
              continue;
            }
            point_records(i, rec);
            const int nr = int(rec.size());
            for (int a = 0; a < nr; ++a) {
              const size_t row = (size_t)rec[a].x * Ie;
              for (int c = a; c < nr; ++c) {
                // a pair of a diagonal block is a record with itself: carry its point instead
                out.pairs[slot[row + rec[c].x]++] =
                    make_int2(rec[a].y, a == c ? int(pb + i) : rec[c].y);
              }
            }
          }
        }, &cuts);
        sub("  pairs placed");
      }
      // dense map for the assembly of the lower triangle: map[j*Ie + i], j <= i
      if (!pcg) out.blk_map.swap(bid);
    }
    // soft constraints in y order (camera_shared_vector_function.hpp:483-629):
    // the rows after the keys, each a copy of one parameter with its own
    // weight; camera constraints have rows only while the cameras are free
    {
      int64_t r = 0;
      auto add = [&](int group, int64_t index, int param) {
        out.cons.push_back(make_int4(group, int(index), param, q));
        out.cons_yw.push_back(make_double2(y[2LL * nk + r],
                                           p.constraint_weights ? p.constraint_weights[r] : 1.0));
        ++r;
      };
      const bool fixP = p.fix_mask & GBA_FIX_POINTS, fixI = p.fix_mask & GBA_FIX_IMAGES;
      for (int64_t c = 0; c < (fixP ? 0 : p.number_of_point_constraints); ++c) {
        const gba_point_constraint& pc = p.point_constraints[c];
        for (int b = 0; b < 3; ++b)
          if (pc.mask & (1u << b)) add(0, pb + pc.point_id, b);
      }
      for (int64_t c = 0; c < (fixI ? 0 : p.number_of_image_constraints); ++c) {
        const gba_image_constraint& ic = p.image_constraints[c];
        if (ic.mask & GBA_IMAGE_CONSTRAIN_ROTATION)
          for (int b = 0; b < 3; ++b) add(1, ib + ic.image_id, b);
        if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_X) add(1, ib + ic.image_id, 3);
        if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_Y) add(1, ib + ic.image_id, 4);
        if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_Z) add(1, ib + ic.image_id, 5);
      }
      if (fc) {   // parameter indices in the problem's camera order
        const uint32_t m = p.intrinsic_computations_mask;
        for (int64_t c = 0; c < p.number_of_camera_constraints; ++c) {
          const gba_camera_constraint& cc = p.camera_constraints[c];
          int off = 0;
          for (int b = 0; b < 3; ++b)
            if (cc.radial_mask & (1u << b)) add(2, cb + cc.camera_id, off + b);
          if (m & GBA_COMPUTE_RADIAL_DISTORTION) off += 3;
          for (int b = 0; b < 2; ++b)
            if (cc.decentering_mask & (1u << b)) add(2, cb + cc.camera_id, off + b);
          if (m & GBA_COMPUTE_DECENTERING_DISTORTION) off += 2;
          for (int b = 0; b < 5; ++b)
            if (cc.intrinsic_mask & (1u << b)) add(2, cb + cc.camera_id, off + b);
        }
      }
      // point priors: 3 rows each after the constraint rows
      // (ba_gcp_constrained_vector_function.hpp:100-108)
      for (int64_t i = 0; i < p.number_of_point_priors; ++i) {
        out.prior_pt.push_back(int(pb + p.point_prior_ids[i]));
        for (int a = 0; a < 3; ++a) out.prior_y.push_back(y[2LL * nk + r + 3 * i + a]);
        for (int j = 0; j < 9; ++j)
          out.prior_info.push_back(p.point_prior_information ? p.point_prior_information[9 * i + j]
                                                             : double(j % 4 == 0));
      }
    }
  };
  if (nprob == 1) {
    build_one(0, host_threads());
  } else {
    // the largest problems first, so no large one starts last
    std::vector<int> by_size(nprob);
    for (int q = 0; q < nprob; ++q) by_size[q] = q;
    std::stable_sort(by_size.begin(), by_size.end(), [&](int a, int b) {
      return problems[a].number_of_keys > problems[b].number_of_keys;
    });
    const int nth = std::min(host_threads(), nprob);
    std::atomic<int> next{0};
    host_parallel(nth, nth, [&](int64_t, int64_t, int) {
      for (int u = next++; u < nprob; u = next++) build_one(by_size[u], 1);
    });
  }
  for (int q = 0; q < nprob; ++q)
    if (pieces[q].err) return pieces[q].err;
  phase("problems");

  // ---- blocks on the device: the keys go up now, the device counts the
  // pairs of every code and returns the block list, which is split into the
  // problems' pieces (the layout of the host's count, block for block)
  int* dv_key_img = nullptr;
  int* dv_pt_key_off = nullptr;
  int* dv_pt_prob = nullptr;
  int* dv_bid = nullptr;
  int4* dv_pinfo = nullptr;
  int dv_blocks = 0;
  std::vector<int> code_base(nprob, 0);
  if (dev_blocks) {
    for (int q = 0; q < nprob; ++q) pt_key_off[pbase[q]] = int(kbase[q]);
    pt_key_off[P] = int(K);
    std::vector<int4> pinfo(nprob);
    long long L = 0, ub = 0, total = 0, min_blocks = 0;
    int qlast = -1, max_ie = 0;
    for (int q = 0; q < nprob; ++q) {
      const int n = prob[q].num_ext;   // the images (no free cameras)
      pinfo[q] = make_int4(int(ibase[q]), n, int(L), 0);
      code_base[q] = int(L);
      L += (long long)n * n;
      ub += (long long)n * (n + 1) / 2;
      min_blocks += n;
      if (n > 0) qlast = q;
      max_ie = std::max(max_ie, n);
      total += pieces[q].n_pairs;
    }
    if (total > INT32_MAX) return GBA_ERR_INVALID;
    dv_key_img = arena.upload(key_img);
    dv_pt_key_off = arena.upload(pt_key_off);
    dv_pt_prob = arena.upload(pt_prob);
    dv_pinfo = arena.upload(pinfo);
    std::vector<int> code, first, pblk(nprob, 0);
    if (qlast >= 0) {
      int* d_cnt = arena.alloc<int>(size_t(L));
      int* d_off = arena.alloc<int>(size_t(L));
      dv_bid = arena.alloc<int>(size_t(L));
      int* d_scratch = arena.alloc<int>(size_t(scan_scratch_ints(L)));
      int* d_code = arena.alloc<int>(size_t(ub));
      int* d_first = arena.alloc<int>(size_t(ub));
      int* d_pblk = arena.alloc<int>(size_t(nprob));
      int* d_info = arena.alloc<int>(2);
      const int nl = count_blocks_on_device(nprob, qlast, max_ie, int(P), dv_pinfo, dv_pt_key_off, dv_key_img,
                                            dv_pt_prob, L, d_cnt, dv_bid, d_off, d_scratch, d_code, d_first,
                                            d_pblk, d_info, stream);
      if (nl < 0) return GBA_ERR;
      count_launches(nl);
      GBA_CUDA(cudaGetLastError());
      int info[2] = {0, 0};
      GBA_CUDA(cudaMemcpyAsync(info, d_info, sizeof(info), cudaMemcpyDeviceToHost, stream));
      GBA_CUDA(cudaStreamSynchronize(stream));
      dv_blocks = info[0];
      if (info[1] != total || dv_blocks < min_blocks || dv_blocks > ub) return GBA_ERR;   // never expected
      code.resize(dv_blocks);
      first.resize(dv_blocks);
      GBA_CUDA(cudaMemcpyAsync(code.data(), d_code, sizeof(int) * code.size(), cudaMemcpyDeviceToHost, stream));
      GBA_CUDA(cudaMemcpyAsync(first.data(), d_first, sizeof(int) * first.size(), cudaMemcpyDeviceToHost, stream));
      GBA_CUDA(cudaMemcpyAsync(pblk.data(), d_pblk, sizeof(int) * nprob, cudaMemcpyDeviceToHost, stream));
      GBA_CUDA(cudaStreamSynchronize(stream));
    }
    // problem q's blocks run from its first block to the next problem's with images
    std::vector<int> pend(nprob, dv_blocks);
    for (int q = nprob - 2, nxt = dv_blocks; q >= 0; --q) {
      if (prob[q + 1].num_ext > 0) nxt = pblk[q + 1];
      pend[q] = nxt;
    }
    bool bad = false;
    long long pair_base = 0;
    for (int q = 0; q < nprob; ++q) {
      Piece& pc = pieces[q];
      const int n = prob[q].num_ext;
      pc.blk_ij.clear();
      pc.blk_off.assign(1, 0);
      if (n > 0) {
        const int b0 = pblk[q], b1 = pend[q];
        if (b0 < 0 || b1 < b0 || b1 > dv_blocks || first[b0] != pair_base) {
          bad = true;
          break;
        }
        pc.blk_ij.resize(b1 - b0);
        pc.blk_off.resize(size_t(b1 - b0) + 1);
        for (int t = b0; t < b1; ++t) {
          pc.blk_ij[t - b0] = make_int2(code[t] / n, code[t] % n);
          pc.blk_off[t - b0] = first[t] - pair_base;
        }
        pc.blk_off[b1 - b0] = pc.n_pairs;
      }
      pair_base += pc.n_pairs;
    }
    if (bad) return GBA_ERR;   // the device's blocks disagree with the counts: never expected
    phase("blocks (device)");
  }

  // ---- concatenation in problem order: a serial pass sizes every list and
  // gives each problem its slices, then the problems fill them in parallel
  // (the layout is exactly that of appending the problems one after another)
  // camera records are Z records K .. K+R-1, after the keys
  struct Bases {
    long long img_items = 0, pairs = 0, recs = 0, blocks = 0, items = 0, blk_map = 0;
    long long key_chunks = 0, pt_chunks = 0, img_chunks = 0, cons = 0, priors = 0;
  };
  std::vector<Bases> base(nprob + 1);
  for (int q = 0; q < nprob; ++q) {
    const Piece& pc = pieces[q];
    const gba_problem& p = problems[q];
    const long long np = p.number_of_points, ni = p.number_of_images, nk = p.number_of_keys;
    Bases b = base[q];
    b.img_items += (long long)pc.img_items.size();
    b.pairs += pc.blk_off.empty() ? 0 : pc.blk_off.back();   // on the host or (below) the device
    b.recs += (long long)pc.rec_ext.size();
    const long long nblk = (long long)pc.blk_ij.size();
    b.blocks += nblk;
    for (long long t = 0; t < nblk; ++t) {
      const long long cntp = pc.blk_off[t + 1] - pc.blk_off[t];
      b.items += std::max<long long>(1, (cntp + pair_item - 1) / pair_item);
    }
    b.blk_map += (long long)pc.blk_map.size();
    b.key_chunks += (nk + key_item - 1) / key_item;
    b.pt_chunks += (np + kPointChunk - 1) / kPointChunk;
    b.img_chunks += (ni + kImageChunk - 1) / kImageChunk;
    b.cons += (long long)pc.cons.size();
    b.priors += (long long)pc.prior_pt.size();
    base[q + 1] = b;
  }
  const Bases& tot = base[nprob];
  if (tot.pairs > INT32_MAX || (long long)K + tot.recs > INT32_MAX || tot.items > INT32_MAX)
    return GBA_ERR_INVALID;
  n_pairs = tot.pairs;
  img_items.resize(tot.img_items);
  img_item_off.assign(size_t(I) + 1, 0);
  // the pair lists (the largest array): one problem's list moves into place;
  // a batch's lists go straight from each problem to its slice on the device
  int2* d_pairs = nprob > 1 && !dev_blocks ? arena.alloc<int2>(size_t(tot.pairs)) : nullptr;
  std::atomic<int> pair_upload_failed{0};
  std::vector<int> pt_rec_off;
  std::vector<int2> rec_info(tot.recs);
  if (any_free) pt_rec_off.assign(P + 1, int(K));
  blk_ij.resize(tot.blocks);
  blk_item_off.assign(size_t(tot.blocks) + 1, 0);
  items.resize(tot.items);
  if (!pcg) {
    if (nprob == 1)
      blk_map.swap(pieces[0].blk_map);
    else
      blk_map.resize(tot.blk_map);
  }
  key_chunks.resize(tot.key_chunks);
  pt_chunks.resize(tot.pt_chunks);
  img_chunks.resize(tot.img_chunks);
  cons.resize(tot.cons);
  cons_yw.resize(tot.cons);
  prior_pt.resize(tot.priors);
  prior_y.resize(3 * tot.priors);
  prior_info.resize(9 * tot.priors);
  prob_key_chunk_off.assign(nprob + 1, 0);
  prob_pt_chunk_off.assign(nprob + 1, 0);
  prob_img_chunk_off.assign(nprob + 1, 0);
  prob_cons_off.assign(nprob + 1, 0);
  prob_prior_off.assign(nprob + 1, 0);
  for (int q = 0; q < nprob; ++q) {   // first entries (shared with the previous problem's last)
    pt_key_off[pbase[q]] = int(kbase[q]);
    img_key_off[ibase[q]] = int(kbase[q]);
  }
  for (int q = 0; q <= nprob; ++q) {
    prob_key_chunk_off[q] = int(base[q].key_chunks);
    prob_pt_chunk_off[q] = int(base[q].pt_chunks);
    prob_img_chunk_off[q] = int(base[q].img_chunks);
    prob_cons_off[q] = int(base[q].cons);
    prob_prior_off[q] = int(base[q].priors);
  }
  auto fill_one = [&](int q) {
    Piece& pc = pieces[q];
    ProbInfo& pi = prob[q];
    const gba_problem& p = problems[q];
    const Bases& b = base[q];
    const int np = int(p.number_of_points), ni = int(p.number_of_images), nk = int(p.number_of_keys);
    const int64_t pb = pbase[q], ib = ibase[q], kb = kbase[q];
    std::copy(pc.img_items.begin(), pc.img_items.end(), img_items.begin() + b.img_items);
    for (int i = 0, acc = int(b.img_items); i < ni; ++i) {
      acc += pc.img_item_cnt[i];
      img_item_off[ib + i + 1] = acc;
    }
    const long long rec_base = (long long)K + b.recs;
    if (!pc.rec_ext.empty()) {
      for (int2& pr : pc.pairs) {   // camera records: -(local + 1) -> global record
        if (pr.x < 0) pr.x = int(rec_base - 1 - pr.x);
        if (pr.y < 0) pr.y = int(rec_base - 1 - pr.y);
      }
      for (int i = 0; i < np; ++i) pt_rec_off[pb + i] = int(rec_base + pc.pt_rec_off[i]);
      for (size_t r = 0; r < pc.rec_ext.size(); ++r) {
        const int e = pc.rec_ext[r];
        rec_info[b.recs + r] = make_int2(int(cbase[q]) + (e - ni) / pi.nc, pi.ext_begin + e);
      }
    } else if (any_free) {
      for (int i = 0; i < np; ++i) pt_rec_off[pb + i] = int(rec_base);
    }
    if (nprob == 1)
      pairs.swap(pc.pairs);
    else if (!pc.pairs.empty() &&
             cudaMemcpyAsync(d_pairs + b.pairs, pc.pairs.data(), sizeof(int2) * pc.pairs.size(),
                             cudaMemcpyHostToDevice, stream) != cudaSuccess)
      pair_upload_failed = 1;
    const int block_begin = int(b.blocks);
    std::copy(pc.blk_ij.begin(), pc.blk_ij.end(), blk_ij.begin() + b.blocks);
    const int nblk = int(pc.blk_ij.size());
    pi.block_begin = block_begin;
    pi.num_blocks = nblk;
    pi.item_begin = int(b.items);
    long long it = b.items;
    for (int t = 0; t < nblk; ++t) {
      const long long s0 = b.pairs + pc.blk_off[t], s1 = b.pairs + pc.blk_off[t + 1];
      long long s_ = s0;
      do {
        const long long e = std::min(s1, s_ + pair_item);
        items[it++] = make_int4(block_begin + t, int(s_), int(e), q);
        s_ = e;
      } while (s_ < s1);
      blk_item_off[block_begin + t + 1] = int(it);
    }
    pi.num_items = int(it - b.items);
    blk_map_off[q] = dev_blocks ? code_base[q] : b.blk_map;
    if (!pcg && nprob > 1)
      for (size_t e = 0; e < pc.blk_map.size(); ++e)
        blk_map[b.blk_map + e] = pc.blk_map[e] >= 0 ? pc.blk_map[e] + block_begin : -1;
    // work chunks
    long long c = b.key_chunks;
    for (int s_ = 0; s_ < nk; s_ += key_item)
      key_chunks[c++] = Chunk{q, int(kb + s_), int(kb + std::min(nk, s_ + key_item)), 0};
    c = b.pt_chunks;
    for (int s_ = 0; s_ < np; s_ += kPointChunk)
      pt_chunks[c++] = Chunk{q, int(pb + s_), int(pb + std::min(np, s_ + kPointChunk)), 0};
    c = b.img_chunks;
    for (int s_ = 0; s_ < ni; s_ += kImageChunk)
      img_chunks[c++] = Chunk{q, int(ib + s_), int(ib + std::min(ni, s_ + kImageChunk)), 0};
    std::copy(pc.cons.begin(), pc.cons.end(), cons.begin() + b.cons);
    std::copy(pc.cons_yw.begin(), pc.cons_yw.end(), cons_yw.begin() + b.cons);
    std::copy(pc.prior_pt.begin(), pc.prior_pt.end(), prior_pt.begin() + b.priors);
    std::copy(pc.prior_y.begin(), pc.prior_y.end(), prior_y.begin() + 3 * b.priors);
    std::copy(pc.prior_info.begin(), pc.prior_info.end(), prior_info.begin() + 9 * b.priors);
    std::vector<int>().swap(pc.blk_map);   // release as we go
    std::vector<int2>().swap(pc.pairs);
  };
  if (nprob == 1) {
    fill_one(0);
  } else {
    const int nth = std::min(host_threads(), nprob);
    std::atomic<int> next{0};
    host_parallel(nth, nth, [&](int64_t, int64_t, int) {
      for (int q = next++; q < nprob; q = next++) fill_one(q);
    });
  }
  if (pair_upload_failed) {
    cudaGetLastError();
    throw CudaError{GBA_ERR_CUDA};
  }
  if (d_pairs) arena.uploaded += (long long)(sizeof(int2) * tot.pairs);
  pt_key_off[P] = int(K);
  img_key_off[I] = int(K);
  const int R = int(rec_info.size());
  if (any_free) pt_rec_off[P] = int(K) + R;

  phase("host structure");
  // ---- device allocations
  DevPlan& D = d;
  D.B = nprob;
  D.precision = opt.precision;
  D.loss = opt.loss;
  D.huber_delta = opt.huber_delta;
  D.tau = opt.tau;
  D.eps1 = opt.eps1;
  D.eps2 = opt.eps2;
  D.ftol = opt.function_tolerance;
  D.max_iterations = opt.max_iterations;
  D.has_key_weights = any_weights;
  D.max_n = max_n;
  D.max_nt = max_nt;
  D.prob = arena.upload(prob);
  D.state = arena.alloc<LMState>(nprob);
  D.K = int(K);
  D.key_img = dv_key_img ? dv_key_img : arena.upload(key_img);
  D.key_pt = arena.upload(key_pt);
  D.key_obs = arena.upload(key_obs);
  D.key_wl = any_weights ? arena.upload(key_wl) : nullptr;
  D.P = int(P);
  D.pt_key_off = dv_pt_key_off ? dv_pt_key_off : arena.upload(pt_key_off);
  D.pt_prob = dv_pt_prob ? dv_pt_prob : arena.upload(pt_prob);
  D.I = int(I);
  D.img_key_off = arena.upload(img_key_off);
  D.img_keys = arena.upload(img_keys);
  D.img_prob = arena.upload(img_prob);
  D.img_cam = arena.upload(img_cam);
  D.n_img_items = int(img_items.size());
  D.img_items = arena.upload(img_items);
  D.img_item_off = arena.upload(img_item_off);
  D.img_item_partial = arena.alloc<double>(28 * std::max<size_t>(img_items.size(), 1));
  // with free cameras each parity has its own camera arrays (the fixed
  // cameras' values in both)
  D.cam64[0] = arena.upload(cam64);
  D.cam32[0] = arena.upload(cam32);
  D.cam64[1] = any_free ? arena.upload(cam64) : D.cam64[0];
  D.cam32[1] = any_free ? arena.upload(cam32) : D.cam32[0];
  D.cam_ff[0] = D.cam_ff[1] = nullptr;
  if (mixed) {
    std::vector<float2> cam_ff(10 * std::max<int64_t>(C, 1));
    auto split = [](double v) {
      float hi = float(v);
      return make_float2(hi, float(v - double(hi)));
    };
    for (int64_t c = 0; c < C; ++c) {
      for (int j = 0; j < 9; ++j) cam_ff[10 * c + j] = split(cam64[10 * c + j]);
      cam_ff[10 * c + 9] = split(cam64[10 * c + 5] * cam64[10 * c + 9]);   // f * a
    }
    // the keys' double-float pairs are split on the device from key_obs
    float2* obs_ff = arena.alloc<float2>(2 * K);
    launch_split_keys(D, obs_ff, stream);
    count_launches(1);
    D.key_obs_ff = obs_ff;
    D.cam_ff[0] = arena.upload(cam_ff);
    D.cam_ff[1] = any_free ? arena.upload(cam_ff) : D.cam_ff[0];
  }
  for (int t = 0; t < 2; ++t) {
    D.img_rot_ff[t] = mixed ? arena.alloc<float2>(12 * I) : nullptr;
    D.x_ff[t] = mixed ? arena.alloc<float2>(3 * P) : nullptr;
    D.x_pt[t] = arena.alloc<double>(3 * P);
    D.x_img[t] = arena.alloc<double>(6 * I);
    D.img_rot[t] = arena.alloc<double>(12 * I);
    D.img_lin[t] = arena.alloc<char>(12 * I * tsz);
    D.RW[t] = arena.alloc<char>(4 * K * tsz);
  }
  D.x0_pt = arena.alloc<double>(3 * P);
  D.x0_img = arena.alloc<double>(6 * I);
  D.JR[0] = arena.alloc<char>(size_t(kJRStride) * K * tsz);
  D.JR[1] = arena.alloc<char>(size_t(kJRStride) * K * tsz);
  // GBA_SEPARATE_LINEARIZE=1: every iteration relinearizes in its own launch
  D.fuse_lin = std::getenv("GBA_SEPARATE_LINEARIZE") == nullptr;
  D.z_n = (K + R + 31) / 32 * 32;
  D.Z = arena.alloc<char>(std::max<size_t>(size_t(kZStride) * (K + R), 18 * size_t(D.z_n)) * tsz);
  D.PV = arena.alloc<char>(12 * P * tsz);
  D.PS = arena.alloc<char>(12 * P * tsz);
  D.U = arena.alloc<double>(36 * I);
  D.gi = arena.alloc<double>(6 * I);
  D.S = arena.alloc<char>(size_t(std::max<long long>(s_off, 1)) * tsz);
  D.b = arena.alloc<char>(size_t(std::max<int64_t>(6 * I_ext, 1)) * tsz);
  D.Linv = arena.alloc<char>(pcg ? 1 : size_t(nprob) * std::max(max_nt, 1) * kTile * kTile * tsz);
  D.factor_flag = arena.alloc<int>(nprob);
  D.free_cams = any_free ? 1 : 0;
  D.Ctot = int(C);
  D.R = R;
  D.I_ext = int(I_ext);
  if (any_free) {
    std::vector<int> img_ext(I), cam_img_off(C + 1, 0), cam_imgs(I);
    std::vector<int4> cam_info(C);
    for (int q = 0; q < nprob; ++q) {
      const ProbInfo& pq = prob[q];
      for (int i = 0; i < pq.num_images; ++i) img_ext[pq.image_begin + i] = pq.ext_begin + i;
      for (int c = 0; c < pq.num_cams; ++c)
        cam_info[pq.cam_begin + c] =
            make_int4(pq.cps, int(problems[q].intrinsic_computations_mask), q,
                      pq.cps ? pq.ext_begin + pq.num_images + c * pq.nc : 0);
    }
    for (int64_t i = 0; i < I; ++i) cam_img_off[img_cam[i] + 1]++;
    for (int64_t c = 0; c < C; ++c) cam_img_off[c + 1] += cam_img_off[c];
    {
      std::vector<int> fill(cam_img_off.begin(), cam_img_off.end() - 1);
      for (int64_t i = 0; i < I; ++i) cam_imgs[fill[img_cam[i]]++] = int(i);
    }
    std::vector<int> prob_cam_off(nprob + 1);
    for (int q = 0; q <= nprob; ++q) prob_cam_off[q] = int(cbase[q]);
    D.img_ext = arena.upload(img_ext);
    D.cam_info = arena.upload(cam_info);
    D.cam_img_off = arena.upload(cam_img_off);
    D.cam_imgs = arena.upload(cam_imgs);
    D.prob_cam_off = arena.upload(prob_cam_off);
    D.x_cam[0] = arena.alloc<double>(10 * C);
    D.x_cam[1] = arena.alloc<double>(10 * C);
    D.x0_cam = arena.alloc<double>(10 * C);
    GBA_CUDA(cudaMemsetAsync(D.x0_cam, 0, sizeof(double) * 10 * std::max<int64_t>(C, 1), stream));
    D.JC[0] = arena.alloc<char>(size_t(20) * K * tsz);
    D.JC[1] = arena.alloc<char>(size_t(20) * K * tsz);
    D.pt_rec_off = arena.upload(pt_rec_off);
    D.rec_info = arena.upload(rec_info);
    D.img_item_cam = arena.alloc<double>(size_t(kImgCamVals) * std::max<size_t>(img_items.size(), 1));
    D.Ei = arena.alloc<double>(60 * I);
    D.img_cam_sum = arena.alloc<double>(size_t(kImgCamVals) * std::max<int64_t>(I, 1));
    D.Uc = arena.alloc<double>(100 * C);
    D.gc = arena.alloc<double>(10 * C);
    D.cam_sum = arena.alloc<double>(3 * C);
    GBA_CUDA(cudaMemsetAsync(D.cam_sum, 0, sizeof(double) * 3 * std::max<int64_t>(C, 1), stream));
  }
  D.df_grid = 0;
  D.df_trace = nullptr;
  D.pcg = pcg ? 1 : 0;
  D.pcg_max_iterations = opt.pcg_max_iterations;
  D.pcg_tol2 = opt.pcg_relative_tolerance * opt.pcg_relative_tolerance;
  if (pcg) {
    // block-sparse reduced system over the reduced-system images (images,
    // then the camera parts of free cameras): the global pair of each
    // block, the diagonal block of each, and each one's blocks by neighbour
    const int64_t E = I_ext;
    const size_t nb = blk_ij.size();
    std::vector<int2> blk_gij(nb);
    std::vector<int> img_diag_blk(E, -1), adj_off(E + 1, 0), ext_prob(E, 0);
    std::vector<Chunk> ext_chunks;
    std::vector<int> prob_ext_chunk_off(1, 0);
    for (int q = 0; q < nprob; ++q) {
      const ProbInfo& pq = prob[q];
      for (int t = pq.block_begin; t < pq.block_begin + pq.num_blocks; ++t)
        blk_gij[t] = make_int2(pq.ext_begin + blk_ij[t].x, pq.ext_begin + blk_ij[t].y);
      for (int e = 0; e < pq.num_ext; ++e) ext_prob[pq.ext_begin + e] = q;
      for (int e = 0; e < pq.num_ext; e += kImageChunk)
        ext_chunks.push_back(Chunk{q, pq.ext_begin + e, pq.ext_begin + std::min(pq.num_ext, e + kImageChunk), 0});
      prob_ext_chunk_off.push_back(int(ext_chunks.size()));
    }
    for (size_t t = 0; t < nb; ++t) {
      adj_off[blk_gij[t].x + 1]++;
      if (blk_gij[t].y != blk_gij[t].x) adj_off[blk_gij[t].y + 1]++;
      else img_diag_blk[blk_gij[t].x] = int(t);
    }
    for (int64_t i = 0; i < E; ++i) adj_off[i + 1] += adj_off[i];
    std::vector<int2> adj(adj_off[E]);
    std::vector<int> fill(adj_off.begin(), adj_off.end() - 1);
    for (size_t t = 0; t < nb; ++t) {
      const int a = blk_gij[t].x, c = blk_gij[t].y;
      adj[fill[a]++] = make_int2(int(t), c << 1);
      if (c != a) adj[fill[c]++] = make_int2(int(t), a << 1 | 1);
    }
    for (int64_t i = 0; i < E; ++i)
      std::sort(adj.begin() + adj_off[i], adj.begin() + adj_off[i + 1],
                [](const int2& u, const int2& v) { return (u.y >> 1) < (v.y >> 1); });
    for (int64_t i = 0; i < E; ++i)
      if (img_diag_blk[i] < 0) return GBA_ERR;   // every reduced-system image has its diagonal block
    D.blk_gij = arena.upload(blk_gij);
    D.img_diag_blk = arena.upload(img_diag_blk);
    D.adj_off = arena.upload(adj_off);
    D.adj = arena.upload(adj);
    D.ext_prob = arena.upload(ext_prob);
    D.ext_chunks = arena.upload(ext_chunks);
    D.n_ext_chunks = int(ext_chunks.size());
    D.prob_ext_chunk_off = arena.upload(prob_ext_chunk_off);
    D.Sblk = arena.alloc<char>(std::max<size_t>(nb, 1) * 36 * tsz);
    D.Minv = arena.alloc<char>(size_t(std::max<int64_t>(E, 1)) * 36 * tsz);
    const size_t v6 = size_t(std::max<int64_t>(6 * E, 1)) * tsz;
    D.pcg_r = arena.alloc<char>(v6);
    D.pcg_z = arena.alloc<char>(v6);
    D.pcg_q = arena.alloc<char>(v6);
    D.pcg_p[0] = arena.alloc<char>(v6);
    D.pcg_p[1] = arena.alloc<char>(v6);
    D.pcg_part = arena.alloc<double>(kPcgSlots * std::max<size_t>(ext_chunks.size(), 1));
    D.pcg_done = arena.alloc<int>(nprob);
    // GBA_PCG_UNROLLED=1 keeps one launch pair per iteration in graphs too
    if (std::getenv("GBA_PCG_UNROLLED") == nullptr) {
      D.pcg_it = arena.alloc<int>(4);
      D.pcg_extra = reinterpret_cast<unsigned long long*>(D.pcg_it + 2);
      GBA_CUDA(cudaMemsetAsync(D.pcg_it, 0, 4 * sizeof(int), stream));
      GBA_CUDA(cudaStreamCreateWithFlags(&pcg_stream, cudaStreamNonBlocking));
      GBA_CUDA(cudaHostAlloc(&h_pcg_extra, sizeof(unsigned long long), cudaHostAllocDefault));
      *h_pcg_extra = 0;
      D.pcg_body_stream = pcg_stream;
    }
  }
  if (!pcg)
    if (int e = prepare_cholesky_solve(max_nt, opt.precision)) return e;
  // bounded waits of the cluster backward solve; GBA_SOLVE_SPIN_LIMIT lowers
  // the limit and GBA_SOLVE_DROP_STEP withholds one step's delta, to test
  // that path
  D.solve_spin_limit = 1LL << 22;
  D.solve_drop_step = -1;
  if (const char* sl = std::getenv("GBA_SOLVE_SPIN_LIMIT")) {
    const long long v = std::atoll(sl);
    if (v > 0) D.solve_spin_limit = v;
  }
  if (const char* ds = std::getenv("GBA_SOLVE_DROP_STEP")) {
    const int v = std::atoi(ds);
    if (v >= 0) D.solve_drop_step = v;
  }
  if (!pcg && nprob == 1 && !opt.shared_device && max_nt >= 2) {
    int grid = 0, mo = 0;
    std::vector<int> own_off;
    std::vector<int2> own;
    if (dataflow_layout(max_nt, mixed, device, &grid, &mo, &own_off, &own)) {
      D.df_grid = grid;
      D.df_max_own = mo;
      // bounded waits: a CTA that finds nothing ready for this many polls
      // records GBA_ERR_TIMEOUT; GBA_DF_SPIN_LIMIT lowers it to test that path
      D.df_spin_limit = 1LL << 22;
      if (const char* sl = std::getenv("GBA_DF_SPIN_LIMIT")) {
        const long long v = std::atoll(sl);
        if (v > 0) D.df_spin_limit = v;
      }
      D.df_own_off = arena.upload(own_off);
      D.df_own = arena.upload(own);
      D.df_flags = arena.alloc<unsigned>(size_t(max_nt) * max_nt);
      D.df_sync = arena.alloc<unsigned>(4);
      GBA_CUDA(cudaMemsetAsync(D.df_flags, 0, sizeof(unsigned) * size_t(max_nt) * max_nt, stream));
      GBA_CUDA(cudaMemsetAsync(D.df_sync, 0, sizeof(unsigned) * 4, stream));
      const char* tp = std::getenv("GBA_FACTOR_TRACE");
      if (tp && *tp) {   // diagnostics: task timeline of the factorization, written at sync
        trace_path = tp;
        D.df_trace = arena.alloc<unsigned long long>(size_t(grid) * kDfTraceCap * 4);
      }
    }
  }
  // batched small systems: one factor-and-solve launch (GBA_CHOL_COLUMNS=1
  // keeps the per-column launches, for comparison)
  D.chol_small = !pcg && D.df_grid == 0 && std::getenv("GBA_CHOL_COLUMNS") == nullptr &&
                 prepare_chol_small(max_nt, opt.precision);
  D.blk_map = dev_blocks && !pcg ? dv_bid : arena.upload(blk_map);
  int dev_pair_bad = 0;
  int* d_pair_bad = nullptr;
  if (dev_blocks) {
    // every point's pairs with their block ids, sorted stably by block on
    // the device: the host's placement, without its scattered writes and the
    // copy of the list
    const long long n = tot.pairs;
    long long hist_ints = 0, scratch_ints = 0;
    pairs_sort_scratch(n, int(P), &hist_ints, &scratch_ints);
    int* k0 = arena.alloc<int>(size_t(n));
    int* k1 = arena.alloc<int>(size_t(n));
    int2* v0 = arena.alloc<int2>(size_t(n));
    int2* v1 = arena.alloc<int2>(size_t(n));
    int* hist = arena.alloc<int>(size_t(hist_ints));
    int* scratch = arena.alloc<int>(size_t(scratch_ints));
    int* pp = arena.alloc<int>(size_t(P) + 1);
    d_pair_bad = arena.alloc<int>(1);
    GBA_CUDA(cudaMemsetAsync(d_pair_bad, 0, sizeof(int), stream));
    int2* sorted = nullptr;
    count_launches(build_pairs_on_device(int(P), dv_blocks, dv_pinfo, dv_pt_key_off, dv_key_img, dv_pt_prob, pp,
                                         dv_bid, n, k0, v0, k1, v1, hist, scratch, d_pair_bad, &sorted, stream));
    GBA_CUDA(cudaGetLastError());
    D.pairs = sorted;
  } else {
    D.pairs = d_pairs ? d_pairs : arena.upload(pairs);
  }
  D.items = arena.upload(items);
  D.blk_ij = arena.upload(blk_ij);
  D.s_elems = pcg ? 0 : s_off;
  D.blk_prob = nullptr;
  if (!pcg && !any_free && !blk_ij.empty()) {   // the dense system assembled block by block
    std::vector<int> blk_prob(blk_ij.size());
    for (int q = 0; q < nprob; ++q)
      for (int t = prob[q].block_begin; t < prob[q].block_begin + prob[q].num_blocks; ++t) blk_prob[t] = q;
    D.blk_prob = arena.upload(blk_prob);
  }
  D.blk_item_off = arena.upload(blk_item_off);
  D.n_items = int(items.size());
  // Z layout: planes in image order when the assembly's key pairs walk
  // each image's keys densely (a block's pairs are a large share of both
  // images' keys: the loads of a warp's 32 pairs then fall in few lines),
  // else records in key order.  Only where the records lie changes.
  {
    double num = 0.0, den = 0.0;
    for (size_t b = 0; b + 1 < blk_item_off.size(); ++b) {
      const int t0 = blk_item_off[b], t1 = blk_item_off[b + 1];
      if (t1 <= t0) continue;
      const int2 ij = blk_ij[b];
      const ProbInfo& pi = prob[items[t0].w];
      if (ij.x == ij.y || ij.x >= pi.num_images || ij.y >= pi.num_images) continue;
      const double nb = double(items[t1 - 1].z - items[t0].y);
      const int gi = pi.image_begin + ij.x, gj = pi.image_begin + ij.y;
      const double ki = std::max(1, img_key_off[gi + 1] - img_key_off[gi]);
      const double kj = std::max(1, img_key_off[gj + 1] - img_key_off[gj]);
      num += nb * nb * 0.5 * (1.0 / ki + 1.0 / kj);
      den += nb;
    }
    z_density = den > 0 ? num / den : 0.0;
    int layout = opt.z_layout;
    if (const char* zl = std::getenv("GBA_Z_LAYOUT")) layout = std::atoi(zl);   // for comparisons
    D.z_planes = layout == GBA_Z_PLANES || (layout != GBA_Z_RECORDS && z_density >= kZPlanesDensity);
    if (D.z_planes) {   // the pairs as slots of the planes
      int* key_slot = arena.alloc<int>(std::max<int64_t>(K, 1));
      count_launches(launch_z_slots(D, key_slot, stream));
    }
  }
  D.n_blocks = int(blk_ij.size());
  D.blk_map_off = arena.upload(blk_map_off);
  D.item_partial = arena.alloc<double>(size_t(kItemStride) * std::max<size_t>(items.size(), 1));
  D.n_key_chunks = int(key_chunks.size());
  D.key_z_split = (key_item + 255) / 256;   // one key per thread of the Z kernel
  D.n_pt_chunks = int(pt_chunks.size());
  D.n_img_chunks = int(img_chunks.size());
  D.key_chunks = arena.upload(key_chunks);
  D.pt_chunks = arena.upload(pt_chunks);
  D.img_chunks = arena.upload(img_chunks);
  D.prob_key_chunk_off = arena.upload(prob_key_chunk_off);
  D.prob_pt_chunk_off = arena.upload(prob_pt_chunk_off);
  D.prob_img_chunk_off = arena.upload(prob_img_chunk_off);
  D.key_chunk_sum = arena.alloc<double>(2 * std::max<size_t>(key_chunks.size(), 1));
  // the LM control folded into k_backsub and the candidate cost: every
  // problem needs a CTA in both (keys, and points or images);
  // GBA_CTRL_KERNELS=1 keeps the separate control launches
  {
    bool fold = std::getenv("GBA_CTRL_KERNELS") == nullptr;
    for (int q = 0; q < nprob && fold; ++q)
      fold = prob_key_chunk_off[q + 1] > prob_key_chunk_off[q] &&
             (prob_pt_chunk_off[q + 1] > prob_pt_chunk_off[q] ||
              prob_img_chunk_off[q + 1] > prob_img_chunk_off[q]);
    D.fold_ctrl = fold ? 1 : 0;
    D.fold_count = arena.alloc<unsigned>(2 * size_t(std::max(nprob, 1)));
    GBA_CUDA(cudaMemsetAsync(D.fold_count, 0, sizeof(unsigned) * 2 * size_t(std::max(nprob, 1)), stream));
  }
  D.n_cons = int(cons.size());
  D.cons = nullptr;
  D.pt_cons_off = nullptr;
  D.img_cons_off = nullptr;
  D.cons_cost = nullptr;
  D.n_priors = int(prior_pt.size());
  D.pt_prior_off = nullptr;
  if (!prior_pt.empty()) {   // priors of each point, in prior order
    std::vector<int> off(P + 1, 0), by_pt(prior_pt.size());
    for (int v : prior_pt) off[v + 1]++;
    for (int64_t i = 0; i < P; ++i) off[i + 1] += off[i];
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (size_t i = 0; i < prior_pt.size(); ++i) by_pt[fill[prior_pt[i]]++] = int(i);
    D.pt_prior_off = arena.upload(off);
    D.prior_by_pt = arena.upload(by_pt);
    D.prior_pt = arena.upload(prior_pt);
    D.prior_y = arena.upload(prior_y);
    D.prior_info = arena.upload(prior_info);
    D.prob_prior_off = arena.upload(prob_prior_off);
  }
  if (!cons.empty() || !prior_pt.empty()) {
    D.prob_cons_off = arena.upload(prob_cons_off);
    D.cons_cost = arena.alloc<double>(nprob);
  }
  if (!cons.empty()) {
    // rows of each point / image in y order, for the linearization
    std::vector<int> pt_off(P + 1, 0), img_off(I + 1, 0);
    for (const int4& c : cons)
      if (c.x < 2) (c.x == 0 ? pt_off[c.y + 1] : img_off[c.y + 1])++;
    for (int64_t i = 0; i < P; ++i) pt_off[i + 1] += pt_off[i];
    for (int64_t i = 0; i < I; ++i) img_off[i + 1] += img_off[i];
    std::vector<int> by_pt(pt_off[P]), by_img(img_off[I]);
    std::vector<int> fp(pt_off.begin(), pt_off.end() - 1), fi(img_off.begin(), img_off.end() - 1);
    for (size_t r = 0; r < cons.size(); ++r) {
      if (cons[r].x == 0) by_pt[fp[cons[r].y]++] = int(r);
      else if (cons[r].x == 1) by_img[fi[cons[r].y]++] = int(r);
    }
    D.cons = arena.upload(cons);
    D.cons_yw = arena.upload(cons_yw);
    D.pt_cons_off = arena.upload(pt_off);
    D.cons_by_pt = arena.upload(by_pt);
    D.img_cons_off = arena.upload(img_off);
    D.cons_by_img = arena.upload(by_img);
  }
  D.pt_chunk_sum = arena.alloc<double>(3 * std::max<size_t>(pt_chunks.size(), 1));
  D.img_chunk_sum = arena.alloc<double>(3 * std::max<size_t>(img_chunks.size(), 1));
  D.launch_counter = nullptr;
  GBA_CUDA(cudaMemsetAsync(D.state, 0, sizeof(LMState) * nprob, stream));
  phase("uploads issued");
  GBA_CUDA(cudaStreamSynchronize(stream));
  if (d_pair_bad) {   // a sorted position outside the list: never expected
    GBA_CUDA(cudaMemcpy(&dev_pair_bad, d_pair_bad, sizeof(int), cudaMemcpyDeviceToHost));
    if (dev_pair_bad) return GBA_ERR;
  }
  phase("uploads done");
  setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (timing) {
    double prev = 0;
    for (const auto& ph : phases) {
      std::fprintf(stderr, "gba build: %-16s %8.2f ms (+%.2f)\n", ph.first, ph.second, ph.second - prev);
      prev = ph.second;
    }
  }
  return GBA_OK;
}

// The launch sequence of one solve.  When profiling, an event is recorded
// after each stage and tagged with it.
void Plan::enqueue(bool profile, Part part) {
  cudaStream_t s = stream;
  long long n = 0;
  const bool prologue = part == kAll || part == kPrologue;
  const int iterations = part == kAll ? opt.max_iterations : (part == kIteration ? 1 : 0);
  size_t ev_i = 0;
  auto mark = [&](int stage) {
    if (!profile) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    GBA_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusActive)   // an event-record node in the graph
      GBA_CUDA(cudaEventRecordWithFlags(prof_events[ev_i], s, cudaEventRecordExternal));
    else
      GBA_CUDA(cudaEventRecord(prof_events[ev_i], s));
    prof_stage[ev_i] = stage;
    ++ev_i;
  };
  if (prologue) {
    mark(-1);
    n += launch_init(d, s);
    mark(GBA_STAGE_CONTROL);
    n += launch_image_prep(d, 0, s);
    mark(GBA_STAGE_IMAGE_PREP);
    n += launch_cost(d, 0, s);
    mark(GBA_STAGE_COST);
    n += launch_ctrl_initial_cost(d, s);
    mark(GBA_STAGE_CONTROL);
    n += launch_linearize(d, s);
    mark(GBA_STAGE_LINEARIZE);
    n += launch_image_reduce(d, s);
    mark(GBA_STAGE_IMAGE_REDUCE);
    n += launch_ctrl_after_linearize(d, s);
    mark(GBA_STAGE_CONTROL);
  }
  for (int it = 0; it < iterations; ++it) {
    // The image sums of the last linearization (nothing to do after the
    // prologue's, or after a rejected step: they check relin) and the
    // after-linearization control.  The point Schur and the key-pair
    // assembly do not read them, so they run beside them on a second
    // stream (the per-stage profile keeps one stream); a problem the control
    // stops only wastes that scratch work, as every later stage checks it.
    const bool side = !profile && side_stream != nullptr;
    if (side) {
      GBA_CUDA(cudaEventRecord(ev_fork, s));
      GBA_CUDA(cudaStreamWaitEvent(side_stream, ev_fork, 0));
      n += launch_image_reduce(d, side_stream);
      n += launch_ctrl_after_linearize(d, side_stream);
      GBA_CUDA(cudaEventRecord(ev_join, side_stream));
    } else {
      n += launch_image_reduce(d, s);
      mark(GBA_STAGE_IMAGE_REDUCE);
      n += launch_ctrl_after_linearize(d, s);
      mark(GBA_STAGE_CONTROL);
    }
    n += launch_point_schur(d, s);
    mark(GBA_STAGE_POINT_SCHUR);
    n += launch_assemble_items(d, s);
    mark(GBA_STAGE_ASSEMBLE);
    if (side) GBA_CUDA(cudaStreamWaitEvent(s, ev_join, 0));
    if (d.pcg) {
      n += launch_assemble_blocks(d, s);
      mark(GBA_STAGE_OTHER);
      n += launch_pcg_setup(d, s);
      mark(GBA_STAGE_FACTOR);
      n += launch_pcg_iterations(d, s);
      mark(GBA_STAGE_SOLVE);
    } else {
      n += launch_assemble_S(d, s);
      mark(GBA_STAGE_OTHER);
      n += launch_cholesky_factor(d, s);
      mark(GBA_STAGE_FACTOR);
      n += launch_cholesky_solve(d, s);
      mark(GBA_STAGE_SOLVE);
    }
    n += launch_backsub(d, s);
    mark(GBA_STAGE_BACKSUB);
    n += launch_ctrl_step(d, s);
    mark(GBA_STAGE_CONTROL);
    n += launch_image_prep(d, 1, s);
    mark(GBA_STAGE_IMAGE_PREP);
    n += launch_cost(d, 1, s);
    mark(GBA_STAGE_COST);
    n += launch_ctrl_accept(d, s);
    mark(GBA_STAGE_CONTROL);
    n += launch_linearize(d, s, !d.fuse_lin);
    mark(GBA_STAGE_LINEARIZE);
  }
  if (part == kAll || part == kEpilogue) {
    if (part == kEpilogue || opt.max_iterations > 0) {
      n += launch_image_reduce(d, s);
      mark(GBA_STAGE_IMAGE_REDUCE);
      n += launch_ctrl_after_linearize(d, s);
      mark(GBA_STAGE_CONTROL);
    }
  }
  GBA_CUDA(cudaGetLastError());
  launches_last_run = n;
}

int Plan::run() {
  const bool profile = opt.profile != 0;
  if (profile) {
    const size_t need = 16 + size_t(opt.max_iterations) * 20;
    while (prof_events.size() < need) {
      cudaEvent_t e;
      GBA_CUDA(cudaEventCreate(&e));
      prof_events.push_back(e);
    }
    if (!graph_exec) prof_stage.assign(prof_events.size(), -2);
  }
  GBA_CUDA(cudaSetDevice(device));
  cudaGetLastError();   // a stale error from other code on this thread is not ours
  GBA_CUDA(cudaEventRecord(ev0, stream));
  if (opt.use_cuda_graph) {
    if (!graph_exec) {
      cudaGraph_t g;
      GBA_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      try {
        enqueue(profile);
      } catch (...) {
        cudaStreamEndCapture(stream, &g);
        throw;
      }
      GBA_CUDA(cudaStreamEndCapture(stream, &g));
      GBA_CUDA(cudaGraphInstantiate(&graph_exec, g, 0));
      cudaGraphDestroy(g);
      graph_launches = launches_last_run;
    }
    GBA_CUDA(cudaGraphLaunch(graph_exec, stream));
    launches_last_run = graph_launches;
  } else if (!profile && opt.max_iterations > 0) {
    // one-shot: the prologue launched directly, then one LM iteration
    // captured once (its launches do not depend on the iteration) and
    // replayed max_iterations times
    enqueue(false, kPrologue);
    const long long pro = launches_last_run;
    if (!iter_exec) {
      cudaGraph_t g;
      GBA_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      try {
        enqueue(false, kIteration);
      } catch (...) {
        cudaStreamEndCapture(stream, &g);
        throw;
      }
      GBA_CUDA(cudaStreamEndCapture(stream, &g));
      GBA_CUDA(cudaGraphInstantiate(&iter_exec, g, 0));
      cudaGraphDestroy(g);
      iter_launches = launches_last_run;
    }
    for (int it = 0; it < opt.max_iterations; ++it) GBA_CUDA(cudaGraphLaunch(iter_exec, stream));
    enqueue(false, kEpilogue);
    launches_last_run += pro + iter_launches * opt.max_iterations;
  } else {
    enqueue(profile);
  }
  if (h_pcg_extra) {
    GBA_CUDA(cudaMemcpyAsync(h_pcg_extra, d.pcg_extra, sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, stream));
    d2h_bytes += sizeof(unsigned long long);
  }
  GBA_CUDA(cudaEventRecord(ev1, stream));
  g_launches += launches_last_run;
  ran = true;
  return GBA_OK;
}

int Plan::sync() {
  GBA_CUDA(cudaStreamSynchronize(stream));
  GBA_CUDA(cudaGetLastError());
  if (h_pcg_extra) {
    // each pass of the device-side PCG loop beyond a loop's first is five
    // launches the launch sequence did not count
    const long long extra = 5LL * (long long)(*h_pcg_extra - pcg_extra_seen);
    pcg_extra_seen = *h_pcg_extra;
    launches_last_run += extra;
    g_launches += extra;
  }
  if (d.df_trace && !trace_path.empty()) write_trace();
  if (opt.profile) {
    std::fill(stage_ms, stage_ms + GBA_NUM_STAGES, 0.0);
    for (size_t i = 1; i < prof_stage.size(); ++i) {
      if (prof_stage[i] < 0) break;
      float ms = 0;
      if (cudaEventElapsedTime(&ms, prof_events[i - 1], prof_events[i]) != cudaSuccess) {
        cudaGetLastError();
        ms = 0;
      }
      stage_ms[prof_stage[i]] += ms;
    }
  }
  return GBA_OK;
}

}  // namespace gba

// ===========================================================================
// C ABI
// ===========================================================================
struct gba_plan {
  gba::Plan impl;
};

namespace {

template <typename F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const gba::CudaError& e) {
    return e.status;
  } catch (const std::bad_alloc&) {
    return GBA_ERR_OOM;
  } catch (...) {
    return GBA_ERR;
  }
}

int check_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return GBA_ERR_NO_DEVICE;
  }
  return GBA_OK;
}

double bits_to_double(unsigned long long b) {
  double v;
  std::memcpy(&v, &b, sizeof(v));
  return v;
}

// A problem's report from its LM state and the plan's timings.
void fill_report(const gba::Plan& P, int q, const gba::LMState& st, gba_report* r) {
  std::memset(r, 0, sizeof(*r));
  r->status = st.status;
  r->stop_reason = st.stop;
  r->iterations = st.iter;
  r->accepted = st.accepted;
  r->rejected = st.rejected;
  r->factor_failures = st.factor_fail;
  r->pcg_iterations = st.pcg_iters;
  r->initial_cost = st.initial_cost;
  r->final_cost = st.F;
  const int K = P.prob[q].num_keys;
  r->final_rmse = K > 0 ? std::sqrt(std::max(st.raw, 0.0) / K) : 0.0;   // plain residuals
  r->final_mu = st.mu;
  r->final_gradient_inf_norm = bits_to_double(st.ginf_bits);
  r->setup_ms = P.setup_ms;
  float ms = 0;
  if (P.ran) cudaEventElapsedTime(&ms, P.ev0, P.ev1);
  r->solve_ms = ms;
  for (int s = 0; s < GBA_NUM_STAGES; ++s) r->stage_ms[s] = P.stage_ms[s];
  r->h2d_bytes = P.h2d_bytes + P.arena.uploaded;
  r->d2h_bytes = P.d2h_bytes;
}

}  // namespace

extern "C" {

int64_t gba_params_per_camera(uint32_t m) { return gba::params_per_camera(m); }

int64_t gba_x_size(const gba_problem* p) {
  if (!p) return -1;
  int64_t n = 0;
  if (!(p->fix_mask & GBA_FIX_POINTS)) n += 3 * p->number_of_points;
  if (!(p->fix_mask & GBA_FIX_IMAGES)) n += 6 * p->number_of_images;
  if (!(p->fix_mask & GBA_FIX_CAMERAS))
    n += gba::params_per_camera(p->intrinsic_computations_mask) * p->number_of_cameras;
  return n;
}

int64_t gba_y_size(const gba_problem* p) {
  if (!p) return -1;
  int64_t n = 2 * p->number_of_keys;
  if (!(p->fix_mask & GBA_FIX_POINTS))
    for (int64_t c = 0; c < p->number_of_point_constraints; ++c) {
      uint32_t m = p->point_constraints[c].mask;
      n += ((m & 1) != 0) + ((m & 2) != 0) + ((m & 4) != 0);
    }
  if (!(p->fix_mask & GBA_FIX_IMAGES))
    for (int64_t c = 0; c < p->number_of_image_constraints; ++c) {
      uint32_t m = p->image_constraints[c].mask;
      n += ((m & 1) ? 3 : 0) + ((m & 2) != 0) + ((m & 4) != 0) + ((m & 8) != 0);
    }
  if (!(p->fix_mask & GBA_FIX_CAMERAS))
    for (int64_t c = 0; c < p->number_of_camera_constraints; ++c) {
      const gba_camera_constraint& cc = p->camera_constraints[c];
      n += __builtin_popcount(cc.radial_mask & 7u) + __builtin_popcount(cc.decentering_mask & 3u) +
           __builtin_popcount(cc.intrinsic_mask & 31u);
    }
  if (p->number_of_point_priors > 0) n += 3 * p->number_of_point_priors;
  return n;
}

void gba_default_options(gba_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->max_iterations = 50;
  o->tau = 1e-3;
  o->eps1 = 1e-8;
  o->eps2 = 1e-8;
  o->precision = GBA_PRECISION_FP64;
  o->loss = GBA_LOSS_TRIVIAL;
  o->huber_delta = 1.0;
  o->linear_solver = GBA_LINEAR_DENSE_CHOLESKY;
  o->pcg_max_iterations = 100;
  o->pcg_relative_tolerance = 1e-6;
  o->use_cuda_graph = 1;
  o->profile = 0;
  o->device = 0;
}

const char* gba_status_string(int s) {
  switch (s) {
    case GBA_OK: return "ok";
    case GBA_ERR: return "failure";
    case GBA_ERR_INVALID: return "invalid argument or size mismatch";
    case GBA_ERR_BAD_INDEX: return "image/point/camera id out of range";
    case GBA_ERR_DUPLICATE: return "duplicate (image, point) key";
    case GBA_ERR_UNSUPPORTED: return "model variant not supported on the device path";
    case GBA_ERR_NOT_SPD: return "reduced system not positive definite";
    case GBA_ERR_NAN: return "non-finite cost";
    case GBA_ERR_OOM: return "device out of memory";
    case GBA_ERR_CUDA: return "CUDA runtime error";
    case GBA_ERR_TIMEOUT: return "bounded device wait ran out";
    case GBA_ERR_NO_DEVICE: return "no CUDA device";
    case GBA_ERR_BUSY: return "admission refused";
    case GBA_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
  }
}

const char* gba_version(void) { return "gba 0.1 (sm_103a)"; }

int64_t gba_kernel_launch_count(void) { return gba::g_launches.load(); }

int gba_plan_create(const gba_problem* problems, const double* const* near_ys, int32_t n,
                    const gba_options* options, gba_plan** out) {
  if (!problems || !options || !out || n <= 0) return GBA_ERR_INVALID;
  *out = nullptr;
  if (int e = check_device()) return e;
  if (options->linear_solver != GBA_LINEAR_DENSE_CHOLESKY && options->linear_solver != GBA_LINEAR_PCG)
    return GBA_ERR_INVALID;
  if (options->linear_solver == GBA_LINEAR_PCG &&
      (options->pcg_max_iterations < 1 || !(options->pcg_relative_tolerance >= 0.0)))
    return GBA_ERR_INVALID;
  if (options->precision != GBA_PRECISION_FP64 && options->precision != GBA_PRECISION_MIXED)
    return GBA_ERR_INVALID;
  if (options->max_iterations < 0 || !(options->function_tolerance >= 0.0)) return GBA_ERR_INVALID;
  if (options->pair_item < 0 || options->image_item < 0 || options->pair_item > (1 << 24) ||
      options->image_item > (1 << 24) || options->key_item < 0 || options->key_item > (1 << 24))
    return GBA_ERR_INVALID;
  if (options->z_layout < GBA_Z_AUTO || options->z_layout > GBA_Z_PLANES) return GBA_ERR_INVALID;
  gba_plan* p = nullptr;
  try {
    p = new gba_plan();
  } catch (...) {
    return GBA_ERR_OOM;
  }
  int err = guarded([&] { return p->impl.build(problems, near_ys, n, options); });
  if (err) {
    delete p;
    return err;
  }
  *out = p;
  return GBA_OK;
}

int gba_plan_destroy(gba_plan* p) {
  delete p;
  return GBA_OK;
}

int gba_plan_number_of_problems(const gba_plan* p) { return p ? p->impl.B : 0; }

int gba_plan_set_initial_x(gba_plan* p, int32_t q, const double* x0) {
  if (!p || !x0 || q < 0 || q >= p->impl.B) return GBA_ERR_INVALID;
  return guarded([&] {
    gba::Plan& P = p->impl;
    const gba::ProbInfo& pi = P.prob[q];
    GBA_CUDA(cudaMemcpyAsync(const_cast<double*>(P.d.x0_pt) + 3LL * pi.point_begin, P.pts_of(q, x0),
                             sizeof(double) * 3 * pi.num_points, cudaMemcpyHostToDevice, P.stream));
    GBA_CUDA(cudaMemcpyAsync(const_cast<double*>(P.d.x0_img) + 6LL * pi.image_begin,
                             P.imgs_of(q, x0), sizeof(double) * 6 * pi.num_images,
                             cudaMemcpyHostToDevice, P.stream));
    std::vector<double> cams;
    if (pi.cps > 0) {   // free cameras: cps parameters each, ten-wide on the device
      const double* xc = x0 + P.x_cam_off(q);
      cams.assign(10 * size_t(pi.num_cams), 0.0);
      for (int c = 0; c < pi.num_cams; ++c)
        std::copy(xc + (size_t)pi.cps * c, xc + (size_t)pi.cps * (c + 1), cams.begin() + 10 * c);
      GBA_CUDA(cudaMemcpyAsync(P.d.x0_cam + 10LL * pi.cam_begin, cams.data(),
                               sizeof(double) * cams.size(), cudaMemcpyHostToDevice, P.stream));
    }
    GBA_CUDA(cudaStreamSynchronize(P.stream));
    P.h2d_bytes += (long long)sizeof(double) *
                   (3LL * pi.num_points + 6LL * pi.num_images + (long long)cams.size());
    return GBA_OK;
  });
}

int gba_plan_run(gba_plan* p) {
  if (!p) return GBA_ERR_INVALID;
  return guarded([&] { return p->impl.run(); });
}

int gba_plan_synchronize(gba_plan* p) {
  if (!p) return GBA_ERR_INVALID;
  return guarded([&] { return p->impl.sync(); });
}

int gba_plan_get_x(gba_plan* p, int32_t q, double* x) {
  if (!p || !x || q < 0 || q >= p->impl.B) return GBA_ERR_INVALID;
  return guarded([&] {
    gba::Plan& P = p->impl;
    gba::LMState st;
    GBA_CUDA(cudaStreamSynchronize(P.stream));
    GBA_CUDA(cudaMemcpy(&st, P.d.state + q, sizeof(st), cudaMemcpyDeviceToHost));
    const gba::ProbInfo& pi = P.prob[q];
    const int par = P.ran ? st.parity : 0;
    const double* xp = P.ran ? P.d.x_pt[par] : P.d.x0_pt;
    const double* xi = P.ran ? P.d.x_img[par] : P.d.x0_img;
    if (!(pi.fix & 1))
      GBA_CUDA(cudaMemcpyAsync(x, xp + 3LL * pi.point_begin, sizeof(double) * 3 * pi.num_points,
                               cudaMemcpyDeviceToHost, P.stream));
    if (!(pi.fix & 2))
      GBA_CUDA(cudaMemcpyAsync(x + P.x_img_off(q), xi + 6LL * pi.image_begin,
                               sizeof(double) * 6 * pi.num_images, cudaMemcpyDeviceToHost, P.stream));
    std::vector<double> cams;
    if (pi.cps > 0) {
      const double* xc = P.ran ? P.d.x_cam[par] : P.d.x0_cam;
      cams.resize(10 * size_t(pi.num_cams));
      GBA_CUDA(cudaMemcpyAsync(cams.data(), xc + 10LL * pi.cam_begin, sizeof(double) * cams.size(),
                               cudaMemcpyDeviceToHost, P.stream));
    }
    GBA_CUDA(cudaStreamSynchronize(P.stream));
    double* xo = x + P.x_cam_off(q);
    for (int c = 0; c < (pi.cps > 0 ? pi.num_cams : 0); ++c)
      std::copy(cams.begin() + 10 * c, cams.begin() + 10 * c + pi.cps, xo + (size_t)pi.cps * c);
    P.d2h_bytes += (long long)sizeof(st) +
                   (long long)sizeof(double) * (3LL * pi.num_points + 6LL * pi.num_images +
                                                (long long)cams.size());
    return GBA_OK;
  });
}

int gba_plan_get_report(gba_plan* p, int32_t q, gba_report* r) {
  if (!p || !r || q < 0 || q >= p->impl.B) return GBA_ERR_INVALID;
  return guarded([&] {
    gba::Plan& P = p->impl;
    gba::LMState st;
    GBA_CUDA(cudaStreamSynchronize(P.stream));
    GBA_CUDA(cudaMemcpy(&st, P.d.state + q, sizeof(st), cudaMemcpyDeviceToHost));
    P.d2h_bytes += (long long)sizeof(st);
    fill_report(P, q, st, r);
    return GBA_OK;
  });
}

}  // extern "C"

namespace {

// Every problem's x and report in one device gather and a few copies (the
// batch path of gba_solve_batch; the per-problem calls would synchronize the
// stream once per problem).
int get_all(gba::Plan& P, double* const* xs, gba_report* reports) {
  return guarded([&] {
    GBA_CUDA(cudaStreamSynchronize(P.stream));
    std::vector<gba::LMState> st(P.B);
    GBA_CUDA(cudaMemcpy(st.data(), P.d.state, sizeof(gba::LMState) * P.B, cudaMemcpyDeviceToHost));
    const long long np = 3LL * P.d.P, ni = 6LL * P.d.I, nc = P.d.free_cams ? 10LL * P.d.Ctot : 0;
    const size_t nx = size_t(np + ni + nc);
    gba::HostBuf<double> stage(nx);
    double* const h = stage.data();
    if (nx) {
      double* dx = P.arena.alloc<double>(nx);
      gba::launch_gather_x(P.d, P.ran ? 1 : 0, dx, P.stream);
      gba::count_launches(1);
      GBA_CUDA(cudaMemcpyAsync(h, dx, sizeof(double) * nx, cudaMemcpyDeviceToHost, P.stream));
      GBA_CUDA(cudaStreamSynchronize(P.stream));
      GBA_CUDA(cudaGetLastError());
    }
    P.d2h_bytes += (long long)(sizeof(gba::LMState) * P.B + sizeof(double) * nx);
    const int nth = std::min(gba::host_threads(), P.B);
    std::atomic<int> next{0};
    gba::host_parallel(nth, nth, [&](int64_t, int64_t, int) {
      for (int q = next++; q < P.B; q = next++) {
        const gba::ProbInfo& pi = P.prob[q];
        double* x = xs[q];
        if (!(pi.fix & 1))
          std::copy(h + 3LL * pi.point_begin, h + 3LL * (pi.point_begin + pi.num_points), x);
        if (!(pi.fix & 2))
          std::copy(h + np + 6LL * pi.image_begin, h + np + 6LL * (pi.image_begin + pi.num_images),
                    x + P.x_img_off(q));
        double* xc = x + P.x_cam_off(q);
        for (int c = 0; c < (pi.cps > 0 ? pi.num_cams : 0); ++c)
          std::copy(h + np + ni + 10LL * (pi.cam_begin + c), h + np + ni + 10LL * (pi.cam_begin + c) + pi.cps,
                    xc + (size_t)pi.cps * c);
        if (reports) fill_report(P, q, st[q], &reports[q]);
      }
    });
    return GBA_OK;
  });
}

// Every problem's x0 scattered on the host and uploaded in a few copies.
int set_all_x0(gba::Plan& P, const double* const* xs) {
  return guarded([&] {
    const long long np = 3LL * P.d.P, ni = 6LL * P.d.I, nc = P.d.free_cams ? 10LL * P.d.Ctot : 0;
    const size_t nx = size_t(np + ni + nc);
    gba::HostBuf<double> stage(nx);
    double* const h = stage.data();
    std::fill(h + np + ni, h + nx, 0.0);   // the camera slots past each camera's parameters
    const int nth = std::min(gba::host_threads(), P.B);
    std::atomic<int> next{0};
    gba::host_parallel(nth, nth, [&](int64_t, int64_t, int) {
      for (int q = next++; q < P.B; q = next++) {
        const gba::ProbInfo& pi = P.prob[q];
        const double* x = xs[q];
        const double* xp = P.pts_of(q, x);
        const double* xi = P.imgs_of(q, x);
        std::copy(xp, xp + 3LL * pi.num_points, h + 3LL * pi.point_begin);
        std::copy(xi, xi + 6LL * pi.num_images, h + np + 6LL * pi.image_begin);
        const double* xc = x + P.x_cam_off(q);
        for (int c = 0; c < (pi.cps > 0 ? pi.num_cams : 0); ++c)
          std::copy(xc + (size_t)pi.cps * c, xc + (size_t)pi.cps * (c + 1), h + np + ni + 10LL * (pi.cam_begin + c));
      }
    });
    if (np)
      GBA_CUDA(cudaMemcpyAsync(const_cast<double*>(P.d.x0_pt), h, sizeof(double) * np, cudaMemcpyHostToDevice,
                               P.stream));
    if (ni)
      GBA_CUDA(cudaMemcpyAsync(const_cast<double*>(P.d.x0_img), h + np, sizeof(double) * ni,
                               cudaMemcpyHostToDevice, P.stream));
    if (nc)
      GBA_CUDA(cudaMemcpyAsync(P.d.x0_cam, h + np + ni, sizeof(double) * nc, cudaMemcpyHostToDevice, P.stream));
    GBA_CUDA(cudaStreamSynchronize(P.stream));
    P.h2d_bytes += (long long)(sizeof(double) * nx);
    return GBA_OK;
  });
}

}  // namespace

extern "C" {

int gba_plan_query(gba_plan* p) {
  if (!p) return GBA_ERR_INVALID;
  if (!p->impl.ran) return GBA_OK;
  cudaError_t e = cudaEventQuery(p->impl.ev1);
  if (e == cudaSuccess) return GBA_OK;
  if (e == cudaErrorNotReady) {
    cudaGetLastError();
    return GBA_ERR_BUSY;
  }
  cudaGetLastError();
  return GBA_ERR_CUDA;
}

int gba_plan_last_run_ms(gba_plan* p, double* ms) {
  if (!p || !ms) return GBA_ERR_INVALID;
  return guarded([&] {
    float f = 0;
    GBA_CUDA(cudaEventElapsedTime(&f, p->impl.ev0, p->impl.ev1));
    *ms = f;
    return GBA_OK;
  });
}

int gba_plan_kernel_stats(gba_plan* p, int32_t stage, double* total_ms, int32_t* launches) {
  if (!p || stage < 0 || stage >= GBA_NUM_STAGES) return GBA_ERR_INVALID;
  if (total_ms) *total_ms = p->impl.stage_ms[stage];
  if (launches) *launches = p->impl.opt.max_iterations;
  return GBA_OK;
}

int gba_plan_last_run_launches(gba_plan* p, int64_t* n) {
  if (!p || !n) return GBA_ERR_INVALID;
  *n = p->impl.launches_last_run;
  return GBA_OK;
}

int gba_plan_device_bytes(gba_plan* p, int64_t* bytes) {
  if (!p || !bytes) return GBA_ERR_INVALID;
  *bytes = int64_t(p->impl.arena.bytes);
  return GBA_OK;
}

int gba_plan_structure(gba_plan* p, gba_plan_structure_info* out) {
  if (!p || !out) return GBA_ERR_INVALID;
  const gba::Plan& P = p->impl;
  std::memset(out, 0, sizeof(*out));
  out->problems = P.B;
  out->keys = P.d.K;
  out->points = P.d.P;
  out->images = P.d.I;
  out->key_pairs = P.n_pairs;
  out->pair_items = P.d.n_items;
  out->blocks = P.d.n_blocks;
  out->image_items = P.d.n_img_items;
  out->camera_records = P.d.R;
  out->max_reduced_size = P.d.max_n;
  out->factor_schedule = P.d.pcg ? -1 : P.d.df_grid > 0 ? 1 : P.d.chol_small ? 2 : 0;
  out->z_layout = P.d.z_planes ? GBA_Z_PLANES : GBA_Z_RECORDS;
  out->forked = P.side_stream != nullptr ? 1 : 0;
  return GBA_OK;
}

int gba_plan_set_initial_x_all(gba_plan* p, const double* const* x0s) {
  if (!p || !x0s) return GBA_ERR_INVALID;
  for (int q = 0; q < p->impl.B; ++q)
    if (!x0s[q] && p->impl.x_size[q] > 0) return GBA_ERR_INVALID;
  return set_all_x0(p->impl, x0s);
}

int gba_plan_get_all(gba_plan* p, double* const* xs, gba_report* reports) {
  if (!p || !xs) return GBA_ERR_INVALID;
  for (int q = 0; q < p->impl.B; ++q)
    if (!xs[q] && p->impl.x_size[q] > 0) return GBA_ERR_INVALID;
  return get_all(p->impl, xs, reports);
}

int gba_batch_create(const gba_problem* problems, const double* const* near_ys, int32_t n,
                     const gba_options* options, gba_batch** batch) {
  return gba_plan_create(problems, near_ys, n, options, batch);
}

int gba_batch_submit(gba_batch* b, const double* const* x0s) {
  int err = gba_plan_set_initial_x_all(b, x0s);
  return err ? err : gba_plan_run(b);
}

int gba_batch_poll(gba_batch* b, double* const* xs, gba_report* reports) {
  if (!b) return GBA_ERR_INVALID;
  const int st = gba_plan_query(b);
  if (st != GBA_OK) return st;
  int err = gba_plan_synchronize(b);   // the run is over: picks up its errors and profile
  return err ? err : gba_plan_get_all(b, xs, reports);
}

int gba_batch_destroy(gba_batch* b) { return gba_plan_destroy(b); }

int gba_solve_batch(const gba_problem* problems, const double* const* near_ys, int32_t n,
                    const gba_options* options, double* const* x_inout, gba_report* reports) {
  return gba_solve_batch_into(problems, near_ys, n, options, x_inout, x_inout, reports);
}

int gba_solve_batch_into(const gba_problem* problems, const double* const* near_ys, int32_t n,
                         const gba_options* options, const double* const* x0, double* const* x_out,
                         gba_report* reports) {
  if (!x0 || !x_out || !options) return GBA_ERR_INVALID;
  // A one-shot solve runs its launch sequence once: capturing all of it into
  // a CUDA graph would cost more than it saves, so the plan captures one LM
  // iteration and replays it.
  gba_options once = *options;
  once.use_cuda_graph = 0;
  // GBA_BUILD_TIMING=1 prints the phases of the call to stderr
  const bool timing = std::getenv("GBA_BUILD_TIMING") != nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  auto phase = [&](const char* name) {
    if (!timing) return;
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    std::fprintf(stderr, "gba solve: %-16s %8.2f ms\n", name, ms);
  };
  gba_plan* plan = nullptr;
  int err = gba_plan_create(problems, near_ys, n, &once, &plan);
  if (err) return err;
  phase("plan built");
  for (int q = 0; q < n && !err; ++q)
    if ((!x0[q] || !x_out[q]) && plan->impl.x_size[q] > 0) err = GBA_ERR_INVALID;
  if (!err) err = set_all_x0(plan->impl, x0);
  phase("x0 uploaded");
  if (!err) err = gba_plan_run(plan);
  phase("launched");
  if (!err) err = gba_plan_synchronize(plan);
  phase("solved");
  if (!err) err = get_all(plan->impl, x_out, reports);
  phase("x read back");
  int first_status = GBA_OK;
  if (!err && reports)
    for (int q = 0; q < n; ++q)
      if (reports[q].status != GBA_OK) { first_status = reports[q].status; break; }
  gba_plan_destroy(plan);
  phase("plan destroyed");
  return err ? err : first_status;
}

int gba_solve(const gba_problem* problem, const double* near_y, const gba_options* options,
              double* x_inout, gba_report* report) {
  const double* ys[1] = {near_y};
  double* xs[1] = {x_inout};
  gba_report local;
  return gba_solve_batch(problem, ys, 1, options, xs, report ? report : &local);
}

int gba_autotune(const gba_problem* problems, const double* const* near_ys, const double* const* x0,
                 int32_t n, const gba_options* options, gba_tuning* out) {
  if (!problems || !near_ys || !x0 || !options || !out || n <= 0) return GBA_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  gba_options base = *options;
  base.max_iterations = std::min(std::max(options->max_iterations, 1), 2);
  base.eps1 = -1.0;
  base.eps2 = -1.0;
  base.function_tolerance = 0.0;
  base.profile = 0;
  base.use_cuda_graph = 1;
  int timed = 0;
  // one candidate: a plan, a warm-up run (graph capture), the best of three
  // timed replays, per LM iteration
  int resolved_layout = 0;   // the layout the last candidate's plan used
  auto time_one = [&](int pair_item, int image_item, int key_item, double* ms_per_it,
                      int z_layout) -> int {
    gba_options o = base;
    o.pair_item = pair_item;
    o.image_item = image_item;
    o.key_item = key_item;
    o.z_layout = z_layout;
    gba_plan* plan = nullptr;
    int err = gba_plan_create(problems, near_ys, n, &o, &plan);
    if (err) return err;
    resolved_layout = plan->impl.d.z_planes ? GBA_Z_PLANES : GBA_Z_RECORDS;
    err = set_all_x0(plan->impl, x0);
    double best = 0.0;
    for (int r = 0; r < 4 && !err; ++r) {
      err = gba_plan_run(plan);
      if (!err) err = gba_plan_synchronize(plan);
      float ms = 0.0f;
      if (!err && r > 0 && cudaEventElapsedTime(&ms, plan->impl.ev0, plan->impl.ev1) == cudaSuccess)
        best = best > 0.0 ? std::min(best, double(ms)) : double(ms);
    }
    gba_plan_destroy(plan);
    if (err) return err;
    ++timed;
    *ms_per_it = best / base.max_iterations;
    return GBA_OK;
  };
  double t_default = 0.0;
  if (int e = time_one(gba::kPairItem, gba::kImageItem, gba::kKeyChunk, &t_default, base.z_layout)) return e;
  int best_pair = gba::kPairItem, best_image = gba::kImageItem, best_key = gba::kKeyChunk;
  int best_layout = resolved_layout;
  double t_best = t_default;
  for (int pi : {256, 512, 2048, 4096}) {
    double t = 0.0;
    if (time_one(pi, gba::kImageItem, gba::kKeyChunk, &t, best_layout) == GBA_OK && t < t_best) {
      t_best = t;
      best_pair = pi;
    }
  }
  for (int ii : {256, 1024}) {
    double t = 0.0;
    if (time_one(best_pair, ii, gba::kKeyChunk, &t, best_layout) == GBA_OK && t < t_best) {
      t_best = t;
      best_image = ii;
    }
  }
  for (int ki : {256, 512, 2048}) {
    double t = 0.0;
    if (time_one(best_pair, best_image, ki, &t, best_layout) == GBA_OK && t < t_best) {
      t_best = t;
      best_key = ki;
    }
  }
  if (base.z_layout == GBA_Z_AUTO) {   // the other layout of the Z records
    const int other = best_layout == GBA_Z_PLANES ? GBA_Z_RECORDS : GBA_Z_PLANES;
    double t = 0.0;
    if (time_one(best_pair, best_image, best_key, &t, other) == GBA_OK && t < t_best) {
      t_best = t;
      best_layout = other;
    }
  }
  out->z_layout = best_layout;
  out->pair_item = best_pair;
  out->image_item = best_image;
  out->key_item = best_key;
  out->ms_per_iteration = t_best;
  out->default_ms_per_iteration = t_default;
  out->candidates = timed;
  return GBA_OK;
}

// ---- single-stage entry points ---------------------------------------------
namespace {

// A plan for one problem at x, brought to the point where the image
// rotations of x exist on the device.
int stage_plan(const gba_problem* problem, const double* near_y, const double* x,
               int precision, gba_plan** out, gba_options* opt_out) {
  gba_options o;
  gba_default_options(&o);
  o.precision = precision;
  o.max_iterations = 1;
  o.eps1 = -1.0;
  o.eps2 = -1.0;
  o.use_cuda_graph = 0;
  std::vector<double> zeros;
  if (!near_y) {
    zeros.assign(std::max<int64_t>(gba_y_size(problem), 0), 0.0);
    near_y = zeros.data();
  }
  int err = gba_plan_create(problem, &near_y, 1, &o, out);
  if (err) return err;
  err = gba_plan_set_initial_x(*out, 0, x);
  if (err) {
    gba_plan_destroy(*out);
    return err;
  }
  if (opt_out) *opt_out = o;
  return GBA_OK;
}

}  // namespace

int gba_vector_function(const gba_problem* problem, const double* x, double* y, int32_t precision) {
  if (!problem || !x || !y) return GBA_ERR_INVALID;
  gba_plan* plan = nullptr;
  int err = stage_plan(problem, nullptr, x, precision, &plan, nullptr);
  if (err) return err;
  err = guarded([&] {
    gba::Plan& P = plan->impl;
    cudaStream_t s = P.stream;
    gba::launch_init(P.d, s);
    gba::launch_image_prep(P.d, 0, s);
    double* dy = P.arena.alloc<double>(2 * std::max(P.d.K, 1));
    gba::launch_vector_function(P.d, dy, s);
    gba::g_launches += 4;
    GBA_CUDA(cudaStreamSynchronize(s));
    GBA_CUDA(cudaGetLastError());
    std::vector<double> ys(2 * P.d.K);
    GBA_CUDA(cudaMemcpy(ys.data(), dy, sizeof(double) * ys.size(), cudaMemcpyDeviceToHost));
    const auto& perm = P.key_sorted_to_orig[0];
    for (int t = 0; t < P.d.K; ++t) {
      y[2 * perm[t]] = ys[2 * t];
      y[2 * perm[t] + 1] = ys[2 * t + 1];
    }
    // constraint rows copy their parameter (x = [points 3P][images 6I]
    // [cameras], fixed groups dropped; a fixed group has no rows)
    int64_t r = 2 * problem->number_of_keys;
    const bool fixP = problem->fix_mask & GBA_FIX_POINTS, fixI = problem->fix_mask & GBA_FIX_IMAGES;
    const int64_t img0 = P.x_img_off(0);
    for (int64_t c = 0; c < (fixP ? 0 : problem->number_of_point_constraints); ++c) {
      const gba_point_constraint& pc = problem->point_constraints[c];
      for (int b = 0; b < 3; ++b)
        if (pc.mask & (1u << b)) y[r++] = x[3 * pc.point_id + b];
    }
    for (int64_t c = 0; c < (fixI ? 0 : problem->number_of_image_constraints); ++c) {
      const gba_image_constraint& ic = problem->image_constraints[c];
      const double* xi = x + img0 + 6 * ic.image_id;
      if (ic.mask & GBA_IMAGE_CONSTRAIN_ROTATION)
        for (int b = 0; b < 3; ++b) y[r++] = xi[b];
      if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_X) y[r++] = xi[3];
      if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_Y) y[r++] = xi[4];
      if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_Z) y[r++] = xi[5];
    }
    if (!(problem->fix_mask & GBA_FIX_CAMERAS)) {
      const uint32_t m = problem->intrinsic_computations_mask;
      const int64_t cps = gba::params_per_camera(m);
      const double* xc = x + P.x_cam_off(0);
      for (int64_t c = 0; c < problem->number_of_camera_constraints; ++c) {
        const gba_camera_constraint& cc = problem->camera_constraints[c];
        const double* xv = xc + cps * cc.camera_id;
        int off = 0;
        for (int b = 0; b < 3; ++b)
          if (cc.radial_mask & (1u << b)) y[r++] = xv[off + b];
        if (m & GBA_COMPUTE_RADIAL_DISTORTION) off += 3;
        for (int b = 0; b < 2; ++b)
          if (cc.decentering_mask & (1u << b)) y[r++] = xv[off + b];
        if (m & GBA_COMPUTE_DECENTERING_DISTORTION) off += 2;
        for (int b = 0; b < 5; ++b)
          if (cc.intrinsic_mask & (1u << b)) y[r++] = xv[off + b];
      }
    }
    for (int64_t i = 0; i < problem->number_of_point_priors; ++i)   // point priors
      for (int a = 0; a < 3; ++a) y[r++] = x[3 * problem->point_prior_ids[i] + a];
    return GBA_OK;
  });
  gba_plan_destroy(plan);
  return err;
}

int gba_jacobian(const gba_problem* problem, const double* x, double* point_blocks,
                 double* image_blocks, double* camera_blocks, int32_t precision) {
  if (!problem || !x) return GBA_ERR_INVALID;
  gba_plan* plan = nullptr;
  int err = stage_plan(problem, nullptr, x, precision, &plan, nullptr);
  if (err) return err;
  err = guarded([&] {
    gba::Plan& P = plan->impl;
    cudaStream_t s = P.stream;
    gba::launch_init(P.d, s);
    gba::launch_image_prep(P.d, 0, s);
    const int K = std::max(P.d.K, 1);
    double* jp = P.arena.alloc<double>(6 * K);
    double* ji = P.arena.alloc<double>(12 * K);
    const int cps = P.prob[0].cps;   // > 0 only with free cameras
    double* jc = (camera_blocks && cps > 0) ? P.arena.alloc<double>(20 * K) : nullptr;
    gba::launch_jacobian_out(P.d, jp, ji, jc, s);
    gba::g_launches += 4;
    GBA_CUDA(cudaStreamSynchronize(s));
    GBA_CUDA(cudaGetLastError());
    std::vector<double> hp(6 * P.d.K), hi(12 * P.d.K), hc(jc ? 20 * P.d.K : 0);
    GBA_CUDA(cudaMemcpy(hp.data(), jp, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost));
    GBA_CUDA(cudaMemcpy(hi.data(), ji, sizeof(double) * hi.size(), cudaMemcpyDeviceToHost));
    if (jc) GBA_CUDA(cudaMemcpy(hc.data(), jc, sizeof(double) * hc.size(), cudaMemcpyDeviceToHost));
    const auto& perm = P.key_sorted_to_orig[0];
    const uint32_t mask = problem->intrinsic_computations_mask;
    for (int t = 0; t < P.d.K; ++t) {
      if (point_blocks) std::copy(&hp[6 * t], &hp[6 * t] + 6, point_blocks + 6LL * perm[t]);
      if (image_blocks) std::copy(&hi[12 * t], &hi[12 * t] + 12, image_blocks + 12LL * perm[t]);
      if (jc)   // 2 x cps, row-major, the computed columns
        for (int r = 0; r < 2; ++r)
          for (int m = 0; m < cps; ++m)
            camera_blocks[2LL * cps * perm[t] + cps * r + m] =
                hc[20 * t + 10 * r + gba::camera_full_column(mask, m)];
    }
    return GBA_OK;
  });
  gba_plan_destroy(plan);
  return err;
}

int gba_cost(const gba_problem* problem, const double* x, const double* near_y,
             const gba_options* options, double* cost) {
  if (!problem || !x || !near_y || !cost) return GBA_ERR_INVALID;
  gba_options o;
  gba_default_options(&o);
  if (options) o = *options;
  gba_plan* plan = nullptr;
  int err = stage_plan(problem, near_y, x, o.precision, &plan, nullptr);
  if (err) return err;
  err = guarded([&] {
    gba::Plan& P = plan->impl;
    P.d.loss = o.loss;
    P.d.huber_delta = o.huber_delta;
    cudaStream_t s = P.stream;
    gba::launch_init(P.d, s);
    gba::launch_image_prep(P.d, 0, s);
    gba::launch_cost(P.d, 0, s);
    gba::launch_ctrl_initial_cost(P.d, s);
    gba::g_launches += 5;
    GBA_CUDA(cudaStreamSynchronize(s));
    GBA_CUDA(cudaGetLastError());
    gba::LMState st;
    GBA_CUDA(cudaMemcpy(&st, P.d.state, sizeof(st), cudaMemcpyDeviceToHost));
    *cost = st.F;
    return std::isfinite(st.F) ? GBA_OK : GBA_ERR_NAN;
  });
  gba_plan_destroy(plan);
  return err;
}

int gba_schur_step(const gba_problem* problem, const double* x, const double* near_y, double mu,
                   const gba_options* options, double* delta_x) {
  if (!problem || !x || !near_y || !delta_x) return GBA_ERR_INVALID;
  gba_options o;
  gba_default_options(&o);
  if (options) o = *options;
  gba_plan* plan = nullptr;
  int err = stage_plan(problem, near_y, x, o.precision, &plan, nullptr);
  if (err) return err;
  err = guarded([&] {
    gba::Plan& P = plan->impl;
    P.d.loss = o.loss;
    P.d.huber_delta = o.huber_delta;
    cudaStream_t s = P.stream;
    gba::launch_init(P.d, s);
    gba::launch_image_prep(P.d, 0, s);
    gba::launch_cost(P.d, 0, s);
    gba::launch_ctrl_initial_cost(P.d, s);
    gba::launch_linearize(P.d, s);
    gba::launch_image_reduce(P.d, s);
    gba::launch_ctrl_after_linearize(P.d, s);
    GBA_CUDA(cudaStreamSynchronize(s));
    // override mu
    GBA_CUDA(cudaMemcpy(reinterpret_cast<char*>(P.d.state) + offsetof(gba::LMState, mu), &mu,
                        sizeof(double), cudaMemcpyHostToDevice));
    gba::launch_point_schur(P.d, s);
    long long nl = 0;
    if (P.d.pcg) {
      nl += gba::launch_assemble_items(P.d, s);
      nl += gba::launch_assemble_blocks(P.d, s);
      nl += gba::launch_pcg_setup(P.d, s);
      nl += gba::launch_pcg_iterations(P.d, s);
    } else {
      nl += gba::launch_assemble(P.d, s);
      nl += gba::launch_cholesky(P.d, s);
    }
    gba::launch_backsub(P.d, s);
    gba::g_launches += 9 + nl;
    GBA_CUDA(cudaStreamSynchronize(s));
    GBA_CUDA(cudaGetLastError());
    int flag = 0;
    GBA_CUDA(cudaMemcpy(&flag, P.d.factor_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return GBA_ERR_NOT_SPD;
    const gba::ProbInfo& pi = P.prob[0];
    std::vector<double> x0p(3 * pi.num_points), x1p(3 * pi.num_points), di(6 * pi.num_images);
    GBA_CUDA(cudaMemcpy(x0p.data(), P.d.x_pt[0], sizeof(double) * x0p.size(), cudaMemcpyDeviceToHost));
    GBA_CUDA(cudaMemcpy(x1p.data(), P.d.x_pt[1], sizeof(double) * x1p.size(), cudaMemcpyDeviceToHost));
    if (P.d.precision == GBA_PRECISION_MIXED) {
      std::vector<float> df(di.size());
      GBA_CUDA(cudaMemcpy(df.data(), P.d.b, sizeof(float) * df.size(), cudaMemcpyDeviceToHost));
      std::copy(df.begin(), df.end(), di.begin());
    } else {
      GBA_CUDA(cudaMemcpy(di.data(), P.d.b, sizeof(double) * di.size(), cudaMemcpyDeviceToHost));
    }
    // the free groups only, in the caller's x layout
    if (!(pi.fix & 1))
      for (size_t i = 0; i < x0p.size(); ++i) delta_x[i] = x0p[i] - x1p[i];
    if (!(pi.fix & 2)) std::copy(di.begin(), di.end(), delta_x + P.x_img_off(0));
    if (pi.cps > 0) {   // free cameras: x_c - (x_c - delta_c)
      std::vector<double> c0(10 * size_t(pi.num_cams)), c1(c0.size());
      GBA_CUDA(cudaMemcpy(c0.data(), P.d.x_cam[0], sizeof(double) * c0.size(), cudaMemcpyDeviceToHost));
      GBA_CUDA(cudaMemcpy(c1.data(), P.d.x_cam[1], sizeof(double) * c1.size(), cudaMemcpyDeviceToHost));
      double* dc = delta_x + P.x_cam_off(0);
      for (int c = 0; c < pi.num_cams; ++c)
        for (int m = 0; m < pi.cps; ++m) dc[(size_t)pi.cps * c + m] = c0[10 * c + m] - c1[10 * c + m];
    }
    return GBA_OK;
  });
  gba_plan_destroy(plan);
  return err;
}

}  // extern "C"
