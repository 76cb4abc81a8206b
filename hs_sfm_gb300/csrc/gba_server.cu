// gba_server.cu -- continuous-batching request loop over resident plans.
//
// One worker thread runs the loop:
//   1. harvest: every in-flight micro-batch whose plan has finished on the
//      device (event query, no blocking) hands its results to the requests and
//      returns its memory to the budget;
//   2. admit: while in-flight slots remain, the queued requests that fit the
//      remaining device-memory budget (FIFO, up to max_batch) are packed into
//      one plan on a fresh stream and launched -- new work starts while earlier
//      micro-batches are still running;
//   3. otherwise sleep until a submission arrives or a short poll interval ends.
// Plans allocate stream-ordered, so admitting and retiring never synchronize
// the device.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gba.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

int64_t ppc(uint32_t m) { return gba_params_per_camera(m); }

// Deep copy of a request's inputs; prob points into the vectors below.
struct Request {
  int64_t ticket = 0;
  gba_problem prob{};
  std::vector<int64_t> fm, icm;
  std::vector<double> fix_points, fix_images, fix_cameras, kci, cw, y, x0;
  std::vector<gba_point_constraint> pc;
  std::vector<gba_image_constraint> ic;
  std::vector<gba_camera_constraint> cc;
  int64_t bytes = 0, x_size = 0;
  enum State { QUEUED, RUNNING, DONE, CANCELLED } state = QUEUED;
  bool cancel_requested = false;
  int status = GBA_OK;
  std::vector<double> x;
  gba_report report{};
  Clock::time_point t_submit, t_admit, t_done;

  void copy_from(const gba_problem& p, const double* near_y, const double* x_init) {
    prob = p;
    fm.assign(p.feature_maps, p.feature_maps + 2 * p.number_of_keys);
    icm.assign(p.image_camera_map, p.image_camera_map + p.number_of_images);
    prob.feature_maps = fm.data();
    prob.image_camera_map = icm.data();
    const int64_t cps = ppc(p.intrinsic_computations_mask);
    if (p.fix_points) fix_points.assign(p.fix_points, p.fix_points + 3 * p.number_of_points);
    if (p.fix_images) fix_images.assign(p.fix_images, p.fix_images + 6 * p.number_of_images);
    if (p.fix_cameras) fix_cameras.assign(p.fix_cameras, p.fix_cameras + cps * p.number_of_cameras);
    prob.fix_points = p.fix_points ? fix_points.data() : nullptr;
    prob.fix_images = p.fix_images ? fix_images.data() : nullptr;
    prob.fix_cameras = p.fix_cameras ? fix_cameras.data() : nullptr;
    if (p.number_of_point_constraints > 0 && p.point_constraints)
      pc.assign(p.point_constraints, p.point_constraints + p.number_of_point_constraints);
    if (p.number_of_image_constraints > 0 && p.image_constraints)
      ic.assign(p.image_constraints, p.image_constraints + p.number_of_image_constraints);
    if (p.number_of_camera_constraints > 0 && p.camera_constraints)
      cc.assign(p.camera_constraints, p.camera_constraints + p.number_of_camera_constraints);
    prob.point_constraints = pc.empty() ? nullptr : pc.data();
    prob.image_constraints = ic.empty() ? nullptr : ic.data();
    prob.camera_constraints = cc.empty() ? nullptr : cc.data();
    if (p.key_covariance_inverse)
      kci.assign(p.key_covariance_inverse, p.key_covariance_inverse + 4 * p.number_of_keys);
    prob.key_covariance_inverse = kci.empty() ? nullptr : kci.data();
    const int64_t ys = gba_y_size(&p);
    if (p.constraint_weights && ys > 2 * p.number_of_keys)
      cw.assign(p.constraint_weights, p.constraint_weights + (ys - 2 * p.number_of_keys));
    prob.constraint_weights = cw.empty() ? nullptr : cw.data();
    y.assign(near_y, near_y + ys);
    x_size = gba_x_size(&p);
    x0.assign(x_init, x_init + x_size);
  }
};

struct Batch {
  gba_plan* plan = nullptr;
  std::vector<Request*> reqs;
  int64_t bytes = 0;
};

}  // namespace

struct gba_server {
  gba_server_config cfg{};
  int64_t budget = 0;
  std::mutex m;
  std::condition_variable wake;   // worker
  std::condition_variable done;   // waiters
  std::deque<Request*> queue;
  std::vector<Batch> in_flight;
  std::map<int64_t, std::unique_ptr<Request>> requests;
  int64_t next_ticket = 1;
  int64_t admitted = 0;
  gba_server_stats stats{};
  bool stop = false;
  std::thread worker;

  void harvest_locked(Batch& b) {
    int qst = gba_plan_synchronize(b.plan);
    // every request's x and report in one gather
    std::vector<double*> xs(b.reqs.size());
    std::vector<gba_report> reps(b.reqs.size());
    for (size_t q = 0; q < b.reqs.size(); ++q) {
      b.reqs[q]->x.assign(size_t(b.reqs[q]->x_size), 0.0);
      xs[q] = b.reqs[q]->x.data();
    }
    if (qst == GBA_OK) qst = gba_plan_get_all(b.plan, xs.data(), reps.data());
    for (size_t q = 0; q < b.reqs.size(); ++q) {
      Request* r = b.reqs[q];
      r->t_done = Clock::now();
      if (r->cancel_requested) {
        r->state = Request::CANCELLED;
        r->status = GBA_ERR_CANCELLED;
        continue;
      }
      int st = qst;
      if (st == GBA_OK) {
        r->report = reps[q];
        st = r->report.status;
      }
      r->report.queue_ms = ms_between(r->t_submit, r->t_admit);
      r->report.latency_ms = ms_between(r->t_submit, r->t_done);
      r->status = st;
      r->state = Request::DONE;
      stats.completed++;
    }
    gba_plan_destroy(b.plan);
    admitted -= b.bytes;
    stats.in_flight_requests -= int64_t(b.reqs.size());
  }

  void loop() {
    std::unique_lock<std::mutex> lk(m);
    while (!stop) {
      bool progressed = false;
      for (size_t i = 0; i < in_flight.size();) {
        if (gba_plan_query(in_flight[i].plan) != GBA_ERR_BUSY) {
          harvest_locked(in_flight[i]);
          in_flight.erase(in_flight.begin() + long(i));
          progressed = true;
        } else {
          ++i;
        }
      }
      if (progressed) done.notify_all();
      if (int(in_flight.size()) < cfg.max_in_flight && !queue.empty()) {
        Batch b;
        while (!queue.empty() && int(b.reqs.size()) < cfg.max_batch) {
          Request* r = queue.front();
          if (r->cancel_requested) {
            queue.pop_front();
            r->state = Request::CANCELLED;
            r->status = GBA_ERR_CANCELLED;
            done.notify_all();
            continue;
          }
          if (admitted + b.bytes + r->bytes > budget) break;   // FIFO: wait for memory
          queue.pop_front();
          r->state = Request::RUNNING;
          r->t_admit = Clock::now();
          b.reqs.push_back(r);
          b.bytes += r->bytes;
        }
        if (!b.reqs.empty()) {
          admitted += b.bytes;
          stats.in_flight_requests += int64_t(b.reqs.size());
          lk.unlock();
          std::vector<gba_problem> probs;
          std::vector<const double*> ys;
          for (Request* r : b.reqs) {
            probs.push_back(r->prob);
            ys.push_back(r->y.data());
          }
          gba_options o = cfg.solve;
          o.use_cuda_graph = 0;   // a micro-batch plan runs once
          o.shared_device = 1;    // several micro-batches run at the same time
          int st = gba_plan_create(probs.data(), ys.data(), int32_t(probs.size()), &o, &b.plan);
          if (st == GBA_OK) {
            std::vector<const double*> x0s;
            for (Request* r : b.reqs) x0s.push_back(r->x0.data());
            st = gba_plan_set_initial_x_all(b.plan, x0s.data());
          }
          if (st == GBA_OK) st = gba_plan_run(b.plan);
          lk.lock();
          if (st != GBA_OK) {
            for (Request* r : b.reqs) {
              r->state = Request::DONE;
              r->status = st;
              r->t_done = Clock::now();
              r->report.latency_ms = ms_between(r->t_submit, r->t_done);
            }
            if (b.plan) gba_plan_destroy(b.plan);
            admitted -= b.bytes;
            stats.in_flight_requests -= int64_t(b.reqs.size());
            done.notify_all();
          } else {
            in_flight.push_back(b);
            stats.batches_launched++;
          }
          continue;
        }
      }
      wake.wait_for(lk, in_flight.empty() ? std::chrono::milliseconds(20)
                                          : std::chrono::milliseconds(0) + std::chrono::microseconds(100));
    }
  }

  int result_locked(int64_t ticket, double* x_out, gba_report* report, bool* ready) {
    auto it = requests.find(ticket);
    if (it == requests.end()) return GBA_ERR_INVALID;
    Request* r = it->second.get();
    if (r->state == Request::QUEUED || r->state == Request::RUNNING) {
      *ready = false;
      return GBA_ERR_BUSY;
    }
    *ready = true;
    int st = r->status;
    if (r->state == Request::CANCELLED) st = GBA_ERR_CANCELLED;
    if (x_out && r->state == Request::DONE && !r->x.empty())
      std::memcpy(x_out, r->x.data(), sizeof(double) * r->x.size());
    if (report) *report = r->report;
    requests.erase(it);
    return st;
  }
};

extern "C" {

int64_t gba_estimate_device_bytes(const gba_problem* p, int32_t precision) {
  if (!p) return -1;
  const int64_t tsz = precision == GBA_PRECISION_MIXED ? 4 : 8;
  const int64_t K = p->number_of_keys, P = p->number_of_points, I = p->number_of_images;
  const int64_t C = p->number_of_cameras;
  // free cameras: nc six-wide parts per camera in the reduced system and up
  // to nc camera records per (point, camera seen)
  const int64_t cps = ppc(p->intrinsic_computations_mask);
  const bool free_cams = !(p->fix_mask & GBA_FIX_CAMERAS) && cps > 0 && C > 0;
  const int64_t nc = free_cams ? (cps + 5) / 6 : 0;
  int64_t pairs = 0, recs = 0;
  if (K > 0 && p->feature_maps) {
    std::vector<int32_t> cnt(size_t(std::max<int64_t>(P, 1)), 0);
    for (int64_t k = 0; k < K; ++k) {
      const int64_t pt = p->feature_maps[2 * k + 1];
      if (pt >= 0 && pt < P) cnt[size_t(pt)]++;
    }
    for (int32_t c : cnt) {
      const int64_t r = free_cams ? std::min<int64_t>(c, C) * nc : 0;   // records, at most
      pairs += (c + r) * (c + r + 1) / 2;
      recs += r;
    }
  }
  const int64_t Ie = I + C * nc;
  const int64_t n = 6 * Ie, nt = (n + 31) / 32;
  const int64_t blocks = Ie * (Ie + 1) / 2;
  const int64_t items = pairs / 1024 + blocks + 1;
  int64_t b = 0;
  b += K * (4 + 4 + 16 + 4 + 8 * tsz + 40 * tsz + 20 * tsz);   // indices, obs, RW, JR (x2), Z
  if (p->key_covariance_inverse) b += K * 24;
  if (precision == GBA_PRECISION_MIXED) b += K * 16 + P * 48 + I * 192;   // double-float mirrors
  b += P * (4 + 4 + 48 + 24 + 24 * tsz + 24);                 // offsets, x, x0, PV, PS, sums
  b += I * (4 * 4 + 48 + 96 + 48 + 192 + 24 * tsz + 288 + 48 + 6 * tsz + 28 * 8);
  b += (K / 512 + 1) * (16 + 28 * 8);                         // image reduce items
  b += C * (80 + 40 + 80);
  b += n * n * tsz + nt * 1024 * tsz;                          // reduced system, tile inverses
  b += pairs * 8 + items * (16 + 352) + blocks * 12 + Ie * Ie * 4;
  if (free_cams) {
    b += recs * (20 * tsz + 12) + P * 4;                        // camera Z records, offsets
    b += K * 40 * tsz + (K / 512 + 1) * 128 * 8 + I * (60 * 8 + 128 * 8 + 4);   // J_c (x2), sums, E, ext
    b += C * (3 * 80 + 100 * 8 + 10 * 8 + 3 * 8 + 2 * (80 + 40 + 80) + 16 + 8) + I * 4;
  }
  const int64_t rows = gba_y_size(p) - 2 * K;                   // constraint and prior rows
  if (rows > 0) b += rows * 32 + (P + I + 2) * 8 + p->number_of_point_priors * 96;
  return b + (1 << 20);                                        // bookkeeping slack
}

void gba_default_server_config(gba_server_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  gba_default_options(&c->solve);
  c->solve.precision = GBA_PRECISION_MIXED;
  c->memory_budget_bytes = 0;
  c->max_batch = 64;
  c->max_in_flight = 4;
}

int gba_server_create(const gba_server_config* config, gba_server** out) {
  if (!config || !out) return GBA_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return GBA_ERR_NO_DEVICE;
  }
  if (config->max_batch < 1 || config->max_in_flight < 1) return GBA_ERR_INVALID;
  gba_server* s = new (std::nothrow) gba_server();
  if (!s) return GBA_ERR_OOM;
  s->cfg = *config;
  s->budget = config->memory_budget_bytes;
  if (s->budget <= 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaSetDevice(config->solve.device) != cudaSuccess ||
        cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      delete s;
      return GBA_ERR_CUDA;
    }
    s->budget = int64_t(double(free_b) * 0.8);
  }
  s->stats.budget_bytes = s->budget;
  s->worker = std::thread([s] {
    cudaSetDevice(s->cfg.solve.device);
    s->loop();
  });
  *out = s;
  return GBA_OK;
}

int gba_server_destroy(gba_server* s) {
  if (!s) return GBA_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
  }
  s->wake.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (Batch& b : s->in_flight) {
    gba_plan_synchronize(b.plan);
    gba_plan_destroy(b.plan);
  }
  delete s;
  return GBA_OK;
}

int gba_server_submit(gba_server* s, const gba_problem* problem, const double* near_y,
                      const double* x0, int64_t* ticket) {
  if (!s || !problem || !near_y || !x0 || !ticket) return GBA_ERR_INVALID;
  std::unique_ptr<Request> r(new (std::nothrow) Request());
  if (!r) return GBA_ERR_OOM;
  r->copy_from(*problem, near_y, x0);
  r->bytes = gba_estimate_device_bytes(&r->prob, s->cfg.solve.precision);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->m);
  if (r->bytes > s->budget) {
    s->stats.refused++;
    return GBA_ERR_BUSY;
  }
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  s->queue.push_back(r.get());
  s->requests[r->ticket] = std::move(r);
  s->stats.submitted++;
  s->wake.notify_all();
  return GBA_OK;
}

int gba_server_poll(gba_server* s, int64_t ticket, double* x_out, gba_report* report) {
  if (!s) return GBA_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->m);
  bool ready = false;
  return s->result_locked(ticket, x_out, report, &ready);
}

int gba_server_wait(gba_server* s, int64_t ticket, double timeout_ms, double* x_out,
                    gba_report* report) {
  if (!s) return GBA_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->m);
  const Clock::time_point until =
      Clock::now() + std::chrono::microseconds(int64_t(std::max(0.0, timeout_ms) * 1000.0));
  for (;;) {
    bool ready = false;
    const int st = s->result_locked(ticket, x_out, report, &ready);
    if (ready || st == GBA_ERR_INVALID) return st;
    if (timeout_ms < 0) {
      s->done.wait_for(lk, std::chrono::milliseconds(50));
    } else {
      if (Clock::now() >= until) return GBA_ERR_BUSY;
      s->done.wait_until(lk, until);
    }
  }
}

int gba_server_cancel(gba_server* s, int64_t ticket) {
  if (!s) return GBA_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->requests.find(ticket);
  if (it == s->requests.end()) return GBA_ERR_INVALID;
  Request* r = it->second.get();
  if (r->state == Request::DONE) return GBA_OK;
  r->cancel_requested = true;
  s->stats.cancelled++;
  s->wake.notify_all();
  return GBA_OK;
}

int gba_server_get_stats(gba_server* s, gba_server_stats* out) {
  if (!s || !out) return GBA_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->m);
  *out = s->stats;
  out->queued = int64_t(s->queue.size());
  out->in_flight_batches = int64_t(s->in_flight.size());
  out->admitted_bytes = s->admitted;
  return GBA_OK;
}

}  // extern "C"
