// server.cu -- continuous-batching reconstruction server.
//
// Requests (a plan, a sinogram, an outer-iteration count, an arrival time)
// are admitted into a running batch as soon as they have arrived and their
// device state fits the HBM admission budget and a slot is free.  The requests
// of one geometry form a batch on its own stream; a round advances all of them
// by one outer iteration (image step + edge step of
// origin/GoldenC/src/main.c:43-47) with one launch per kernel, and the rounds
// of different geometries run concurrently, so the work of different requests
// overlaps on the device.  A
// request leaves the batch after its last iteration: f and v are copied out,
// its state is freed and its slot goes to the next request.  Sinogram, f, v
// and the CG state stay in HBM from admission to completion.
//
// Each request's arithmetic depends only on its own data and geometry (the
// projector variant is fixed for the server's lifetime), so its result is the
// same alone and in any mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <thread>
#include <vector>

#include "solver.h"

namespace medimg {

cudaError_t launch_fill(float *p, float v, size_t n, cudaStream_t st);
size_t psnr_scratch_bytes();
int psnr_with_scratch(const float *d_x, const float *d_ref, int64_t n, double peak, void *scratch, double *h_psnr,
                      cudaStream_t st);

namespace {
double now_s() {
  using namespace std::chrono;
  return duration_cast<duration<double>>(steady_clock::now().time_since_epoch()).count();
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}
}  // namespace

struct Request {
  int64_t id = 0;
  Plan *plan = nullptr;
  std::vector<float> sino;
  int iter_alt = 0;
  double arrival = 0.0;  // seconds after the server clock starts
  int state = 0;         // 0 pending, 1 active, 2 done
  ScanDev dev{};
  void *mem = nullptr;
  size_t bytes = 0;
  int iters_done = 0;
  double t_admit = 0.0, t_done = 0.0;
  Ctl ctl{};
  std::vector<float> f, v;
  // quality stop: the request finishes as soon as PSNR(f, ref) >= target
  // (measured on the GPU after every outer iteration), or after iter_alt
  std::vector<float> ref;
  float *d_ref = nullptr;  // in the request's state allocation
  double target_psnr = 0.0, peak = 0.0, psnr = NAN;
  bool psnr_stop = false;
};

// The requests of one geometry: one batch, advanced one outer iteration per
// round on its own stream, so requests of a slow geometry (a cone volume, a
// 1024^2 slice) do not hold back those of a fast one; the GPU runs the groups'
// rounds concurrently.
struct Group {
  Plan *plan = nullptr;
  Batch batch;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  void *psnr_scratch = nullptr;  // partial sums of the quality checks
  std::vector<Request *> active;
  std::vector<Request *> round;  // the requests the round in flight advances
  bool dirty = true, in_flight = false;
  double r0 = 0.0;
  ~Group() {
    if (psnr_scratch) cudaFree(psnr_scratch);
    if (ev) cudaEventDestroy(ev);
    if (st) cudaStreamDestroy(st);
  }
};

struct Server {
  at_server_config cfg{};
  at_params prm{};
  int rpt = 1;
  cudaStream_t st = nullptr;  // the caller-side stream (creation only)
  std::map<int64_t, std::unique_ptr<Request>> reqs;
  std::vector<Request *> pending;  // arrival order
  std::map<const Plan *, std::unique_ptr<Group>> groups;
  int nactive = 0;
  int64_t next_id = 1;
  size_t used = 0, peak = 0;
  int64_t rounds = 0, completed = 0, psnr_stops = 0;
  double t0 = -1.0, busy = 0.0, t_first = -1.0, t_last = 0.0;
  int64_t slices = 0;

  ~Server() {
    for (auto &kv : groups) cudaStreamSynchronize(kv.second->st);
    for (auto &kv : reqs)
      if (kv.second->mem) cudaFree(kv.second->mem);
    groups.clear();
    if (st) cudaStreamDestroy(st);
  }

  int group_of(Plan *plan, Group **out) {
    auto &g = groups[plan];
    if (!g) {
      g = std::make_unique<Group>();
      g->plan = plan;
      g->batch.params = prm;
      AT_CUDA_TRY(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking));
      AT_CUDA_TRY(cudaEventCreateWithFlags(&g->ev, cudaEventDisableTiming));
      AT_CUDA_TRY(cudaMalloc(&g->psnr_scratch, psnr_scratch_bytes()));
    }
    *out = g.get();
    return AT_OK;
  }

  // device bytes of a request: its solver state, and its reference image
  // when it has a quality stop
  size_t request_bytes(const Request &r) const {
    return scan_bytes(*r.plan, rpt) + ((sizeof(float) * r.ref.size() + 255) & ~(size_t)255);
  }

  int admit(Request *r, double t) {
    Group *g = nullptr;
    int rc = group_of(r->plan, &g);
    if (rc) return rc;
    cudaStream_t gs = g->st;
    r->bytes = request_bytes(*r);
    cudaError_t e = cudaMallocAsync(&r->mem, r->bytes, gs);
    if (e != cudaSuccess) return cuda_error(e, "server: state allocation");
    carve_scan(r->dev, *r->plan, rpt, (char *)r->mem);
    if (!r->ref.empty()) {
      r->d_ref = reinterpret_cast<float *>((char *)r->mem + scan_bytes(*r->plan, rpt));
      AT_CUDA_TRY(cudaMemcpyAsync(r->d_ref, r->ref.data(), sizeof(float) * r->ref.size(), cudaMemcpyHostToDevice, gs));
    }
    r->ctl = make_ctl(prm);
    AT_CUDA_TRY(cudaMemcpyAsync(r->dev.ctl, &r->ctl, sizeof(Ctl), cudaMemcpyHostToDevice, gs));
    AT_CUDA_TRY(cudaMemcpyAsync(r->dev.buf[B_G], r->sino.data(), sizeof(float) * r->sino.size(),
                                cudaMemcpyHostToDevice, gs));
    AT_CUDA_TRY(cudaMemsetAsync(r->dev.buf[B_F], 0, sizeof(float) * r->dev.npix, gs));  // main.c:36
    AT_CUDA_TRY(launch_fill(r->dev.buf[B_V], 1.f, r->dev.npix, gs));                   // main.c:37-40
    if (const size_t bpb = bp_scratch_bytes(*r->plan)) AT_CUDA_TRY(cudaMemsetAsync(r->dev.bp_acc, 0, bpb, gs));
    used += r->bytes;
    peak = std::max(peak, used);
    r->state = 1;
    r->t_admit = t;
    g->active.push_back(r);
    g->dirty = true;
    nactive++;
    return AT_OK;
  }

  int retire(Group *g, Request *r, double t) {
    r->f.resize(r->dev.npix);
    r->v.resize(r->dev.npix);
    AT_CUDA_TRY(cudaMemcpyAsync(r->f.data(), r->dev.buf[B_F], sizeof(float) * r->dev.npix, cudaMemcpyDeviceToHost,
                                g->st));
    AT_CUDA_TRY(cudaMemcpyAsync(r->v.data(), r->dev.buf[B_V], sizeof(float) * r->dev.npix, cudaMemcpyDeviceToHost,
                                g->st));
    AT_CUDA_TRY(cudaFreeAsync(r->mem, g->st));
    AT_CUDA_TRY(cudaStreamSynchronize(g->st));
    r->mem = nullptr;
    used -= r->bytes;
    r->state = 2;
    r->t_done = t;
    r->d_ref = nullptr;
    r->sino.clear();
    r->sino.shrink_to_fit();
    r->ref.clear();
    r->ref.shrink_to_fit();
    completed++;
    slices++;
    nactive--;
    t_last = std::max(t_last, t);
    g->dirty = true;
    return AT_OK;
  }

  int run(double max_seconds) {
    if (t0 < 0) t0 = now_s();
    const double start = now_s();
    int rc;
    while (!pending.empty() || nactive > 0) {
      const double t = now_s() - t0;
      if (now_s() - start > max_seconds) break;
      // admission: arrived requests in order, while slots and budget allow
      while (!pending.empty() && pending.front()->arrival <= t && nactive < cfg.max_active) {
        Request *r = pending.front();
        if (used + request_bytes(*r) > cfg.hbm_budget_bytes) {
          if (nactive == 0) return set_error(AT_EBUDGET, "server: request does not fit the HBM budget");
          break;
        }
        if ((rc = admit(r, t))) return rc;
        if (t_first < 0) t_first = r->arrival;
        pending.erase(pending.begin());
      }
      if (nactive == 0) {  // idle until the next arrival
        const double wait = pending.front()->arrival - (now_s() - t0);
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
        continue;
      }
      // start a round in every idle group that has requests
      for (auto &kv : groups) {
        Group *g = kv.second.get();
        if (g->in_flight || g->active.empty()) continue;
        if (g->dirty) {
          std::vector<ScanDev> scans;
          for (auto *r : g->active) scans.push_back(r->dev);
          if ((rc = g->batch.set(scans.data(), (int)scans.size(), g->plan->kind == AT_GEOM_CONE ? AT_GEOM_CONE
                                                                                                 : AT_GEOM_FAN,
                                 rpt, g->st)))
            return rc;
          g->dirty = false;
        }
        g->r0 = now_s();
        g->round = g->active;  // requests admitted during the round join the next one
        if ((rc = g->batch.enqueue_outer(g->st))) return rc;
        AT_CUDA_TRY(cudaEventRecord(g->ev, g->st));
        g->in_flight = true;
      }
      // finish the rounds that are done
      bool progressed = false;
      for (auto &kv : groups) {
        Group *g = kv.second.get();
        if (!g->in_flight) continue;
        const cudaError_t q = cudaEventQuery(g->ev);
        if (q == cudaErrorNotReady) continue;
        AT_CUDA_TRY(q);
        const double r1 = now_s();
        busy += r1 - g->r0;
        rounds++;
        g->in_flight = false;
        progressed = true;
        for (auto *r : g->round) {
          ++r->iters_done;
          bool done = r->iters_done >= r->iter_alt;
          if (r->target_psnr > 0) {  // the quality stop, on the GPU
            if ((rc = psnr_with_scratch(r->dev.buf[B_F], r->d_ref, r->dev.npix, r->peak, g->psnr_scratch, &r->psnr,
                                        g->st)))
              return rc;
            if (r->psnr >= r->target_psnr) {
              r->psnr_stop = !done;
              psnr_stops += r->psnr_stop ? 1 : 0;
              done = true;
            }
          }
          if (done) {
            if ((rc = retire(g, r, now_s() - t0))) return rc;
            g->active.erase(std::find(g->active.begin(), g->active.end(), r));
          }
        }
        g->round.clear();
      }
      if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return AT_OK;
  }
};

}  // namespace medimg

struct at_server {
  medimg::Server s;
};

using namespace medimg;

#define AT_API extern "C" __attribute__((visibility("default")))

AT_API int at_server_create(const at_server_config *cfg, at_server **out) {
  if (!cfg || !out) return set_error(AT_EINVAL, "at_server_create: null argument");
  *out = nullptr;
  if (cfg->max_active < 1) return set_error(AT_EINVAL, "at_server_create: max_active must be >= 1");
  if (cfg->iter_image < 2 || cfg->iter_edge < 1) return set_error(AT_EINVAL, "at_server_create: bad iteration counts");
  if (cfg->mode != 0 && cfg->mode != 1) return set_error(AT_EINVAL, "at_server_create: mode must be 0 or 1");
  auto S = std::make_unique<at_server>();
  S->s.cfg = *cfg;
  S->s.prm = at_params{cfg->alpha, cfg->beta, cfg->epsilon, 0, cfg->iter_image, cfg->iter_edge, cfg->mode};
  S->s.rpt = cfg->fp_rays_per_thread > 0 ? cfg->fp_rays_per_thread : 1;
  if (S->s.rpt != 1 && S->s.rpt != 2 && S->s.rpt != 4)
    return set_error(AT_EINVAL, "at_server_create: fp_rays_per_thread must be 1, 2 or 4");
  cudaError_t e = cudaStreamCreateWithFlags(&S->s.st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_error(e, "at_server_create: stream");
  *out = S.release();
  return AT_OK;
}

AT_API void at_server_destroy(at_server *s) { delete s; }

AT_API int at_server_submit(at_server *srv, at_plan *plan, const float *h_sino, int32_t iter_alt, double arrival_s,
                            int64_t *id) {
  if (!srv || !plan || !h_sino || !id) return set_error(AT_EINVAL, "at_server_submit: null argument");
  if (plan->p.kind == AT_GEOM_GOLDNC)
    return set_error(AT_EINVAL, "at_server_submit: fan-beam, ray-table and cone-beam plans only");
  if (iter_alt < 1) return set_error(AT_EINVAL, "at_server_submit: iter_alt must be >= 1");
  Server &S = srv->s;
  if (scan_bytes(plan->p, S.rpt) > S.cfg.hbm_budget_bytes)
    return set_error(AT_EBUDGET, "at_server_submit: the request alone exceeds the HBM admission budget");
  auto r = std::make_unique<Request>();
  r->id = S.next_id++;
  r->plan = &plan->p;
  r->sino.assign(h_sino, h_sino + (size_t)plan->p.nviews * plan->p.ndets);
  r->iter_alt = iter_alt;
  r->arrival = arrival_s;
  Request *raw = r.get();
  auto it = std::upper_bound(S.pending.begin(), S.pending.end(), raw,
                             [](const Request *a, const Request *b) { return a->arrival < b->arrival; });
  S.pending.insert(it, raw);
  *id = raw->id;
  S.reqs[raw->id] = std::move(r);
  return AT_OK;
}

AT_API int at_server_submit_psnr(at_server *srv, at_plan *plan, const float *h_sino, int32_t iter_alt,
                                 double arrival_s, const float *h_ref, double target_psnr_db, double peak,
                                 int64_t *id) {
  if (!srv || !h_ref || !(target_psnr_db > 0))
    return set_error(AT_EINVAL, "at_server_submit_psnr: a reference image and a positive target are required");
  if (!plan || !id) return set_error(AT_EINVAL, "at_server_submit_psnr: null argument");
  Server &S = srv->s;
  const size_t npix = (size_t)plan->p.nz * plan->p.n * plan->p.n;
  if (scan_bytes(plan->p, S.rpt) + sizeof(float) * npix + 256 > S.cfg.hbm_budget_bytes)
    return set_error(AT_EBUDGET, "at_server_submit_psnr: the request alone exceeds the HBM admission budget");
  const int rc = at_server_submit(srv, plan, h_sino, iter_alt, arrival_s, id);
  if (rc) return rc;
  Request &r = *S.reqs[*id];
  r.ref.assign(h_ref, h_ref + npix);
  r.target_psnr = target_psnr_db;
  r.peak = peak;
  return AT_OK;
}

AT_API int at_server_result_info(const at_server *srv, int64_t id, int32_t *iterations, double *psnr_db,
                                 int32_t *stopped_by_psnr) {
  if (!srv) return set_error(AT_EINVAL, "at_server_result_info: null argument");
  auto it = srv->s.reqs.find(id);
  if (it == srv->s.reqs.end()) return set_error(AT_EINVAL, "at_server_result_info: unknown request");
  const Request &r = *it->second;
  if (r.state != 2) return set_error(AT_ESTATE, "at_server_result_info: request not finished");
  if (iterations) *iterations = r.iters_done;
  if (psnr_db) *psnr_db = r.psnr;
  if (stopped_by_psnr) *stopped_by_psnr = r.psnr_stop ? 1 : 0;
  return AT_OK;
}

AT_API int at_server_run(at_server *srv, double max_seconds) {
  if (!srv) return set_error(AT_EINVAL, "at_server_run: null argument");
  const int rc = srv->s.run(max_seconds > 0 ? max_seconds : 1e30);
  return rc ? rc : check_wait_timeouts();
}

AT_API int at_server_result(at_server *srv, int64_t id, float *h_f, float *h_v, double *latency_s, double *wait_s) {
  if (!srv) return set_error(AT_EINVAL, "at_server_result: null argument");
  auto it = srv->s.reqs.find(id);
  if (it == srv->s.reqs.end()) return set_error(AT_EINVAL, "at_server_result: unknown request");
  Request &r = *it->second;
  if (r.state != 2) return set_error(AT_ESTATE, "at_server_result: request not finished");
  if (h_f) std::memcpy(h_f, r.f.data(), sizeof(float) * r.f.size());
  if (h_v) std::memcpy(h_v, r.v.data(), sizeof(float) * r.v.size());
  if (latency_s) *latency_s = r.t_done - r.arrival;
  if (wait_s) *wait_s = r.t_admit - r.arrival;
  return AT_OK;
}

AT_API int at_server_get_stats(const at_server *srv, at_server_stats *out) {
  if (!srv || !out) return set_error(AT_EINVAL, "at_server_get_stats: null argument");
  const Server &S = srv->s;
  std::vector<double> lat;
  for (auto &kv : S.reqs)
    if (kv.second->state == 2) lat.push_back(kv.second->t_done - kv.second->arrival);
  std::memset(out, 0, sizeof(*out));
  out->submitted = (int64_t)S.reqs.size();
  out->completed = S.completed;
  out->rounds = S.rounds;
  out->p50_latency_s = percentile(lat, 0.50);
  out->p99_latency_s = percentile(lat, 0.99);
  out->max_latency_s = lat.empty() ? 0.0 : *std::max_element(lat.begin(), lat.end());
  const double span = S.t_last - (S.t_first < 0 ? 0.0 : S.t_first);
  out->slices_per_s = span > 0 ? S.completed / span : 0.0;
  out->busy_s = S.busy;
  out->peak_state_bytes = S.peak;
  out->psnr_stops = S.psnr_stops;
  return AT_OK;
}
