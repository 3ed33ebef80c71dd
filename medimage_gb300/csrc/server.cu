// server.cu -- continuous-batching reconstruction server.
//
// Requests (a plan, a sinogram, an outer-iteration count, an arrival time)
// are admitted into a running batch as soon as they have arrived and their
// device state fits the HBM admission budget and a slot is free.  Every round
// advances all admitted requests by one outer iteration (image step + edge
// step of origin/GoldenC/src/main.c:43-47) with one launch per kernel for the
// whole mix, so the work of different requests overlaps on the device.  A
// request leaves the batch after its last iteration: f and v are copied out,
// its state is freed and its slot goes to the next request.  Sinogram, f, v
// and the CG state stay in HBM from admission to completion.
//
// Each request's arithmetic depends only on its own data and geometry (the
// projector variant is fixed for the server's lifetime), so its result is the
// same alone and in any mix.  Fan-beam and ray-table slices share one batch,
// cone-beam volumes another; a round advances both.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <thread>
#include <vector>

#include "solver.h"

namespace at {

cudaError_t launch_fill(float *p, float v, size_t n, cudaStream_t st);

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
};

struct Server {
  at_server_config cfg{};
  at_params prm{};
  int rpt = 1;
  cudaStream_t st = nullptr;
  std::map<int64_t, std::unique_ptr<Request>> reqs;
  std::vector<Request *> pending;  // arrival order
  std::vector<Request *> active;
  Batch batch[2];  // 0: fan beam and ray tables, 1: cone beam
  bool has[2] = {false, false};
  bool dirty = true;
  int64_t next_id = 1;
  size_t used = 0, peak = 0;
  int64_t rounds = 0, completed = 0;
  double t0 = -1.0, busy = 0.0, t_first = -1.0, t_last = 0.0;
  int64_t slices = 0;

  ~Server() {
    for (auto &kv : reqs)
      if (kv.second->mem) cudaFree(kv.second->mem);
    if (st) cudaStreamDestroy(st);
  }

  int admit(Request *r, double t) {
    r->bytes = scan_bytes(*r->plan, rpt);
    cudaError_t e = cudaMallocAsync(&r->mem, r->bytes, st);
    if (e != cudaSuccess) return cuda_error(e, "server: state allocation");
    carve_scan(r->dev, *r->plan, rpt, (char *)r->mem);
    r->ctl = make_ctl(prm);
    AT_CUDA_TRY(cudaMemcpyAsync(r->dev.ctl, &r->ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
    AT_CUDA_TRY(cudaMemcpyAsync(r->dev.buf[B_G], r->sino.data(), sizeof(float) * r->sino.size(),
                                cudaMemcpyHostToDevice, st));
    AT_CUDA_TRY(cudaMemsetAsync(r->dev.buf[B_F], 0, sizeof(float) * r->dev.npix, st));  // main.c:36
    AT_CUDA_TRY(launch_fill(r->dev.buf[B_V], 1.f, r->dev.npix, st));                   // main.c:37-40
    if (const size_t bpb = bp_scratch_bytes(*r->plan)) AT_CUDA_TRY(cudaMemsetAsync(r->dev.bp_acc, 0, bpb, st));
    used += r->bytes;
    peak = std::max(peak, used);
    r->state = 1;
    r->t_admit = t;
    active.push_back(r);
    dirty = true;
    return AT_OK;
  }

  int retire(Request *r, double t) {
    r->f.resize(r->dev.npix);
    r->v.resize(r->dev.npix);
    AT_CUDA_TRY(cudaMemcpyAsync(r->f.data(), r->dev.buf[B_F], sizeof(float) * r->dev.npix, cudaMemcpyDeviceToHost, st));
    AT_CUDA_TRY(cudaMemcpyAsync(r->v.data(), r->dev.buf[B_V], sizeof(float) * r->dev.npix, cudaMemcpyDeviceToHost, st));
    AT_CUDA_TRY(cudaFreeAsync(r->mem, st));
    AT_CUDA_TRY(cudaStreamSynchronize(st));
    r->mem = nullptr;
    used -= r->bytes;
    r->state = 2;
    r->t_done = t;
    r->sino.clear();
    r->sino.shrink_to_fit();
    completed++;
    slices++;
    t_last = std::max(t_last, t);
    dirty = true;
    return AT_OK;
  }

  int run(double max_seconds) {
    if (t0 < 0) t0 = now_s();
    const double start = now_s();
    int rc;
    while (!pending.empty() || !active.empty()) {
      const double t = now_s() - t0;
      if (now_s() - start > max_seconds) break;
      // admission: arrived requests in order, while slots and budget allow
      while (!pending.empty() && pending.front()->arrival <= t && (int)active.size() < cfg.max_active) {
        Request *r = pending.front();
        if (used + scan_bytes(*r->plan, rpt) > cfg.hbm_budget_bytes) {
          if (active.empty()) return set_error(AT_EBUDGET, "server: request does not fit the HBM budget");
          break;
        }
        if ((rc = admit(r, t))) return rc;
        if (t_first < 0) t_first = r->arrival;
        pending.erase(pending.begin());
      }
      if (active.empty()) {  // idle until the next arrival
        const double wait = pending.front()->arrival - (now_s() - t0);
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
        continue;
      }
      if (dirty) {
        std::vector<ScanDev> scans[2];
        for (auto *r : active) scans[r->plan->kind == AT_GEOM_CONE ? 1 : 0].push_back(r->dev);
        for (int k = 0; k < 2; k++) {
          has[k] = !scans[k].empty();
          if (has[k] && (rc = batch[k].set(scans[k].data(), (int)scans[k].size(), k ? AT_GEOM_CONE : AT_GEOM_FAN,
                                           rpt, st)))
            return rc;
        }
        dirty = false;
      }
      const double r0 = now_s();
      for (int k = 0; k < 2; k++)
        if (has[k] && (rc = batch[k].enqueue_outer(st))) return rc;
      AT_CUDA_TRY(cudaStreamSynchronize(st));
      const double r1 = now_s();
      busy += r1 - r0;
      rounds++;
      std::vector<Request *> still;
      for (auto *r : active) {
        if (++r->iters_done >= r->iter_alt) {
          if ((rc = retire(r, r1 - t0))) return rc;
        } else {
          still.push_back(r);
        }
      }
      active.swap(still);
    }
    return AT_OK;
  }
};

}  // namespace at

struct at_server {
  at::Server s;
};

using namespace at;

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
  for (auto &b : S->s.batch) b.params = S->s.prm;
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

AT_API int at_server_run(at_server *srv, double max_seconds) {
  if (!srv) return set_error(AT_EINVAL, "at_server_run: null argument");
  return srv->s.run(max_seconds > 0 ? max_seconds : 1e30);
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
  return AT_OK;
}
