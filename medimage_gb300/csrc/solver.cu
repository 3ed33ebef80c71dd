// solver.cpp -- host orchestration of the batched AT solver.
//
// A solver owns, for each scan of its batch, the state buffers of
// origin/GoldenC/src/main.c (f, v, d, p, update, r, q, ...) in one device
// allocation, a control block with the CG scalars, and a trace buffer.  The
// launch sequence of one outer iteration (image step then edge step,
// main.c:43-47) is recorded once into a CUDA graph and replayed; early exits
// are decided on the device, so later launches of a finished step return at
// their first instruction.
#include <algorithm>
#include <cstring>
#include <vector>

#include "solver.h"

namespace at {

int fp_ctas(const ScanDev &S, int rpt);
int bp_ctas(const ScanDev &S);
int pix_ctas(const ScanDev &S);
cudaError_t launch_fp(const Launch &L, int kind, int rpt, int nctas, cudaStream_t st);
cudaError_t launch_bp(const Launch &L, int kind, int nctas, cudaStream_t st);
cudaError_t launch_pixel(int which, const Launch &L, int nctas, cudaStream_t st);
cudaError_t launch_flags(const ScanDev *scans, int nscans, int mode, cudaStream_t st);

void fill_scan_plan(ScanDev &S, const Plan &p) {
  std::memset(&S, 0, sizeof(S));
  S.kind = p.kind;
  S.n = p.n;
  S.nviews = p.nviews;
  S.ndets = p.ndets;
  S.npix = p.n * p.n;
  S.nbins = p.nviews * p.ndets;
  S.nbpv = p.nblocks_per_view;
  S.offgrid = p.offgrid ? 1 : 0;
  S.rays = p.rays_d;
  S.bits = p.bits_d;
  S.blk_word = p.blk_word_d;
  S.blk_nw = p.blk_nw_d;
  S.run = p.run_d;
  S.tile_off = p.tile_off_d;
  S.ntiles_y = p.ntiles_y;
  S.nvb = p.nvb;
  S.bp_term_bits = p.bp_term_bits;
  S.pixel_mm = (float)p.geom.pixel_mm;
  S.gc_seg = p.gc_seg_d;
  S.gc_pair_off = p.gc_pair_off_d;
  S.gc_ent = p.gc_ent_d;
  S.gc_pix_off = p.gc_pix_off_d;
}

namespace {
enum PixKernel { PK_UPD = 0, PK_PP, PK_COMMIT, PK_EDGE_INIT, PK_EDGE_D, PK_EDGE_UPD, PK_SINO, PK_INIT };

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

struct ScanLayout {
  size_t img_bytes, sino_bytes, partial_bytes, trace_bytes, total;
};

ScanLayout layout_of(const Plan &p, int rpt) {
  ScanLayout L;
  const size_t npix = (size_t)p.n * p.n, nbins = (size_t)p.nviews * p.ndets;
  L.img_bytes = align_up(npix * sizeof(float));
  L.sino_bytes = align_up(nbins * sizeof(float));
  ScanDev tmp{};
  tmp.kind = p.kind;
  tmp.n = p.n;
  tmp.nviews = p.nviews;
  tmp.nbpv = p.nblocks_per_view;
  tmp.ntiles_y = p.ntiles_y;
  const int maxcta = std::max({fp_ctas(tmp, rpt), bp_ctas(tmp), pix_ctas(tmp), (int)((nbins + 255) / 256)});
  L.partial_bytes = align_up((size_t)maxcta * 4 * sizeof(double));
  L.trace_bytes = align_up((size_t)kTraceCap * 10 * sizeof(double));
  L.total = L.img_bytes * B_NIMG + L.sino_bytes * (B_NBUF - B_NIMG) + L.partial_bytes + L.trace_bytes +
            align_up(sizeof(Ctl));
  return L;
}
}  // namespace

int Solver::choose_rpt(const std::vector<Plan *> &plans) {
  // rays per thread of the forward projector: the autotuned choice of the
  // batch's first plan (projections are bitwise identical for every choice)
  return plans.empty() ? 1 : plans[0]->fp_rpt;
}

size_t Solver::footprint(const std::vector<Plan *> &plans, int rpt) {
  size_t tot = 0;
  for (auto *p : plans) tot += layout_of(*p, rpt).total;
  return tot + 4096 * 4;
}

int Solver::create(const std::vector<Plan *> &pl, const at_params &prm) {
  if (pl.empty()) return set_error(AT_EINVAL, "solver: no scans");
  const int kind = pl[0]->kind;
  for (auto *p : pl)
    if (p->kind != kind) return set_error(AT_EINVAL, "solver: a batch must hold one geometry kind");
  if (prm.iter_image < 2) return set_error(AT_EINVAL, "solver: iter_image must be >= 2 (the reference divides by iter_image/2)");
  if (prm.iter_edge < 1 || prm.iter_alt < 0) return set_error(AT_EINVAL, "solver: iteration counts must be positive");
  if (prm.mode != 0 && prm.mode != 1) return set_error(AT_EINVAL, "solver: mode must be 0 (exact) or 1 (linear)");
  plans = pl;
  params = prm;
  nscans = (int)pl.size();
  rpt = choose_rpt(pl);
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));

  std::vector<ScanLayout> lay(nscans);
  size_t total = 0;
  for (int s = 0; s < nscans; s++) {
    lay[s] = layout_of(*pl[s], rpt);
    total += lay[s].total;
  }
  if (cudaMalloc(&arena, total) != cudaSuccess) {
    cudaGetLastError();
    return set_error(AT_ENOMEM, "solver: device allocation of " + std::to_string(total) + " bytes failed");
  }
  arena_bytes = total;
  AT_CUDA_TRY(cudaMemset(arena, 0, total));
  host_scans.resize(nscans);
  char *cur = (char *)arena;
  std::vector<int> fp_pref(nscans + 1, 0), pix_pref(nscans + 1, 0), sino_pref(nscans + 1, 0),
      bp_pref(nscans + 1, 0);
  for (int s = 0; s < nscans; s++) {
    const Plan &p = *pl[s];
    ScanDev &S = host_scans[s];
    fill_scan_plan(S, p);
    for (int b = 0; b < B_NIMG; b++) {
      S.buf[b] = (float *)cur;
      cur += lay[s].img_bytes;
    }
    for (int b = B_NIMG; b < B_NBUF; b++) {
      S.buf[b] = (float *)cur;
      cur += lay[s].sino_bytes;
    }
    S.partials = (double *)cur;
    cur += lay[s].partial_bytes;
    S.trace = (double *)cur;
    cur += lay[s].trace_bytes;
    S.ctl = (Ctl *)cur;
    cur += align_up(sizeof(Ctl));
    fp_pref[s + 1] = fp_pref[s] + fp_ctas(S, rpt);
    pix_pref[s + 1] = pix_pref[s] + pix_ctas(S);
    bp_pref[s + 1] = bp_pref[s] + bp_ctas(S);
    sino_pref[s + 1] = sino_pref[s] + (S.nbins + 255) / 256;
  }
  fp_total = fp_pref[nscans];
  pix_total = pix_pref[nscans];
  bp_total = bp_pref[nscans];
  sino_total = sino_pref[nscans];
  AT_CUDA_TRY(cudaMalloc(&scans_d, sizeof(ScanDev) * nscans));
  AT_CUDA_TRY(cudaMemcpy(scans_d, host_scans.data(), sizeof(ScanDev) * nscans, cudaMemcpyHostToDevice));
  AT_CUDA_TRY(cudaMalloc(&prefix_d, sizeof(int) * 4 * (nscans + 1)));
  AT_CUDA_TRY(cudaMemcpy(prefix_d, fp_pref.data(), sizeof(int) * (nscans + 1), cudaMemcpyHostToDevice));
  AT_CUDA_TRY(cudaMemcpy(prefix_d + (nscans + 1), pix_pref.data(), sizeof(int) * (nscans + 1), cudaMemcpyHostToDevice));
  AT_CUDA_TRY(cudaMemcpy(prefix_d + 3 * (nscans + 1), bp_pref.data(), sizeof(int) * (nscans + 1),
                         cudaMemcpyHostToDevice));
  AT_CUDA_TRY(cudaMemcpy(prefix_d + 2 * (nscans + 1), sino_pref.data(), sizeof(int) * (nscans + 1),
                         cudaMemcpyHostToDevice));
  return AT_OK;
}

Solver::~Solver() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  cudaFree(arena);
  cudaFree(scans_d);
  cudaFree(prefix_d);
  if (own_stream) cudaStreamDestroy(own_stream);
}

Launch Solver::base_launch(int family) const {
  Launch L;
  std::memset(&L, 0, sizeof(L));
  L.scans = scans_d;
  L.nscans = nscans;
  L.prefix = prefix_d + family * (nscans + 1);
  L.aux_buf = -1;
  return L;
}

int Solver::reset(cudaStream_t st) {
  int rc;
  if ((rc = reset_ctl(st))) return rc;
  Launch L = base_launch(1);
  L.flow = FLOW_ENABLED;
  AT_CUDA_TRY(launch_pixel(PK_INIT, L, pix_total, st));
  return AT_OK;
}

int Solver::reset_ctl(cudaStream_t st) {
  std::vector<Ctl> ctl(nscans);
  for (int s = 0; s < nscans; s++) {
    Ctl &c = ctl[s];
    std::memset(&c, 0, sizeof(c));
    c.enabled = 1;
    c.iter_image = params.iter_image;
    c.iter_edge = params.iter_edge;
    c.median_every = params.iter_image / 2;
    c.mode = params.mode;
    c.alpha = params.alpha;
    c.beta = params.beta;
    c.eps = params.epsilon;
  }
  // the control blocks are written from a host copy kept alive by the solver
  ctl_host = ctl;
  for (int s = 0; s < nscans; s++)
    AT_CUDA_TRY(cudaMemcpyAsync(host_scans[s].ctl, &ctl_host[s], sizeof(Ctl), cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));  // ctl_host may be rewritten by the next reset
  return AT_OK;
}

int Solver::enable(int scan, bool on, cudaStream_t st) {
  const int v = on ? 1 : 0;
  AT_CUDA_TRY(cudaMemcpyAsync(&host_scans[scan].ctl->enabled, &v, sizeof(int), cudaMemcpyHostToDevice, st));
  return AT_OK;
}

// The launch sequence of one outer iteration (main.c:45-46).
int Solver::enqueue_outer(cudaStream_t st) {
  launches = 0;
  int rc;
  if ((rc = enqueue_image(st))) return rc;
  return enqueue_edge(st);
}

// minimize_in_IMAGE_variable, main.c:81-257
int Solver::enqueue_image(cudaStream_t st) {
  const int K = params.iter_image;
  const bool linear = params.mode == 1;
  const int kind = plans[0]->kind;
  const int m = K / 2;  // median every (int)(IterImage/2) iterations, main.c:180
  auto fp = [&](int stage, int in, int aux, int k) -> int {
    Launch L = base_launch(0);
    L.flow = FLOW_IMAGE;
    L.stage = stage;
    L.in_buf = in;
    L.aux_buf = aux;
    L.k = k;
    AT_CUDA_TRY(launch_fp(L, kind, rpt, fp_total, st));
    launches++;
    return AT_OK;
  };
  auto bp = [&](int stage, int u, int k) -> int {
    Launch L = base_launch(3);
    L.flow = FLOW_IMAGE;
    L.stage = stage;
    L.in_buf = B_R;
    L.out_buf = B_D;
    L.aux_buf = u;
    L.k = k;
    AT_CUDA_TRY(launch_bp(L, kind, bp_total, st));
    launches++;
    return AT_OK;
  };
  auto pix = [&](int which, int flow, int stage, int in, int out, int aux, int k, int flag) -> int {
    Launch L = base_launch(which == PK_SINO ? 2 : 1);
    L.flow = flow;
    L.stage = stage;
    L.in_buf = in;
    L.out_buf = out;
    L.aux_buf = aux;
    L.k = k;
    L.flag = flag;
    AT_CUDA_TRY(launch_pixel(which, L, which == PK_SINO ? sino_total : pix_total, st));
    launches++;
    return AT_OK;
  };
  int rc;
  AT_CUDA_TRY(launch_flags(scans_d, nscans, 0, st));
  launches++;
  // main.c:87-143
  if ((rc = fp(ST_FP0, B_F, linear ? B_AF : -1, 0))) return rc;
  if ((rc = bp(ST_BP0, B_F, 0))) return rc;
  if ((rc = pix(PK_PP, FLOW_IMAGE, ST_PP0, B_D, B_P0, -1, 0, 1))) return rc;
  for (int k = 1; k <= K; k++) {  // main.c:145-252
    const int pcur = (k & 1) ? B_P0 : B_P1, pnext = (k & 1) ? B_P1 : B_P0;
    const int ucur = (k & 1) ? B_F : B_U1, unext = (k & 1) ? B_U1 : B_F;
    const bool median = (k % m) == 0;
    if (linear && k >= 2) {
      if ((rc = pix(PK_SINO, FLOW_IMAGE, ST_SQ, -1, -1, -1, k, 0))) return rc;
    } else {
      if ((rc = fp(ST_FPQ, pcur, -1, k))) return rc;
    }
    if ((rc = pix(PK_UPD, FLOW_IMAGE, ST_UPD, pcur, unext, ucur, k, median ? 1 : 0))) return rc;
    if (k == K) break;  // the update pass ends the step at k == K
    if (linear && !median) {
      if ((rc = pix(PK_SINO, FLOW_IMAGE, ST_SA, -1, -1, -1, k, 0))) return rc;
    } else {
      if ((rc = fp(ST_FPA, unext, linear ? B_AF : -1, k))) return rc;
    }
    if ((rc = bp(ST_BPD, unext, k))) return rc;
    if ((rc = fp(ST_FPD, B_D, linear ? B_AD : -1, k))) return rc;
    if ((rc = pix(PK_PP, FLOW_IMAGE, ST_PP, pcur, pnext, -1, k, 0))) return rc;
  }
  if ((rc = pix(PK_COMMIT, FLOW_ENABLED, ST_NONE, -1, -1, -1, 0, 0))) return rc;
  return AT_OK;
}

// minimize_in_EDGE_variable, main.c:259-360
int Solver::enqueue_edge(cudaStream_t st) {
  const int KE = params.iter_edge;
  auto pix = [&](int which, int flow, int stage, int k) -> int {
    Launch L = base_launch(1);
    L.flow = flow;
    L.stage = stage;
    L.k = k;
    AT_CUDA_TRY(launch_pixel(which, L, pix_total, st));
    launches++;
    return AT_OK;
  };
  int rc;
  if ((rc = pix(PK_EDGE_INIT, FLOW_ENABLED, ST_NONE, 0))) return rc;
  AT_CUDA_TRY(launch_flags(scans_d, nscans, 1, st));
  launches++;
  for (int k = 1; k <= KE; k++) {
    if ((rc = pix(PK_EDGE_D, FLOW_EDGE, ST_E1, k))) return rc;
    if ((rc = pix(PK_EDGE_UPD, FLOW_EDGE, ST_E2, k))) return rc;
  }
  return AT_OK;
}

int Solver::ensure_graph(cudaStream_t st) {
  if (graph_exec) return AT_OK;
  cudaStream_t cap = own_stream;
  AT_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_outer(cap);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(cap, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
  graph = g;
  AT_CUDA_TRY(cudaGraphInstantiate(&graph_exec, graph, 0));
  (void)st;
  return AT_OK;
}

int Solver::step(int count, cudaStream_t st) {
  int rc;
  if ((rc = ensure_graph(st))) return rc;
  for (int i = 0; i < count; i++) AT_CUDA_TRY(cudaGraphLaunch(graph_exec, st));
  return AT_OK;
}

int Solver::run(cudaStream_t st) {
  int rc;
  if ((rc = reset(st))) return rc;
  return step(params.iter_alt, st);
}

}  // namespace at
