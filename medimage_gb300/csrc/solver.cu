// solver.cu -- host orchestration of the batched AT solver.
//
// Each scan of a batch owns the state buffers of origin/GoldenC/src/main.c
// (f, v, d, p, update, r, q, ...), a control block with the CG scalars, FP64
// partial sums and a trace buffer.  A Batch issues the launch sequence of one
// outer iteration (image step then edge step, main.c:43-47) for a set of
// scans; early exits are decided on the device, so later launches of a
// finished step return at their first instruction.  A Solver keeps a fixed
// batch in one allocation and captures its outer iteration once as a CUDA
// graph; the server (server.cu) rebuilds its batch as requests come and go.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

#include "solver.h"

namespace medimg {

int fp_ctas(const ScanDev &S, int rpt);
int fp_group_ctas(const ScanDev &S);
int bp_ctas(const ScanDev &S);
int pix_ctas(const ScanDev &S);
cudaError_t launch_fp(const Launch &L, int kind, int rpt, int nctas, cudaStream_t st);
int launch_fp_group(const Launch &L, const Launch &Lpix, const Launch &L1, const Launch &L2, int nctas, int pix_nctas,
                    int nctas1, int nctas2, const SlabLaunch *slab, cudaStream_t st);
int launch_fp_tr(const Launch &L, const Launch &Lpix, int rpt, int nctas, int pix_nctas, const SlabLaunch *slab,
                 cudaStream_t st);
int slab_ctas(const ScanDev &S);
int cone_bp_launches(int chunks);
size_t slab_smem_bytes(int G, int rows, int wbox);
int encode_pack_tmap(CUtensorMap *out, const void *pack, int n, int G, int wbox, int rows);
int launch_bp_group(const Launch &L, const Launch &Lsino, const Launch &Lsmall, int nctas, int sino_nctas,
                    int small_nctas, cudaStream_t st);
cudaError_t launch_bp(const Launch &L, int kind, int nctas, cudaStream_t st, const Launch *Lpix, int pix_nctas);
cudaError_t launch_pixel(int which, const Launch &L, int nctas, cudaStream_t st);
cudaError_t launch_flags(const ScanDev *scans, int nscans, int mode, cudaStream_t st);

void fill_scan_plan(ScanDev &S, const Plan &p) {
  std::memset(&S, 0, sizeof(S));
  S.kind = p.kind;
  S.n = p.n;
  S.nviews = p.nviews;
  S.ndets = p.ndets;
  S.nz = p.nz;
  S.npix = p.nz * p.n * p.n;
  S.nbins = p.nviews * p.ndets;
  S.nbpv = p.nblocks_per_view;
  S.offgrid = p.offgrid ? 1 : 0;
  S.rays = p.rays_d;
  S.bits = p.bits_d;
  S.blk_word = p.blk_word_d;
  S.blk_off = p.blk_off_d;
  S.run = p.run_d;
  S.tile_off = p.tile_off_d;
  S.pt_meta = p.pt_meta_d;
  S.pt_w = p.pt_w_d;
  S.pt_woff = p.pt_woff_d;
  S.pt_use = p.pt_meta_d ? p.bp_table : 0;
  S.ntiles_y = p.ntiles_y;
  S.nvb = p.nvb;
  S.bp_term_bits = p.bp_term_bits;
  S.pixel_mm = (float)p.geom.pixel_mm;
  S.gc_seg = p.gc_seg_d;
  S.gc_pair_off = p.gc_pair_off_d;
  S.gc_ent = p.gc_ent_d;
  S.gc_pix_off = p.gc_pix_off_d;
  S.ndx = p.cone.ndx;
  S.ndy = p.cone.ndy;
  S.half_rows = p.cone.half_rows;
  S.half_cols = p.cone.half_cols;
  S.voxel = p.cone.voxel_mm;
  S.pitch = p.cone.pitch_mm;
  S.sod = p.cone.sod_mm;
  S.sdd = p.cone.sdd_mm;
  S.cone_trig = p.cone_trig_d;
  S.bp_vchunk = p.cone_bp_views;
  if (p.slab.ok) {
    S.slab_views = p.slab.views;
    S.slab_rays = p.slab.rays;
    S.slab_rows = p.slab.rows;
    S.slab_wbox = p.slab.wbox;
    S.slab_nslab = p.slab.nslab;
    S.slab_ndb = p.slab.ndb;
    S.slab_cta = p.slab.cta_d;
    S.slab_wlo = p.slab.wlo_d;
  }
}

namespace {
enum PixKernel { PK_UPD = 0, PK_PP, PK_COMMIT, PK_EDGE_INIT, PK_EDGE_D, PK_EDGE_UPD, PK_SINO, PK_INIT };

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

struct ScanLayout {
  size_t img_bytes, sino_bytes, partial_bytes, trace_bytes, bp_bytes, pack_bytes, total;
};

ScanLayout layout_of(const Plan &p, int rpt) {
  ScanLayout L;
  const size_t npix = (size_t)p.nz * p.n * p.n, nbins = (size_t)p.nviews * p.ndets;
  L.img_bytes = align_up(npix * sizeof(float));
  L.sino_bytes = align_up(nbins * sizeof(float));
  ScanDev tmp;
  fill_scan_plan(tmp, p);
  tmp.bp_split = kBpMaxSplit;  // size the partials for the largest split
  // and for one ray per thread (what grouped forward projections use)
  const int maxcta = std::max({fp_ctas(tmp, rpt), fp_group_ctas(tmp), bp_ctas(tmp), pix_ctas(tmp),
                               (int)((nbins + 255) / 256), p.slab.ok ? p.slab.ncta : 0});
  L.partial_bytes = align_up((size_t)maxcta * 4 * sizeof(double));
  L.trace_bytes = align_up((size_t)kTraceCap * 10 * sizeof(double));
  L.bp_bytes = bp_scratch_bytes(p);
  // fan beam and ray tables: a group's forward-projector inputs, interleaved
  const bool packs = p.kind == AT_GEOM_FAN || p.kind == AT_GEOM_RAYS;
  // (images twice: row-major and transposed)
  L.pack_bytes = packs ? align_up(sizeof(float4) * std::max(2 * (size_t)p.n * p.n, nbins)) : 0;
  L.total = L.img_bytes * B_NIMG + L.sino_bytes * (B_NBUF - B_NIMG) + L.partial_bytes + L.trace_bytes +
            L.bp_bytes + L.pack_bytes + align_up(sizeof(Ctl));
  return L;
}
}  // namespace

size_t scan_bytes(const Plan &p, int rpt) { return layout_of(p, rpt).total; }

void carve_scan(ScanDev &S, const Plan &p, int rpt, char *cur) {
  const ScanLayout lay = layout_of(p, rpt);
  fill_scan_plan(S, p);
  for (int b = 0; b < B_NIMG; b++) {
    S.buf[b] = (float *)cur;
    cur += lay.img_bytes;
  }
  for (int b = B_NIMG; b < B_NBUF; b++) {
    S.buf[b] = (float *)cur;
    cur += lay.sino_bytes;
  }
  S.partials = (double *)cur;
  cur += lay.partial_bytes;
  S.trace = (double *)cur;
  cur += lay.trace_bytes;
  carve_bp_scratch(S, p, cur);
  cur += lay.bp_bytes;
  S.pack = lay.pack_bytes ? (float4 *)cur : nullptr;
  cur += lay.pack_bytes;
  S.ctl = (Ctl *)cur;
}

size_t bp_scratch_bytes(const Plan &p) {
  if (p.kind == AT_GEOM_GOLDNC) return 0;
  const size_t npix = (size_t)p.nz * p.n * p.n;
  return align_up(sizeof(unsigned long long) * npix) + align_up(sizeof(int) * (size_t)p.ntiles) +
         align_up(sizeof(float) * kBpMaxParts) + (p.kind == AT_GEOM_CONE ? 2 * align_up(sizeof(int) * npix) : 0);
}

void carve_bp_scratch(ScanDev &S, const Plan &p, char *cur) {
  S.bp_split = 1;
  if (p.kind == AT_GEOM_GOLDNC) return;
  S.bp_acc = (unsigned long long *)cur;
  cur += align_up(sizeof(unsigned long long) * (size_t)p.nz * p.n * p.n);
  S.bp_cnt = (int *)cur;
  cur += align_up(sizeof(int) * (size_t)p.ntiles);
  S.bpmax = (float *)cur;
  cur += align_up(sizeof(float) * kBpMaxParts);
  if (p.kind == AT_GEOM_CONE) {
    const size_t npix = (size_t)p.nz * p.n * p.n;
    S.bp_acc32 = (int *)cur;
    S.bp_acc32x = (int *)(cur + align_up(sizeof(int) * npix));
  }
}

Ctl make_ctl(const at_params &prm) {
  Ctl c;
  std::memset(&c, 0, sizeof(c));
  c.enabled = 1;
  c.iter_image = prm.iter_image;
  c.iter_edge = prm.iter_edge;
  c.median_every = prm.iter_image / 2;
  c.mode = prm.mode;
  c.alpha = prm.alpha;
  c.beta = prm.beta;
  c.eps = prm.epsilon;
  return c;
}

// ---------------------------------------------------------------- Batch
// Whether batches made from now on run their fan-beam / ray-table projector
// launches persistent (a grid of the resident CTAs pulling work units from a
// queue) or one CTA per unit (the default: measured faster on GB300, see
// at_set_batch_launch_mode).  Results are bitwise the same either way.
std::atomic<int> g_persistent_batches{0};

Batch::~Batch() {
  cudaFree(scans_d);
  cudaFree(prefix_d);
  cudaFree(tmaps_d);
  cudaFree(queue_d);
  cudaFree(order_d);
}

int Batch::set(const ScanDev *scans, int n, int kind_, int rpt_, cudaStream_t st) {
  if (n <= 0) return set_error(AT_EINVAL, "batch: no scans");
  kind = kind_;
  rpt = rpt_;
  if (n > cap) {
    cudaFree(scans_d);
    cudaFree(prefix_d);
    cudaFree(tmaps_d);
    scans_d = nullptr;
    prefix_d = nullptr;
    tmaps_d = nullptr;
    cap = std::max(n, 2 * cap);
    AT_CUDA_TRY(cudaMalloc(&scans_d, sizeof(ScanDev) * cap));
    AT_CUDA_TRY(cudaMalloc(&prefix_d, sizeof(int) * kFamilies * (cap + 1)));
    AT_CUDA_TRY(cudaMalloc(&tmaps_d, sizeof(CUtensorMap) * cap));
  }
  nscans = n;
  std::vector<ScanDev> sc(scans, scans + n);
  // scans sharing a plan (fan beam, ray tables) are projected together, up to
  // kGroupMax per group: the lead (first of them) lists the members and gets
  // the projector CTAs, the others none
  group = 1;
  for (int s = 0; s < n; s++) {
    sc[s].nmem = 1;
    sc[s].mem[0] = s;
  }
  if (kind == AT_GEOM_FAN || kind == AT_GEOM_RAYS) {
    for (int s = 1; s < n; s++) {
      for (int t = 0; t < s; t++) {
        if (sc[t].nmem > 0 && sc[t].nmem < kGroupMax && sc[t].rays == sc[s].rays) {
          sc[t].mem[sc[t].nmem++] = s;
          sc[s].nmem = 0;
          break;
        }
      }
    }
    // back-projection split from the tiles of the whole launch
    int tiles = 0, nvb = 1 << 30;
    for (const auto &S : sc) {
      group = std::max(group, S.nmem);
      if (S.nmem) tiles += S.ntiles_y * S.ntiles_y;
      nvb = std::min(nvb, S.nvb);
    }
    const int split = bp_split_for(tiles, nvb);
    for (auto &S : sc) S.bp_split = split;
  }
  // the slab forward projector, when every plan has slab tables of one CTA
  // shape: each lead's TMA descriptor covers its pack buffer in its group's
  // form, and the launch's shared memory the largest slab buffers
  slab = (kind == AT_GEOM_FAN || kind == AT_GEOM_RAYS);
  for (const auto &S : sc)
    slab = slab && S.slab_cta && S.pack && S.slab_views == sc[0].slab_views && S.slab_rays == sc[0].slab_rays;
  std::vector<CUtensorMap> maps;
  if (slab) {
    slab_launch = SlabLaunch{sc[0].slab_views * sc[0].slab_rays, {0, 0, 0}};
    maps.resize(n);
    for (int s = 0; s < n; s++) {
      ScanDev &S = sc[s];
      const int G = S.nmem >= 3 ? 4 : S.nmem == 2 ? 2 : 1;
      const int form = G == 4 ? 0 : G == 1 ? 1 : 2;
      slab_launch.smem[form] = std::max(slab_launch.smem[form], slab_smem_bytes(G, S.slab_rows, S.slab_wbox));
      S.tmap = tmaps_d + s;
      if (S.nmem == 0) continue;  // a member: its lead's walk reads the group's pack buffer
      int rc = encode_pack_tmap(&maps[s], S.pack, S.n, G, S.slab_wbox, S.slab_rows);
      if (rc) return rc;
    }
    AT_CUDA_TRY(cudaMemcpyAsync(tmaps_d, maps.data(), sizeof(CUtensorMap) * n, cudaMemcpyHostToDevice, st));
  }
  scans = sc.data();
  cone_chunks = 1;
  for (const auto &S : sc)
    if (S.kind == AT_GEOM_CONE) cone_chunks = std::max(cone_chunks, (S.nviews + S.bp_vchunk - 1) / std::max(1, S.bp_vchunk));
  std::vector<int> pref(kFamilies * (n + 1), 0);
  auto add = [&](int fam, int s, int ctas) { pref[fam * (n + 1) + s + 1] = pref[fam * (n + 1) + s] + ctas; };
  for (int s = 0; s < n; s++) {
    const int nm = scans[s].nmem;
    if (group > 1) {
      // grouped projectors walk one ray per thread; groups of three or four
      // and the rest (pairs, scans alone) in launches of their own
      const bool big = nm >= 3, small = nm == 1 || nm == 2;
      const int fpc = slab ? slab_ctas(scans[s]) : fp_group_ctas(scans[s]);
      add(FAM_FP, s, big ? fpc : 0);
      add(FAM_FP1, s, nm == 1 ? fpc : 0);
      add(FAM_FP2, s, nm == 2 ? fpc : 0);
      add(FAM_BP, s, big ? bp_ctas(scans[s]) : 0);
      add(FAM_BPS, s, small ? bp_ctas(scans[s]) : 0);
    } else {
      add(FAM_FP, s, slab ? slab_ctas(scans[s]) : fp_ctas(scans[s], rpt));
      add(FAM_FP1, s, 0);
      add(FAM_FP2, s, 0);
      add(FAM_BP, s, bp_ctas(scans[s]));
      add(FAM_BPS, s, 0);
    }
    add(FAM_PIX, s, pix_ctas(scans[s]));
    add(FAM_SINO, s, (scans[s].nbins + 255) / 256);
  }
  // pixel tables: one kernel form when every scan of a launch agrees, else a
  // choice per CTA
  auto table_mode = [&](int fam) {
    int with = 0, without = 0;
    for (int s = 0; s < n; s++) {
      if (pref[fam * (n + 1) + s + 1] == pref[fam * (n + 1) + s]) continue;
      const ScanDev &S = scans[s];
      const bool t = (kind == AT_GEOM_FAN || kind == AT_GEOM_RAYS) && (S.pt_use & (S.nmem > 1 ? 2 : 1)) != 0;
      (t ? with : without)++;
    }
    return with == 0 ? 0 : without == 0 ? 1 : 2;
  };
  bp_table_main = table_mode(FAM_BP);
  bp_table_small = table_mode(FAM_BPS);
  fp_total = pref[FAM_FP * (n + 1) + n];
  pix_total = pref[FAM_PIX * (n + 1) + n];
  sino_total = pref[FAM_SINO * (n + 1) + n];
  bp_total = pref[FAM_BP * (n + 1) + n];
  fp1_total = pref[FAM_FP1 * (n + 1) + n];
  fp2_total = pref[FAM_FP2 * (n + 1) + n];
  bps_total = pref[FAM_BPS * (n + 1) + n];
  // work orders of the persistent projector launches: per family, the units
  // of each scan in their natural order, scans by decreasing work per unit
  // (segments ~ views x detectors x n), so the cheapest units come last
  persistent = g_persistent_batches.load() != 0 && (kind == AT_GEOM_FAN || kind == AT_GEOM_RAYS);
  if (persistent) {
    std::vector<int> order;
    const int fams[5] = {FAM_FP, FAM_FP1, FAM_FP2, FAM_BP, FAM_BPS};
    for (int f : fams) {
      order_off[f] = (int)order.size();
      std::vector<int> idx;
      for (int s = 0; s < n; s++)
        if (pref[f * (n + 1) + s + 1] > pref[f * (n + 1) + s]) idx.push_back(s);
      auto density = [&](int s) {
        const double units = pref[f * (n + 1) + s + 1] - pref[f * (n + 1) + s];
        return (double)scans[s].nviews * scans[s].ndets * scans[s].n / units;
      };
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return density(a) > density(b); });
      for (int s : idx)
        for (int u = pref[f * (n + 1) + s]; u < pref[f * (n + 1) + s + 1]; u++) order.push_back(u);
    }
    if (!queue_d) {
      AT_CUDA_TRY(cudaMalloc(&queue_d, 2 * sizeof(unsigned)));
      AT_CUDA_TRY(cudaMemsetAsync(queue_d, 0, 2 * sizeof(unsigned), st));
    }
    if (order.size() > order_cap) {
      cudaFree(order_d);
      order_d = nullptr;
      order_cap = std::max(order.size(), 2 * order_cap);
      AT_CUDA_TRY(cudaMalloc(&order_d, sizeof(int) * order_cap));
    }
    if (!order.empty())
      AT_CUDA_TRY(cudaMemcpyAsync(order_d, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, st));
  }
  // pageable sources: the copies are staged before cudaMemcpyAsync returns
  AT_CUDA_TRY(cudaMemcpyAsync(scans_d, scans, sizeof(ScanDev) * n, cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaMemcpyAsync(prefix_d, pref.data(), sizeof(int) * pref.size(), cudaMemcpyHostToDevice, st));
  return AT_OK;
}

// L with family's CTA ranges and, for persistent projector families, its
// work order (other families: no queue)
Launch Batch::retarget(const Launch &L0, int family) const {
  const Launch B = base_launch(family);
  Launch L = L0;
  L.prefix = B.prefix;
  L.queue = B.queue;
  L.order = B.order;
  L.units = B.units;
  return L;
}

Launch Batch::base_launch(int family) const {
  Launch L;
  std::memset(&L, 0, sizeof(L));
  L.scans = scans_d;
  L.nscans = nscans;
  L.prefix = prefix_d + family * (nscans + 1);
  L.aux_buf = -1;
  L.group = (family == FAM_PIX || family == FAM_SINO) ? 1 : group;
  L.chunks = cone_chunks;
  const bool fp = family == FAM_FP || family == FAM_FP1 || family == FAM_FP2;
  if (persistent && (family == FAM_BP || family == FAM_BPS || (fp && !slab))) {
    L.queue = queue_d;
    L.order = order_d + order_off[family];
    const int totals[kFamilies] = {fp_total, pix_total, sino_total, bp_total, fp1_total, fp2_total, bps_total};
    L.units = totals[family];
  }
  return L;
}

int Batch::enqueue_fp(const Launch &L, cudaStream_t st) {
  if (group > 1) {  // interleave each group's inputs, then one walk per group
    const Launch Lp = retarget(L, FAM_PIX), L1 = retarget(L, FAM_FP1), L2 = retarget(L, FAM_FP2);
    const int nl = launch_fp_group(L, Lp, L1, L2, fp_total, pix_total, fp1_total, fp2_total,
                                   slab ? &slab_launch : nullptr, st);
    AT_CUDA_TRY(cudaGetLastError());
    if (nl < 0) return set_error(AT_ECUDA, "grouped forward projection launch failed");
    launches += nl;
  } else if (kind == AT_GEOM_FAN || kind == AT_GEOM_RAYS) {  // transpose each input, then walk
    const Launch Lp = retarget(L, FAM_PIX);
    const int nl = launch_fp_tr(L, Lp, rpt, fp_total, pix_total, slab ? &slab_launch : nullptr, st);
    AT_CUDA_TRY(cudaGetLastError());
    if (nl < 0) return set_error(AT_ECUDA, "forward projection launch failed");
    launches += nl;
  } else {
    AT_CUDA_TRY(launch_fp(L, kind, rpt, fp_total, st));
    launches++;
  }
  return AT_OK;
}

int Batch::enqueue_bp(const Launch &L, cudaStream_t st) {
  if (group > 1) {  // max |r|, interleave each group's sinograms, then one run walk per group
    const Launch Ls = retarget(L, FAM_SINO);
    Launch Lb = L, Lsm = retarget(L, FAM_BPS);
    Lb.bp_table = bp_table_main;
    Lsm.bp_table = bp_table_small;
    launches += launch_bp_group(Lb, Ls, Lsm, bp_total, sino_total, bps_total, st);
    AT_CUDA_TRY(cudaGetLastError());
    return AT_OK;
  }
  const Launch Lp = retarget(L, FAM_PIX);  // the per-pixel finishing pass of the cone-beam back projector
  Launch Lb = L;
  Lb.bp_table = bp_table_main;
  AT_CUDA_TRY(launch_bp(Lb, kind, bp_total, st, &Lp, pix_total));
  // max |r| pass + back projection (cone beam: its chunks, folds and per-pixel finish)
  launches += kind == AT_GEOM_GOLDNC ? 1 : kind == AT_GEOM_CONE ? cone_bp_launches(cone_chunks) : 2;
  return AT_OK;
}

int Batch::enqueue_init(cudaStream_t st) {
  Launch L = base_launch(FAM_PIX);
  L.flow = FLOW_ENABLED;
  AT_CUDA_TRY(launch_pixel(PK_INIT, L, pix_total, st));
  return AT_OK;
}

// The launch sequence of one outer iteration (main.c:45-46).
int Batch::enqueue_outer(cudaStream_t st) {
  launches = 0;
  int rc;
  if ((rc = enqueue_image(st))) return rc;
  return enqueue_edge(st);
}

// minimize_in_IMAGE_variable, main.c:81-257
int Batch::enqueue_image(cudaStream_t st) {
  const int K = params.iter_image;
  const bool linear = params.mode == 1;
  const int m = K / 2;  // median every (int)(IterImage/2) iterations, main.c:180
  auto fp = [&](int stage, int in, int aux, int k) -> int {
    Launch L = base_launch(FAM_FP);
    L.flow = FLOW_IMAGE;
    L.stage = stage;
    L.in_buf = in;
    L.aux_buf = aux;
    L.k = k;
    return enqueue_fp(L, st);
  };
  auto bp = [&](int stage, int u, int k) -> int {
    Launch L = base_launch(FAM_BP);
    L.flow = FLOW_IMAGE;
    L.stage = stage;
    L.in_buf = B_R;
    L.out_buf = B_D;
    L.aux_buf = u;
    L.k = k;
    return enqueue_bp(L, st);
  };
  auto pix = [&](int which, int flow, int stage, int in, int out, int aux, int k, int flag) -> int {
    Launch L = base_launch(which == PK_SINO ? FAM_SINO : FAM_PIX);
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
int Batch::enqueue_edge(cudaStream_t st) {
  const int KE = params.iter_edge;
  auto pix = [&](int which, int flow, int stage, int k) -> int {
    Launch L = base_launch(FAM_PIX);
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

// ---------------------------------------------------------------- Solver
int Solver::choose_rpt(const std::vector<Plan *> &plans) {
  // rays per thread of the forward projector: the autotuned choice of the
  // batch's first plan (projections are bitwise identical for every choice)
  return plans.empty() ? 1 : plans[0]->fp_rpt;
}

size_t Solver::footprint(const std::vector<Plan *> &plans, int rpt) {
  size_t tot = 0;
  for (auto *p : plans) tot += scan_bytes(*p, rpt);
  return tot + 4096 * 4;
}

int Solver::create(const std::vector<Plan *> &pl, const at_params &prm) {
  if (pl.empty()) return set_error(AT_EINVAL, "solver: no scans");
  const int kind = pl[0]->kind;
  // one batch runs one set of kernels: GoldenC, fan beam and ray tables, or cone beam
  auto family = [](int k) { return k == AT_GEOM_RAYS ? AT_GEOM_FAN : k; };
  for (auto *p : pl)
    if (family(p->kind) != family(kind))
      return set_error(AT_EINVAL, "solver: a batch holds GoldenC, fan-beam/ray-table or cone-beam plans, not a mix");
  if (prm.iter_image < 2) return set_error(AT_EINVAL, "solver: iter_image must be >= 2 (the reference divides by iter_image/2)");
  if (prm.iter_edge < 1 || prm.iter_alt < 0) return set_error(AT_EINVAL, "solver: iteration counts must be positive");
  if (prm.mode != 0 && prm.mode != 1) return set_error(AT_EINVAL, "solver: mode must be 0 (exact) or 1 (linear)");
  plans = pl;
  params = prm;
  nscans = (int)pl.size();
  rpt = choose_rpt(pl);
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
  size_t total = 0;
  for (int s = 0; s < nscans; s++) total += scan_bytes(*pl[s], rpt);
  if (cudaMalloc(&arena, total) != cudaSuccess) {
    cudaGetLastError();
    return set_error(AT_ENOMEM, "solver: device allocation of " + std::to_string(total) + " bytes failed");
  }
  arena_bytes = total;
  AT_CUDA_TRY(cudaMemset(arena, 0, total));
  host_scans.resize(nscans);
  char *cur = (char *)arena;
  for (int s = 0; s < nscans; s++) {
    carve_scan(host_scans[s], *pl[s], rpt, cur);
    cur += scan_bytes(*pl[s], rpt);
  }
  batch.params = prm;
  int rc = batch.set(host_scans.data(), nscans, kind, rpt, own_stream);
  if (rc) return rc;
  AT_CUDA_TRY(cudaStreamSynchronize(own_stream));
  return AT_OK;
}

// ---------------------------------------------------------------- ProjSet
int ProjSet::create(const std::vector<Plan *> &pl) {
  if (pl.empty()) return set_error(AT_EINVAL, "projection set: no plans");
  kind = pl[0]->kind;
  auto family = [](int k) { return k == AT_GEOM_RAYS ? AT_GEOM_FAN : k; };
  for (auto *p : pl)
    if (family(p->kind) != family(kind))
      return set_error(AT_EINVAL, "projection set: GoldenC, fan-beam/ray-table or cone-beam plans, not a mix");
  plans = pl;
  rpt = Solver::choose_rpt(pl);
  const int n = (int)pl.size();
  auto pack_of = [](const Plan &p) {
    const size_t elems = std::max(2 * (size_t)p.n * p.n, (size_t)p.nviews * p.ndets);
    return (p.kind == AT_GEOM_FAN || p.kind == AT_GEOM_RAYS) ? align_up(sizeof(float4) * elems) : 0;
  };
  size_t total = 256;
  for (auto *p : pl) total += bp_scratch_bytes(*p) + pack_of(*p);
  if (cudaMalloc(&scratch, total) != cudaSuccess) {
    cudaGetLastError();
    return set_error(AT_ENOMEM, "projection set: device allocation of " + std::to_string(total) + " bytes failed");
  }
  AT_CUDA_TRY(cudaMemset(scratch, 0, total));
  host.resize(n);
  bound.assign(2 * n, nullptr);
  char *cur = (char *)scratch;
  for (int s = 0; s < n; s++) {
    fill_scan_plan(host[s], *pl[s]);
    carve_bp_scratch(host[s], *pl[s], cur);
    cur += bp_scratch_bytes(*pl[s]);
    host[s].pack = pack_of(*pl[s]) ? (float4 *)cur : nullptr;
    cur += pack_of(*pl[s]);
  }
  return AT_OK;
}

int ProjSet::project(bool forward, const float *const *in, float *const *out, cudaStream_t st) {
  const int n = (int)plans.size();
  bool same = true;
  for (int s = 0; s < n; s++) {
    if (!in[s] || !out[s]) return set_error(AT_EINVAL, "projection set: null buffer");
    same &= bound[2 * s] == in[s] && bound[2 * s + 1] == out[s];
    host[s].buf[0] = const_cast<float *>(in[s]);
    host[s].buf[1] = out[s];
  }
  if (!same) {  // re-point the device copy (and the CTA tables) at the new buffers
    int rc = batch.set(host.data(), n, kind, rpt, st);
    if (rc) return rc;
    for (int s = 0; s < n; s++) {
      bound[2 * s] = in[s];
      bound[2 * s + 1] = out[s];
    }
  }
  Launch L = batch.base_launch(forward ? FAM_FP : FAM_BP);
  L.flow = FLOW_ALWAYS;
  L.stage = ST_NONE;
  L.in_buf = 0;
  L.out_buf = 1;
  L.aux_buf = -1;
  return forward ? batch.enqueue_fp(L, st) : batch.enqueue_bp(L, st);
}

ProjSet::~ProjSet() { cudaFree(scratch); }

Solver::~Solver() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  cudaFree(arena);
  if (own_stream) cudaStreamDestroy(own_stream);
}

int Solver::reset(cudaStream_t st) {
  int rc;
  if ((rc = reset_ctl(st))) return rc;
  return batch.enqueue_init(st);
}

int Solver::reset_ctl(cudaStream_t st) {
  ctl_host.assign(nscans, make_ctl(params));
  for (int s = 0; s < nscans; s++)
    AT_CUDA_TRY(cudaMemcpyAsync(host_scans[s].ctl, &ctl_host[s], sizeof(Ctl), cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));  // ctl_host may be rewritten by the next reset
  return AT_OK;
}

int Solver::enable(int scan, bool on, cudaStream_t st) {
  const int v = on ? 1 : 0;
  AT_CUDA_TRY(cudaMemcpyAsync(&host_scans[scan].ctl->enabled, &v, sizeof(int), cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  return AT_OK;
}

int Solver::enqueue_outer(cudaStream_t st) {
  const int rc = batch.enqueue_outer(st);
  launches = batch.launches;
  return rc;
}

int Solver::enqueue_image(cudaStream_t st) { return batch.enqueue_image(st); }
int Solver::enqueue_edge(cudaStream_t st) { return batch.enqueue_edge(st); }

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

}  // namespace medimg

extern "C" __attribute__((visibility("default"))) int at_set_batch_launch_mode(int32_t persistent) {
  if (persistent != 0 && persistent != 1)
    return medimg::set_error(AT_EINVAL, "at_set_batch_launch_mode: 0 (one CTA per unit) or 1 (persistent)");
  medimg::g_persistent_batches.store(persistent);
  return AT_OK;
}
