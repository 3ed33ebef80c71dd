// solver.h -- host side of the batched AT solver (solver.cu) and of the
// continuous-batching server (server.cu).
#pragma once

#include <vector>

#include "solver_dev.cuh"

namespace medimg {

void fill_scan_plan(ScanDev &S, const Plan &p);
// device bytes of one scan's state (images, sinograms, partials, trace, control)
size_t scan_bytes(const Plan &p, int rpt);
// points S's state buffers into `mem` (scan_bytes(p, rpt) bytes, 256-aligned)
void carve_scan(ScanDev &S, const Plan &p, int rpt, char *mem);
// control block of a fresh reconstruction
Ctl make_ctl(const at_params &prm);
// back-projection scratch of one scan (zero when handed to the kernels, left
// zero by them) and how it is laid out; bp_split = 1
size_t bp_scratch_bytes(const Plan &p);
void carve_bp_scratch(ScanDev &S, const Plan &p, char *mem);
// CTAs per back-projection tile for a launch over `tiles` tiles
int bp_split_for(int tiles, int nvb);

// CTA-range families of a batch's launches (rows of Batch::prefix_d)
// (in a batch with groups, the projections of the scans alone and of the
// pairs are launched apart from the groups of three or four: forward
// FAM_FP1 / FAM_FP2, back FAM_BPS)
enum Family { FAM_FP = 0, FAM_PIX = 1, FAM_SINO = 2, FAM_BP = 3, FAM_FP1 = 4, FAM_FP2 = 5, FAM_BPS = 6, kFamilies = 7 };

// The launch sequence of the AT iteration over a set of scans: one launch per
// kernel for the whole set, per-scan CTA ranges from prefix tables.
struct Batch {
  at_params params{};
  int kind = AT_GEOM_FAN, rpt = 1, nscans = 0, cap = 0;
  ScanDev *scans_d = nullptr;
  int *prefix_d = nullptr;  // [kFamilies][cap+1]: CTAs per scan of each family
  int fp_total = 0, pix_total = 0, sino_total = 0, bp_total = 0, fp1_total = 0, fp2_total = 0, bps_total = 0;
  int group = 1;            // largest group of scans sharing a plan (projected together)
  int cone_chunks = 1;      // cone beam: chunks of views of the batch's largest back projection
  // fan back projection: Launch::bp_table of the main launch (groups of three
  // or four, or every scan when nothing is grouped) and of the launch of pairs
  // and scans alone
  int bp_table_main = 0, bp_table_small = 0;
  // slab forward projector: used when every plan of the batch has slab tables
  // of one CTA shape; one TMA descriptor per scan (of its pack buffer, in its
  // group's form)
  bool slab = false;
  SlabLaunch slab_launch{};
  CUtensorMap *tmaps_d = nullptr;
  // persistent projector launches (fan beam and ray tables): a grid of
  // resident CTAs pulls (scan, view block, ray block) / (scan, pixel tile)
  // units from a queue, the units of the costlier scans first
  bool persistent = false;
  unsigned *queue_d = nullptr;  // [2]: next unit, CTAs done (left zero by the kernels)
  int *order_d = nullptr;       // unit order of each projector family
  size_t order_cap = 0;
  int order_off[kFamilies] = {};
  int launches = 0;         // kernel launches of the last enqueue_outer
  Batch() = default;
  Batch(const Batch &) = delete;
  Batch &operator=(const Batch &) = delete;
  ~Batch();
  int set(const ScanDev *scans, int n, int kind, int rpt, cudaStream_t st);
  Launch base_launch(int family) const;
  Launch retarget(const Launch &L, int family) const;
  // one forward / back projection of every scan (L from base_launch(FAM_FP /
  // FAM_BP) with flow, stage and buffers set); scans sharing a plan are grouped
  int enqueue_fp(const Launch &L, cudaStream_t st);
  int enqueue_bp(const Launch &L, cudaStream_t st);
  int enqueue_init(cudaStream_t st);
  int enqueue_outer(cudaStream_t st);
  int enqueue_image(cudaStream_t st);
  int enqueue_edge(cudaStream_t st);
};

// A fixed batch of scans in one device allocation, its outer iteration
// captured once as a CUDA graph.
struct Solver {
  std::vector<Plan *> plans;
  at_params params{};
  int nscans = 0;
  int rpt = 1;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  std::vector<ScanDev> host_scans;
  std::vector<Ctl> ctl_host;  // staging for control-block uploads
  Batch batch;
  cudaStream_t own_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int launches = 0;  // kernel launches per outer iteration

  static int choose_rpt(const std::vector<Plan *> &plans);
  static size_t footprint(const std::vector<Plan *> &plans, int rpt);
  int create(const std::vector<Plan *> &plans, const at_params &prm);
  ~Solver();
  int reset(cudaStream_t st);
  int reset_ctl(cudaStream_t st);
  int enable(int scan, bool on, cudaStream_t st);
  int enqueue_outer(cudaStream_t st);
  int enqueue_image(cudaStream_t st);
  int enqueue_edge(cudaStream_t st);
  int ensure_graph(cudaStream_t st);
  int step(int count, cudaStream_t st);
  int run(cudaStream_t st);
};

// A fixed list of plans projected together (at_projset_*): each call is one
// launch per kernel for the whole list, scans sharing a plan grouped.  Holds
// the scans' projector scratch (back-projection sums, interleaved group
// inputs) in one allocation, so calls on one set must not overlap.
struct ProjSet {
  std::vector<Plan *> plans;
  std::vector<ScanDev> host;
  std::vector<const void *> bound;  // buffers the device copy of `host` points at
  Batch batch;
  void *scratch = nullptr;
  int kind = AT_GEOM_FAN, rpt = 1;
  int create(const std::vector<Plan *> &plans);
  int project(bool forward, const float *const *in, float *const *out, cudaStream_t st);
  ~ProjSet();
};

}  // namespace medimg

struct at_projset {
  medimg::ProjSet p;
};

struct at_solver {
  medimg::Solver s;
};
