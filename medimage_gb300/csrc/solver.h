// solver.h -- host-side batched AT solver (see solver.cu).
#pragma once

#include <vector>

#include "solver_dev.cuh"

namespace at {

void fill_scan_plan(ScanDev &S, const Plan &p);

struct Solver {
  std::vector<Plan *> plans;
  at_params params{};
  int nscans = 0;
  int rpt = 1;  // rays per thread of the forward projector
  void *arena = nullptr;
  size_t arena_bytes = 0;
  std::vector<ScanDev> host_scans;
  ScanDev *scans_d = nullptr;
  int *prefix_d = nullptr;  // [4][nscans+1]: forward-projector, pixel-pass, sinogram-pass, back-projector CTAs
  int fp_total = 0, pix_total = 0, sino_total = 0, bp_total = 0;
  cudaStream_t own_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int launches = 0;  // kernel launches per outer iteration

  static int choose_rpt(const std::vector<Plan *> &plans);
  static size_t footprint(const std::vector<Plan *> &plans, int rpt);
  int create(const std::vector<Plan *> &plans, const at_params &prm);
  ~Solver();
  Launch base_launch(int family) const;
  std::vector<Ctl> ctl_host;  // staging for control-block uploads
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

}  // namespace at

struct at_solver {
  at::Solver s;
};
