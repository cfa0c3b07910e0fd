// w3g_context.cuh -- the opaque w3g_context of include/w3g.h: resident
// device model and state, schedule, captured iteration graph. Shared by the
// C-ABI translation units (w3g_api.cu, w3g_solve.cu).
#pragma once
#include <chrono>
#include <string>
#include <vector>
#include <nvtx3/nvToolsExt.h>
#include "w3g_internal.cuh"

// one captured iteration (w3g_iteration_dev) and what it was captured for
struct IterationGraph {
  cudaGraphExec_t exec = nullptr;
  int what = 0, precision = -1;
  const void *c = nullptr, *u = nullptr, *du = nullptr, *ifv = nullptr;
  w3g::Schedule sched{};
  long long wait_limit = 0;
  int launches = 0;
};

struct w3g_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  w3g::DeviceModel m;
  w3g::DeviceState s;
  int precision = W3G_TANGENT_FP64;
  long long wait_limit = W3G_WAIT_LIMIT_DEFAULT;   // bounded waits of the tensor-core kernels
  int update_mode = W3G_UPDATE_COPY;
  w3g::Schedule sched{W3G_SCHED_PER_TYPE, 0, 0, 1, 1, W3G_ORDER_HEAVY_FIRST};
  IterationGraph graph;
  int ifv_parts = 0;
  int last_launches = 0;
  // host copies needed for state transfer
  std::vector<w3g::BlockDesc> blocks;
  double* h_stage = nullptr;   // pinned staging, max(estiff_total, ...) doubles
  size_t h_stage_n = 0;
  // w3g_tanstf with host Ke: the tangent runs in parts whose Ke goes to the
  // host on copy_stream while the next part computes
  std::vector<w3g::Chunk> h_tchunks;   // host copy of the tangent work items
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t part_done[8] = {};
  // host wall time per entry point (w3g_timers_get)
  double t_tangent = 0.0, t_recover = 0.0, t_update = 0.0;
  long long n_tangent = 0, n_recover = 0, n_update = 0;
};

// One C-ABI call: an NVTX range (visible in Nsight timelines) and its host
// wall time added to one of the context's accumulators, named after
// WARP3D's own timing categories (thyme calc 2 "tangent stiffness" around
// tanstf, calc 6 "sig-eps & internal force" around
// drive_eps_sig_internal_forces; src/thyme.f, src/outime.f).
struct CallScope {
  double* acc;
  long long* count;
  std::chrono::steady_clock::time_point t0;
  CallScope(const char* name, double* a, long long* n) : acc(a), count(n), t0(std::chrono::steady_clock::now()) {
    nvtxRangePushA(name);
  }
  ~CallScope() {
    nvtxRangePop();
    if (acc) {
      *acc += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      ++*count;
    }
  }
};


// records msg as the thread's last error (w3g_last_error) and returns code
int w3g_fail(int code, const std::string& msg);
