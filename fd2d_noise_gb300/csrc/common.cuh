// common.cuh -- shared internals of libfd2d: status plumbing, device buffers,
// launch accounting and the host-side problem setup (grid, taper, indices,
// coefficient tables) of the fd2d_noise solvers.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fd2d.h"

namespace fd2d {

// ---- errors -------------------------------------------------------------------
struct Error {
  fd2d_status code;
  std::string msg;
};

#define FD2D_TRY(expr)                                  \
  do {                                                  \
    fd2d_status _s = (expr);                            \
    if (_s != FD2D_OK) return _s;                       \
  } while (0)

// Records the message on the context and returns the status.
fd2d_status set_error(fd2d_ctx* ctx, fd2d_status s, const std::string& msg);

#define FD2D_CUDA(ctx, expr)                                                        \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess)                                                          \
      return ::fd2d::set_error((ctx), _e == cudaErrorMemoryAllocation ? FD2D_ERR_OOM \
                                                                      : FD2D_ERR_CUDA, \
                               std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// Work done once per CUDA device, the first time a caller reaches it with that
// device current: kernel attributes such as the dynamic shared-memory opt-in
// belong to a device, not to the process.  Callers on several host threads are
// serialised; a failed attempt is retried by the next caller.
class PerDeviceOnce {
 public:
  template <typename F>
  fd2d_status run(fd2d_ctx* ctx, F&& work) {
    int dev = 0;
    FD2D_CUDA(ctx, cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu_);
    if ((size_t)dev < done_.size() && done_[dev]) return FD2D_OK;
    FD2D_TRY(work());
    if ((size_t)dev >= done_.size()) done_.resize((size_t)dev + 1, 0);
    done_[dev] = 1;
    return FD2D_OK;
  }

 private:
  std::mutex mu_;
  std::vector<char> done_;
};

// ---- host problem setup ---------------------------------------------------------
// Everything a solver needs from fd2d_config, derived once on the host.
struct Geometry {
  int nx = 0, nz = 0, nt = 0, ntc = 0, order = 4, r = 2, K = 0, fs = 1, fw = 1, nb = 0;
  double Lx = 0, Lz = 0, dt = 0, dx = 0, dz = 0, dw = 0;
  std::vector<double> x, z, w;
  std::shared_ptr<const std::vector<double>> absbound;  // taper, nx*nz column-major (shared: copies are cheap)
  double c[4] = {0, 0, 0, 0};             // staggered coefficients c_1..c_r
  std::vector<double> t_fwd, t_corr;      // time axes (0:dt:(nt-1)dt and -(nt-1)dt:dt:(nt-1)dt)
  uint64_t key = 0;                       // identity of the configuration (config_hash)
  int64_t npts() const { return (int64_t)nx * nz; }
};

std::vector<double> matlab_colon(double a, double d, double b);
int nearest_node(const std::vector<double>& x, double p);
fd2d_status make_geometry(const fd2d_config* cfg, Geometry& g, std::string& err);
// interpol_matrix (K-by-max(nb,1), column-major): code/run_forward2_correlation.m:121-165
fd2d_status make_interpol_matrix(int K, int nb, std::vector<double>& M, std::string& err);
// 1/sqrt(2 pi) * exp(1i*th) * scale  (evaluated in the reference's order)
inline void dft_coeff(double th, double scale, double& re, double& im) {
  const double s = 1 / std::sqrt(2 * M_PI);
  re = (s * std::cos(th)) * scale;
  im = (s * std::sin(th)) * scale;
}

// ---- device buffers ---------------------------------------------------------------
// A grow-only device allocation owned by a context.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  uint64_t tag = 0;  // identity of the content last uploaded (upload_tagged)
};

}  // namespace fd2d

// Context (opaque in the C ABI).
struct fd2d_ctx {
  int device = 0;
  int precision = FD2D_PREC_FP32;
  int memspace = FD2D_MEM_HOST;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t launches = 0;
  std::string last_error;
  int sm_count = 0;
  // named workspace buffers
  std::vector<std::pair<std::string, fd2d::DevBuf>> bufs;
  // device-side error flag of bounded waits (int32)
  int* d_err = nullptr;
  // instrumentation (fd2d_ctx_set_timing)
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  struct TimerRec { int a, b, cls; int64_t units, count; };
  std::vector<TimerRec> recs;
  double t_ms[FD2D_TIMER_COUNT] = {0, 0, 0};
  int64_t t_cnt[FD2D_TIMER_COUNT] = {0, 0, 0};
  int64_t t_units[FD2D_TIMER_COUNT] = {0, 0, 0};
  // CUDA-graph capture of time loops (fd2d::run_captured)
  bool capturing = false;
  std::vector<cudaEvent_t> cap_ev;    // timing events recorded inside the capture
  std::vector<TimerRec> cap_recs;
  struct GraphEntry {
    uint64_t key = 0;
    uint64_t seen = 0;  // key of the last run launched eagerly (not captured)
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaEvent_t> ev;
    std::vector<TimerRec> recs;
    int64_t launches = 0;  // kernels inside the graph
  };
  std::vector<std::pair<std::string, GraphEntry>> graphs;
  // batches: workspace names of job j carry a prefix; side streams and events
  // fork the jobs' loops into parallel branches of one captured graph
  std::string ws_prefix;
  int64_t mem_budget = 0;  // batch device-memory budget (0: 80 % of free memory)
  int32_t max_dft_chunk = 0;  // snapshots per DFT contraction (0: DFT_CHUNK_DEFAULT, within 2 GiB)
  int32_t max_inj_chunk = 0;  // resident injection planes (0: within 4 GiB)
  std::vector<int32_t> last_lanes;  // lanes of each launch group of the last batch
  int32_t tile_rows = 0;       // step-kernel tile rows: 0 timed per grid, -1 size rule, 16 or 32 forced
  int32_t last_tile_rows = 0;  // tile rows of the last FP32 time loop set up
  std::map<uint64_t, int> tile_choice;  // tuned tile rows by (grid, order, lanes)
  int32_t time_depth = 0;               // steps per launch: 0 timed per grid (orders 2, 4), 1 or 2 forced
  int32_t last_time_depth = 0;          // steps per launch of the last FP32 time loop set up
  std::map<uint64_t, int> depth_choice;  // tuned steps per launch by (grid, order, lanes, tile rows)
  int32_t concurrent_groups = 0;        // lane groups a batch runs side by side (set while planning)
  int32_t shared_gpu = 0;               // other work shares the GPU (fd2d_ctx_set_shared_gpu)
  std::vector<cudaStream_t> side_streams;
  std::vector<cudaEvent_t> fork_events;
};

namespace fd2d {

// Snapshots per DFT contraction unless fd2d_ctx_set_chunks says otherwise.  A
// chunk is summed in two halves, each in FP32 in tensor memory, and the chunks
// in FP64, so every FP32 sum covers at most 320 snapshots: the FP32 mu kernel
// of a 512x512, nt 2500 structure-kernel run (500 snapshots, halves of 250)
// is then within 1e-4 of the FP64 form (1.4e-4 with one FP32 sum over all
// 500), and the 600 snapshots of an nt 3000 Green run take one pass.
constexpr int DFT_CHUNK_DEFAULT = 640;

// Returns a device buffer of at least `bytes` under `name` (grown when needed).
fd2d_status workspace(fd2d_ctx* ctx, const char* name, size_t bytes, void** out);
template <typename T>
fd2d_status workspace_t(fd2d_ctx* ctx, const char* name, size_t count, T** out) {
  return workspace(ctx, name, count * sizeof(T) + 256, reinterpret_cast<void**>(out));
}
// Release every workspace buffer of the context.
void free_workspace(fd2d_ctx* ctx);

// Brackets the next launch(es) with timing events when instrumentation is on.
int timer_begin(fd2d_ctx* ctx, cudaStream_t stream);
// `count` launches of class `cls` doing `units` work ran between begin and end.
void timer_end(fd2d_ctx* ctx, cudaStream_t stream, int begin, int cls, int64_t units, int64_t count = 1);

// Checks the last launch and counts it.
fd2d_status after_launch(fd2d_ctx* ctx, const char* what);
// Start of an entry point: ctx non-NULL, its device current, last error cleared.
fd2d_status check_ctx(fd2d_ctx* ctx);
// End of an entry point: host memspace waits for the stream and reports a
// device-side wait that gave up.
fd2d_status finish_call(fd2d_ctx* ctx);

// Signature of everything a captured time loop depends on (FNV-1a).
struct Sig {
  uint64_t h = 1469598103934665603ull;
  void bytes(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
  }
  template <typename T>
  void add(const T& v) { bytes(&v, sizeof(T)); }
  template <typename T>
  void add_vec(const std::vector<T>& v) { add(v.size()); if (!v.empty()) bytes(v.data(), v.size() * sizeof(T)); }
};

// Runs `body` (a sequence of launches on ctx->stream, no allocation or host
// synchronisation inside) as a CUDA graph.  The instantiated graph is cached
// under `name` and replayed while `key` is unchanged; otherwise the body is
// captured again and the executable graph updated or re-instantiated.
template <typename F>
fd2d_status run_captured(fd2d_ctx* ctx, const char* name, uint64_t key, F&& body);
fd2d_status graph_begin(fd2d_ctx* ctx, const char* name, uint64_t key, bool* replayed, bool* eager);
fd2d_status graph_end(fd2d_ctx* ctx, const char* name, uint64_t key, fd2d_status body_status);

template <typename F>
fd2d_status run_captured(fd2d_ctx* ctx, const char* name, uint64_t key, F&& body) {
  bool replayed = false, eager = false;
  FD2D_TRY(graph_begin(ctx, name, key, &replayed, &eager));
  if (replayed) return FD2D_OK;
  fd2d_status s = body();
  if (eager) return s;
  return graph_end(ctx, name, key, s);
}

// Copies an input array to the device (host memspace) or passes it through.
// n == 0 or src == nullptr gives nullptr.
fd2d_status stage_in(fd2d_ctx* ctx, const char* name, const void* src, size_t bytes,
                     const void** dev);
// Output buffer on the device: the caller's pointer (device memspace) or a
// workspace buffer whose content is copied back by stage_out.
fd2d_status out_buffer(fd2d_ctx* ctx, const char* name, void* user, size_t bytes, void** dev);
fd2d_status stage_out(fd2d_ctx* ctx, void* user, const void* dev, size_t bytes);

// Like upload(), but the content is only generated and copied when the buffer's
// tag differs from `tag` (tables that depend only on the configuration).
fd2d_status workspace_tag(fd2d_ctx* ctx, const char* name, size_t bytes, uint64_t tag, void** out, bool* hit);
template <typename T, typename F>
fd2d_status upload_tagged(fd2d_ctx* ctx, const char* name, uint64_t tag, size_t count, F&& fill, T** dev) {
  bool hit = false;
  void* p = nullptr;
  FD2D_TRY(workspace_tag(ctx, name, (count ? count : 1) * sizeof(T) + 256, tag, &p, &hit));
  *dev = static_cast<T*>(p);
  if (hit || count == 0) return FD2D_OK;
  std::vector<T> h(count);
  fill(h);
  cudaError_t e = cudaMemcpyAsync(p, h.data(), count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return set_error(ctx, FD2D_ERR_CUDA, std::string("upload ") + name + ": " + cudaGetErrorString(e));
  // pageable source: the copy has been staged when cudaMemcpyAsync returns
  return FD2D_OK;
}

// Identity of a configuration (all fields and frequencies).
uint64_t config_hash(const fd2d_config* cfg);

// Uploads a host vector into a named workspace buffer (async on the ctx stream).
template <typename T>
fd2d_status upload(fd2d_ctx* ctx, const char* name, const std::vector<T>& v, T** dev) {
  FD2D_TRY(workspace_t<T>(ctx, name, v.size() ? v.size() : 1, dev));
  if (!v.empty()) {
    cudaError_t e = cudaMemcpyAsync(*dev, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e != cudaSuccess) return set_error(ctx, FD2D_ERR_CUDA, std::string("upload ") + name + ": " + cudaGetErrorString(e));
  }
  return FD2D_OK;
}

// Arguments of one solve, already validated (pointers are device pointers).
struct SolveArgs {
  const double *mu = nullptr, *rho = nullptr, *dmu = nullptr;
  // point sources (indices into the nx*nz grid) and receivers
  std::vector<int> src_idx, rec_idx;
  int mode = 0;
  // forward1
  const float* G_in = nullptr;
  int n_G_in = 0;
  double *G_re = nullptr, *G_im = nullptr;  // outputs (fwd1) or inputs (corr/adj)
  float* G_out = nullptr;
  // correlation / adjoint
  const double *Gin_re = nullptr, *Gin_im = nullptr;
  int n_G = 0;
  const double* spectrum = nullptr;  // K x n_src
  int n_src = 0;
  const double* source_dist = nullptr;
  int n_dist = 0;
  const float* C_in = nullptr;  // Born snapshots (C_in or u_in)
  int n_C_in = 0;
  float* C_out = nullptr;  // C_out or u_out
  // adjoint
  const float* u_fwd = nullptr;
  int n_u_fwd = 0;
  const double *stf_re = nullptr, *stf_im = nullptr;
  int64_t stf_dims[3] = {0, 0, 0};
  double* Kout = nullptr;
  double *sf_re = nullptr, *sf_im = nullptr;
  double* seis = nullptr;
};

// A prepared time loop: `loop` only launches work on ctx->stream (capturable).
struct LoopPlan {
  std::string name;
  uint64_t key = 0;
  std::function<fd2d_status()> loop;
};

// Runs the loops of several prepared solves as parallel branches of one cached
// CUDA graph (fork/join over side streams).
fd2d_status run_parallel(fd2d_ctx* ctx, const char* name, uint64_t key, std::vector<LoopPlan>& plans);

// Precision-specific drivers (solver_fp64.cu / solver_fp32.cu).
// Plans of S lanes a[0..S-1] advanced by one launch per step (S > 1: mode 0, no
// Born term, spectra and seismograms of lane l at constant strides from lane 0's).
fd2d_status fp32_forward1_plan(fd2d_ctx* ctx, const Geometry& g, const SolveArgs* a, int S, LoopPlan& plan);
fd2d_status fp32_correlation_plan(fd2d_ctx* ctx, const Geometry& g, const SolveArgs* a, int S, LoopPlan& plan);
// Solves on grids of different sizes (one configuration each, equal FD order
// and freq_samp, mode 0, no Born term) advanced by one launch per time step.
fd2d_status fp32_multi_forward1_plan(fd2d_ctx* ctx, const std::vector<const Geometry*>& g,
                                     const std::vector<const SolveArgs*>& a, LoopPlan& plan);
fd2d_status fp32_multi_correlation_plan(fd2d_ctx* ctx, const std::vector<const Geometry*>& g,
                                        const std::vector<const SolveArgs*>& a, LoopPlan& plan);
fd2d_status fp64_forward1(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a);
fd2d_status fp64_correlation(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a);
fd2d_status fp64_adjoint(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a);
fd2d_status fp32_forward1(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a);
fd2d_status fp32_correlation(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a);
fd2d_status fp32_adjoint(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a);

}  // namespace fd2d
