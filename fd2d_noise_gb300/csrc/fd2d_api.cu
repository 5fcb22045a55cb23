// fd2d_api.cu -- the C ABI of libfd2d (include/fd2d.h): contexts, argument
// validation, host<->device staging and dispatch to the FP64 / FP32 drivers.
//
// Validation mirrors what the MATLAB solvers would reject (an index past the end
// of an array, mismatched reshape sizes) so callers get an error code where the
// reference raises a MATLAB error.
#include "common.cuh"

#include <cstring>

#include <algorithm>
#include <mutex>

namespace fd2d {

static std::mutex g_err_mu;
static std::string g_global_err;

fd2d_status set_error(fd2d_ctx* ctx, fd2d_status s, const std::string& msg) {
  if (ctx) {
    ctx->last_error = msg;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_global_err = msg;
  }
  return s;
}

// Workspace buffers come from the device's stream-ordered memory pool
// (cudaMallocAsync / cudaFreeAsync on the context's stream): no implicit
// device-wide synchronisation, so contexts working concurrently on other
// streams are not stalled when one of them grows or releases its buffers.
fd2d_status workspace(fd2d_ctx* ctx, const char* name_in, size_t bytes, void** out) {
  const std::string key = ctx->ws_prefix + name_in;
  const char* name = key.c_str();
  for (auto& kv : ctx->bufs) {
    if (kv.first == name) {
      if (kv.second.bytes >= bytes) {
        *out = kv.second.ptr;
        return FD2D_OK;
      }
      // grow: stream-ordered, after the work already queued that uses the old buffer
      cudaFreeAsync(kv.second.ptr, ctx->stream);
      kv.second.ptr = nullptr;
      kv.second.bytes = 0;
      cudaError_t e = cudaMallocAsync(&kv.second.ptr, bytes, ctx->stream);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(ctx, FD2D_ERR_OOM, std::string("cudaMalloc(") + name + ", " +
                                                std::to_string(bytes) + " B): " + cudaGetErrorString(e));
      }
      kv.second.bytes = bytes;
      kv.second.tag = 0;
      *out = kv.second.ptr;
      return FD2D_OK;
    }
  }
  DevBuf b;
  cudaError_t e = cudaMallocAsync(&b.ptr, bytes, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(ctx, FD2D_ERR_OOM, std::string("cudaMalloc(") + name + ", " +
                                            std::to_string(bytes) + " B): " + cudaGetErrorString(e));
  }
  b.bytes = bytes;
  ctx->bufs.emplace_back(name, b);
  *out = b.ptr;
  return FD2D_OK;
}

fd2d_status workspace_tag(fd2d_ctx* ctx, const char* name, size_t bytes, uint64_t tag, void** out, bool* hit) {
  FD2D_TRY(workspace(ctx, name, bytes, out));
  const std::string key = ctx->ws_prefix + name;
  *hit = false;
  for (auto& kv : ctx->bufs)
    if (kv.first == key) {
      *hit = kv.second.tag == tag && tag != 0;
      kv.second.tag = tag;
    }
  return FD2D_OK;
}

void free_workspace(fd2d_ctx* ctx) {
  for (auto& kv : ctx->bufs) cudaFreeAsync(kv.second.ptr, ctx->stream);
  ctx->bufs.clear();
}

fd2d_status after_launch(fd2d_ctx* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ctx, FD2D_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  ++ctx->launches;
  return FD2D_OK;
}

static int next_event(fd2d_ctx* ctx) {
  if (ctx->ev_used == ctx->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    ctx->ev_pool.push_back(e);
  }
  return (int)ctx->ev_used++;
}

// Inside a capture, timing events become external event-record nodes of the
// graph and are owned by its cache entry.
static int capture_event(fd2d_ctx* ctx, cudaStream_t stream) {
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return -1;
  if (cudaEventRecordWithFlags(e, stream, cudaEventRecordExternal) != cudaSuccess) {
    cudaEventDestroy(e);
    return -1;
  }
  ctx->cap_ev.push_back(e);
  return (int)ctx->cap_ev.size() - 1;
}

int timer_begin(fd2d_ctx* ctx, cudaStream_t stream) {
  if (!ctx->timing) return -1;
  if (ctx->capturing) return capture_event(ctx, stream);
  int i = next_event(ctx);
  if (i >= 0) cudaEventRecord(ctx->ev_pool[i], stream);
  return i;
}

void timer_end(fd2d_ctx* ctx, cudaStream_t stream, int begin, int cls, int64_t units, int64_t count) {
  if (!ctx->timing || begin < 0) return;
  if (ctx->capturing) {
    int i = capture_event(ctx, stream);
    if (i >= 0) ctx->cap_recs.push_back({begin, i, cls, units, count});
    return;
  }
  int i = next_event(ctx);
  if (i < 0) return;
  cudaEventRecord(ctx->ev_pool[i], stream);
  ctx->recs.push_back({begin, i, cls, units, count});
}

static fd2d_ctx::GraphEntry* find_graph(fd2d_ctx* ctx, const char* name) {
  for (auto& kv : ctx->graphs)
    if (kv.first == name) return &kv.second;
  return nullptr;
}

static void destroy_graph(fd2d_ctx::GraphEntry& g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  for (auto e : g.ev) cudaEventDestroy(e);
  g = fd2d_ctx::GraphEntry();
}

static fd2d_status launch_graph(fd2d_ctx* ctx, fd2d_ctx::GraphEntry& g) {
  FD2D_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
  ctx->launches += g.launches;
  if (ctx->timing && !g.recs.empty()) {
    // the graph's event nodes are reused by the next replay: read them now
    FD2D_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (const auto& r : g.recs) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, g.ev[r.a], g.ev[r.b]) == cudaSuccess) {
        ctx->t_ms[r.cls] += t;
        ctx->t_cnt[r.cls] += r.count;
        ctx->t_units[r.cls] += r.units;
      }
    }
    cudaGetLastError();
  }
  return FD2D_OK;
}

static thread_local int64_t g_launches_at_capture = 0;

fd2d_status graph_begin(fd2d_ctx* ctx, const char* name, uint64_t key, bool* replayed, bool* eager) {
  *replayed = false;
  *eager = false;
  key ^= ctx->timing ? 0x9e3779b97f4a7c15ull : 0;
  fd2d_ctx::GraphEntry* g = find_graph(ctx, name);
  if (g && g->exec && g->key == key) {
    *replayed = true;
    return launch_graph(ctx, *g);
  }
  // A loop seen for the first time is launched eagerly: capture and
  // instantiation cost more host time than one run (serving requests of ever
  // new shapes run once each).  The second run with the same key captures the
  // graph, later ones replay it.
  if (!g) {
    ctx->graphs.emplace_back(name, fd2d_ctx::GraphEntry());
    g = &ctx->graphs.back().second;
  }
  if (g->seen != key) {
    g->seen = key;
    *eager = true;
    return FD2D_OK;
  }
  ctx->cap_ev.clear();
  ctx->cap_recs.clear();
  g_launches_at_capture = ctx->launches;
  FD2D_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  ctx->capturing = true;
  return FD2D_OK;
}

fd2d_status graph_end(fd2d_ctx* ctx, const char* name, uint64_t key, fd2d_status body_status) {
  key ^= ctx->timing ? 0x9e3779b97f4a7c15ull : 0;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  ctx->capturing = false;
  const int64_t n_kernels = ctx->launches - g_launches_at_capture;
  ctx->launches = g_launches_at_capture;
  auto drop_events = [&]() {
    for (auto ev : ctx->cap_ev) cudaEventDestroy(ev);
    ctx->cap_ev.clear();
    ctx->cap_recs.clear();
  };
  if (body_status != FD2D_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    drop_events();
    cudaGetLastError();
    if (body_status != FD2D_OK) return body_status;
    return set_error(ctx, FD2D_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
  }
  fd2d_ctx::GraphEntry* g = find_graph(ctx, name);
  if (!g) {
    ctx->graphs.emplace_back(name, fd2d_ctx::GraphEntry());
    g = &ctx->graphs.back().second;
  }
  bool updated = false;
  if (g->exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(g->exec, graph, &info) == cudaSuccess) updated = true;
    cudaGetLastError();
  }
  if (!updated) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    g->exec = nullptr;
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      drop_events();
      g->exec = nullptr;
      return set_error(ctx, FD2D_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
  }
  cudaGraphDestroy(graph);
  for (auto ev : g->ev) cudaEventDestroy(ev);
  g->ev = ctx->cap_ev;
  g->recs = ctx->cap_recs;
  ctx->cap_ev.clear();
  ctx->cap_recs.clear();
  g->key = key;
  g->launches = n_kernels;
  return launch_graph(ctx, *g);
}

fd2d_status run_parallel(fd2d_ctx* ctx, const char* name, uint64_t key, std::vector<LoopPlan>& plans) {
  // At most MAX_BRANCHES loops per graph, graphs one after the other (each
  // cached under its own name): on GB300 a 32-solve batch of uneven grids ran
  // 3.6x slower as one 32-branch graph than as four graphs of 8 branches
  // (2.2 s vs 0.61 s).
  constexpr size_t MAX_BRANCHES = 8;
  if (plans.size() > MAX_BRANCHES) {
    for (size_t i = 0; i < plans.size(); i += MAX_BRANCHES) {
      std::vector<LoopPlan> part(plans.begin() + i, plans.begin() + std::min(plans.size(), i + MAX_BRANCHES));
      const std::string part_name = std::string(name) + "#" + std::to_string(i / MAX_BRANCHES);
      FD2D_TRY(run_parallel(ctx, part_name.c_str(), key, part));
    }
    return FD2D_OK;
  }
  Sig sg;
  sg.add(key);
  for (const auto& p : plans) sg.add(p.key);
  // side streams and fork/join events exist before the capture starts
  while (ctx->side_streams.size() < plans.size()) {
    cudaStream_t s;
    FD2D_CUDA(ctx, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    ctx->side_streams.push_back(s);
  }
  while (ctx->fork_events.size() < plans.size() + 1) {
    cudaEvent_t e;
    FD2D_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->fork_events.push_back(e);
  }
  bool replayed = false, eager = false;
  FD2D_TRY(graph_begin(ctx, name, sg.h, &replayed, &eager));
  if (replayed) return FD2D_OK;
  cudaStream_t main = ctx->stream;
  fd2d_status st = FD2D_OK;
  cudaEventRecord(ctx->fork_events[0], main);
  for (size_t j = 0; j < plans.size() && st == FD2D_OK; ++j) {
    cudaStream_t sj = ctx->side_streams[j];
    cudaStreamWaitEvent(sj, ctx->fork_events[0], 0);
    ctx->stream = sj;
    st = plans[j].loop();
    ctx->stream = main;
    cudaEventRecord(ctx->fork_events[j + 1], sj);
    cudaStreamWaitEvent(main, ctx->fork_events[j + 1], 0);
  }
  ctx->stream = main;
  if (eager) return st;
  return graph_end(ctx, name, sg.h, st);
}

fd2d_status stage_in(fd2d_ctx* ctx, const char* name, const void* src, size_t bytes, const void** dev) {
  if (!src || bytes == 0) {
    *dev = nullptr;
    return FD2D_OK;
  }
  if (ctx->memspace == FD2D_MEM_DEVICE) {
    *dev = src;
    return FD2D_OK;
  }
  void* d = nullptr;
  FD2D_TRY(workspace(ctx, name, bytes, &d));
  FD2D_CUDA(ctx, cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  *dev = d;
  return FD2D_OK;
}

fd2d_status out_buffer(fd2d_ctx* ctx, const char* name, void* user, size_t bytes, void** dev) {
  if (!user || bytes == 0) {
    *dev = nullptr;
    return FD2D_OK;
  }
  if (ctx->memspace == FD2D_MEM_DEVICE) {
    *dev = user;
    return FD2D_OK;
  }
  return workspace(ctx, name, bytes, dev);
}

fd2d_status stage_out(fd2d_ctx* ctx, void* user, const void* dev, size_t bytes) {
  if (!user || !dev || bytes == 0 || ctx->memspace == FD2D_MEM_DEVICE) return FD2D_OK;
  FD2D_CUDA(ctx, cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return FD2D_OK;
}

fd2d_status finish_call(fd2d_ctx* ctx) {
  if (ctx->memspace == FD2D_MEM_HOST) FD2D_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int herr = 0;
  if (ctx->memspace == FD2D_MEM_HOST && ctx->d_err) {
    FD2D_CUDA(ctx, cudaMemcpy(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
      cudaMemset(ctx->d_err, 0, sizeof(int));
      return set_error(ctx, FD2D_ERR_TIMEOUT, "a bounded device-side wait gave up (code " + std::to_string(herr) + ")");
    }
  }
  return FD2D_OK;
}

static fd2d_status point_indices(fd2d_ctx* ctx, const Geometry& g, const double* pts_host, int n,
                                 const char* what, std::vector<int>& idx) {
  idx.resize(n);
  if (n == 0) return FD2D_OK;
  if (!pts_host) return set_error(ctx, FD2D_ERR_ARG, std::string(what) + " is NULL");
  for (int i = 0; i < n; ++i) {
    int ix = nearest_node(g.x, pts_host[i]);
    int iz = nearest_node(g.z, pts_host[n + i]);
    idx[i] = ix + g.nx * iz;
  }
  return FD2D_OK;
}

// Positions (src, rec) are small: read them on the host in either memspace.
static fd2d_status host_points(fd2d_ctx* ctx, const double* p, int n, std::vector<double>& out) {
  out.assign((size_t)2 * n, 0.0);
  if (n == 0 || !p) return FD2D_OK;
  if (ctx->memspace == FD2D_MEM_DEVICE) {
    FD2D_CUDA(ctx, cudaMemcpyAsync(out.data(), p, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, ctx->stream));
    FD2D_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } else {
    std::memcpy(out.data(), p, sizeof(double) * 2 * n);
  }
  return FD2D_OK;
}

fd2d_status check_ctx(fd2d_ctx* ctx) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return set_error(ctx, FD2D_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  ctx->last_error.clear();
  return FD2D_OK;
}

}  // namespace fd2d

using namespace fd2d;

extern "C" {

int32_t fd2d_abi_version(void) { return FD2D_ABI_VERSION; }

fd2d_status fd2d_ctx_create(int32_t device, int32_t precision, fd2d_ctx** out) {
  if (!out) return set_error(nullptr, FD2D_ERR_ARG, "out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return set_error(nullptr, FD2D_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  if (device < 0 || device >= n) return set_error(nullptr, FD2D_ERR_ARG, "device index out of range");
  if (precision != FD2D_PREC_FP64 && precision != FD2D_PREC_FP32)
    return set_error(nullptr, FD2D_ERR_ARG, "precision must be FD2D_PREC_FP64 or FD2D_PREC_FP32");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return set_error(nullptr, FD2D_ERR_CUDA, cudaGetErrorString(e));
  {
    // keep freed workspace in the device's pool for reuse by any context
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  fd2d_ctx* c = new fd2d_ctx();
  c->device = device;
  c->precision = precision;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(int));
  if (e != cudaSuccess) {
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return set_error(nullptr, FD2D_ERR_CUDA, cudaGetErrorString(e));
  }
  c->own_stream = true;
  *out = c;
  return FD2D_OK;
}

fd2d_status fd2d_ctx_destroy(fd2d_ctx* ctx) {
  if (!ctx) return FD2D_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->graphs) destroy_graph(kv.second);
  ctx->graphs.clear();
  for (auto s : ctx->side_streams) cudaStreamDestroy(s);
  for (auto e : ctx->fork_events) cudaEventDestroy(e);
  free_workspace(ctx);
  cudaStreamSynchronize(ctx->stream);
  for (auto e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FD2D_OK;
}

fd2d_status fd2d_device_free_bytes(int32_t device, int64_t* free_bytes, int64_t* total_bytes) {
  if (!free_bytes) return set_error(nullptr, FD2D_ERR_ARG, "free_bytes is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return set_error(nullptr, FD2D_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  if (device < 0 || device >= n) return set_error(nullptr, FD2D_ERR_ARG, "device index out of range");
  int prev = 0;
  cudaGetDevice(&prev);
  FD2D_CUDA(nullptr, cudaSetDevice(device));
  size_t f = 0, t = 0;
  e = cudaMemGetInfo(&f, &t);
  if (e == cudaSuccess) {
    cudaMemPool_t pool;
    uint64_t reserved = 0, used = 0;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
      f += (size_t)(reserved - used);
    cudaGetLastError();
  }
  cudaSetDevice(prev);
  if (e != cudaSuccess) return set_error(nullptr, FD2D_ERR_CUDA, std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
  *free_bytes = (int64_t)f;
  if (total_bytes) *total_bytes = (int64_t)t;
  return FD2D_OK;
}

fd2d_status fd2d_ctx_release(fd2d_ctx* ctx, int64_t* bytes) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  FD2D_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t b = 0;
  for (const auto& kv : ctx->bufs) b += (int64_t)kv.second.bytes;
  if (bytes) *bytes = b;
  for (auto& kv : ctx->graphs) destroy_graph(kv.second);
  ctx->graphs.clear();
  free_workspace(ctx);
  return FD2D_OK;
}

int64_t fd2d_ctx_workspace_bytes(const fd2d_ctx* ctx) {
  if (!ctx) return 0;
  int64_t b = 0;
  for (const auto& kv : ctx->bufs) b += (int64_t)kv.second.bytes;
  return b;
}

fd2d_status fd2d_ctx_set_stream(fd2d_ctx* ctx, void* stream) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  // workspace is stream-ordered on the current stream: drain it before switching
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (stream) {
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = (cudaStream_t)stream;
    ctx->own_stream = false;
  } else if (!ctx->own_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return set_error(ctx, FD2D_ERR_CUDA, cudaGetErrorString(e));
    ctx->own_stream = true;
  }
  return FD2D_OK;
}

fd2d_status fd2d_ctx_set_memspace(fd2d_ctx* ctx, int32_t memspace) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  if (memspace != FD2D_MEM_HOST && memspace != FD2D_MEM_DEVICE)
    return set_error(ctx, FD2D_ERR_ARG, "memspace must be FD2D_MEM_HOST or FD2D_MEM_DEVICE");
  ctx->memspace = memspace;
  return FD2D_OK;
}

fd2d_status fd2d_ctx_set_precision(fd2d_ctx* ctx, int32_t precision) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  if (precision != FD2D_PREC_FP64 && precision != FD2D_PREC_FP32)
    return set_error(ctx, FD2D_ERR_ARG, "precision must be FD2D_PREC_FP64 or FD2D_PREC_FP32");
  ctx->precision = precision;
  return FD2D_OK;
}

fd2d_status fd2d_ctx_synchronize(fd2d_ctx* ctx) {
  FD2D_TRY(check_ctx(ctx));
  FD2D_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int herr = 0;
  FD2D_CUDA(ctx, cudaMemcpy(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) {
    cudaMemset(ctx->d_err, 0, sizeof(int));
    return set_error(ctx, FD2D_ERR_TIMEOUT, "a bounded device-side wait gave up (code " + std::to_string(herr) + ")");
  }
  return FD2D_OK;
}

fd2d_status fd2d_ctx_set_timing(fd2d_ctx* ctx, int32_t enable) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  ctx->timing = enable != 0;
  return FD2D_OK;
}

fd2d_status fd2d_ctx_timing(fd2d_ctx* ctx, double* ms, int64_t* launches, int64_t* units) {
  FD2D_TRY(check_ctx(ctx));
  FD2D_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (const auto& r : ctx->recs) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, ctx->ev_pool[r.a], ctx->ev_pool[r.b]) == cudaSuccess) {
      ctx->t_ms[r.cls] += t;
      ctx->t_cnt[r.cls] += r.count;
      ctx->t_units[r.cls] += r.units;
    }
  }
  cudaGetLastError();
  ctx->recs.clear();
  ctx->ev_used = 0;
  for (int c = 0; c < FD2D_TIMER_COUNT; ++c) {
    if (ms) ms[c] = ctx->t_ms[c];
    if (launches) launches[c] = ctx->t_cnt[c];
    if (units) units[c] = ctx->t_units[c];
    ctx->t_ms[c] = 0;
    ctx->t_cnt[c] = 0;
    ctx->t_units[c] = 0;
  }
  return FD2D_OK;
}

int64_t fd2d_ctx_kernel_launches(const fd2d_ctx* ctx) { return ctx ? ctx->launches : 0; }

const char* fd2d_last_error(const fd2d_ctx* ctx) {
  if (ctx) return ctx->last_error.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  thread_local std::string copy;
  copy = g_global_err;
  return copy.c_str();
}

fd2d_status fd2d_query_sizes(const fd2d_config* cfg, int32_t nr, fd2d_sizes* out) {
  if (!out) return set_error(nullptr, FD2D_ERR_ARG, "out is NULL");
  if (nr < 0) return set_error(nullptr, FD2D_ERR_ARG, "nr < 0");
  Geometry g;
  std::string err;
  fd2d_status s = make_geometry(cfg, g, err);
  if (s != FD2D_OK) return set_error(nullptr, s, err);
  const int64_t np = g.npts();
  int nfw = 0;
  for (int n = g.nt; n <= 2 * g.nt - 1; ++n) nfw += (n % g.fw == 0);
  out->ntc = g.ntc;
  out->n_fw_green = nfw;
  out->n_fw_corr = g.ntc / g.fw;
  out->n_kernel_planes = g.nb == 0 ? 2 : g.nb + 1;
  out->npts = np;
  out->G_fft = np * g.K;
  out->G_out = np * nfw;
  out->seis_green = (int64_t)nr * g.nt;
  out->C_out = np * out->n_fw_corr;
  out->seis_corr = (int64_t)nr * g.ntc;
  out->K = np * out->n_kernel_planes;
  return FD2D_OK;
}

fd2d_status fd2d_forward1_green(fd2d_ctx* ctx, const fd2d_config* cfg, const double* mu,
                                const double* rho, const double* src, int32_t ns,
                                const double* rec, int32_t nr, int32_t mode, const double* dmu,
                                const float* G_in, int32_t n_G_in, double* G_fft_re,
                                double* G_fft_im, float* G_out, double* seismograms) {
  FD2D_TRY(check_ctx(ctx));
  Geometry g;
  std::string err;
  fd2d_status s = make_geometry(cfg, g, err);
  if (s != FD2D_OK) return set_error(ctx, s, err);
  if (!mu || !rho) return set_error(ctx, FD2D_ERR_ARG, "mu and rho are required");
  if (ns < 0 || nr < 0 || n_G_in < 0) return set_error(ctx, FD2D_ERR_ARG, "negative count");
  if (!G_fft_re || !G_fft_im) return set_error(ctx, FD2D_ERR_ARG, "G_fft output planes are required");
  if (nr > 0 && !seismograms) return set_error(ctx, FD2D_ERR_ARG, "seismograms output is required");
  int nfw = 0;
  for (int n = g.nt; n <= 2 * g.nt - 1; ++n) nfw += (n % g.fw == 0);
  if (mode != 0 && nfw > 0 && !G_out) return set_error(ctx, FD2D_ERR_ARG, "G_out output is required when mode != 0");
  if (dmu && (!G_in || n_G_in < g.nt))
    return set_error(ctx, FD2D_ERR_INDEX, "Born run needs G_in with at least nt snapshots (G_in(:,:,i_fw_in) for i_fw_in = 1..nt)");
  const size_t np = (size_t)g.npts();
  SolveArgs a;
  a.mode = mode;
  std::vector<double> hp;
  FD2D_TRY(host_points(ctx, src, ns, hp));
  FD2D_TRY(point_indices(ctx, g, hp.data(), ns, "src", a.src_idx));
  FD2D_TRY(host_points(ctx, rec, nr, hp));
  FD2D_TRY(point_indices(ctx, g, hp.data(), nr, "rec", a.rec_idx));
  const void* p;
  FD2D_TRY(stage_in(ctx, "in.mu", mu, np * 8, &p)); a.mu = (const double*)p;
  FD2D_TRY(stage_in(ctx, "in.rho", rho, np * 8, &p)); a.rho = (const double*)p;
  FD2D_TRY(stage_in(ctx, "in.dmu", dmu, dmu ? np * 8 : 0, &p)); a.dmu = (const double*)p;
  if (dmu) {
    FD2D_TRY(stage_in(ctx, "in.G_in", G_in, np * 4 * (size_t)g.nt, &p));
    a.G_in = (const float*)p;
    a.n_G_in = g.nt;
  }
  void* q;
  FD2D_TRY(out_buffer(ctx, "out.G_re", G_fft_re, np * 8 * g.K, &q)); a.G_re = (double*)q;
  FD2D_TRY(out_buffer(ctx, "out.G_im", G_fft_im, np * 8 * g.K, &q)); a.G_im = (double*)q;
  if (mode != 0 && nfw > 0) {
    FD2D_TRY(out_buffer(ctx, "out.G_out", G_out, np * 4 * nfw, &q));
    a.G_out = (float*)q;
  }
  FD2D_TRY(out_buffer(ctx, "out.seis", seismograms, (size_t)nr * g.nt * 8, &q)); a.seis = (double*)q;
  s = ctx->precision == FD2D_PREC_FP64 ? fp64_forward1(ctx, g, a) : fp32_forward1(ctx, g, a);
  if (s != FD2D_OK) return s;
  FD2D_TRY(stage_out(ctx, G_fft_re, a.G_re, np * 8 * g.K));
  FD2D_TRY(stage_out(ctx, G_fft_im, a.G_im, np * 8 * g.K));
  if (a.G_out) FD2D_TRY(stage_out(ctx, G_out, a.G_out, np * 4 * nfw));
  FD2D_TRY(stage_out(ctx, seismograms, a.seis, (size_t)nr * g.nt * 8));
  return finish_call(ctx);
}

fd2d_status fd2d_forward2_correlation(fd2d_ctx* ctx, const fd2d_config* cfg, const double* mu,
                                      const double* rho, const double* G_fft_re,
                                      const double* G_fft_im, int32_t n_G, const double* spectrum,
                                      int32_t n_noise_sources, const double* source_dist,
                                      int32_t n_dist, const double* rec, int32_t nr, int32_t mode,
                                      const double* dmu, const float* C_in, int32_t n_C_in,
                                      double* seismograms, float* C_out) {
  FD2D_TRY(check_ctx(ctx));
  Geometry g;
  std::string err;
  fd2d_status s = make_geometry(cfg, g, err);
  if (s != FD2D_OK) return set_error(ctx, s, err);
  if (!mu || !rho) return set_error(ctx, FD2D_ERR_ARG, "mu and rho are required");
  if (nr < 0 || n_G < 0 || n_C_in < 0 || n_dist < 0) return set_error(ctx, FD2D_ERR_ARG, "negative count");
  if (!G_fft_re || !G_fft_im) return set_error(ctx, FD2D_ERR_ARG, "G_fft is required");
  if (n_G < g.K) return set_error(ctx, FD2D_ERR_INDEX, "G_fft has fewer than n_sample planes");
  if (!spectrum || n_noise_sources < 1) return set_error(ctx, FD2D_ERR_ARG, "spectrum is required");
  if (g.nb == 0 && n_noise_sources != 1)
    return set_error(ctx, FD2D_ERR_SHAPE, "with n_basis_fct == 0 the reference handles one noise source (interpol_matrix * distribution needs one plane)");
  if (!source_dist || n_dist != (g.nb == 0 ? n_noise_sources : g.nb))
    return set_error(ctx, FD2D_ERR_SHAPE, "source_dist must have n_noise_sources (n_basis_fct == 0) or n_basis_fct planes");
  if (nr > 0 && !seismograms) return set_error(ctx, FD2D_ERR_ARG, "seismograms output is required");
  const int nfw = g.ntc / g.fw;
  if (mode != 0 && nfw > 0 && !C_out) return set_error(ctx, FD2D_ERR_ARG, "C_out output is required when mode != 0");
  if (dmu && (!C_in || n_C_in < g.ntc))
    return set_error(ctx, FD2D_ERR_INDEX, "Born run needs C_in with 2*nt-1 snapshots (C_in(:,:,n+1))");
  const size_t np = (size_t)g.npts();
  SolveArgs a;
  a.mode = mode;
  std::vector<double> hp;
  FD2D_TRY(host_points(ctx, rec, nr, hp));
  FD2D_TRY(point_indices(ctx, g, hp.data(), nr, "rec", a.rec_idx));
  const void* p;
  FD2D_TRY(stage_in(ctx, "in.mu", mu, np * 8, &p)); a.mu = (const double*)p;
  FD2D_TRY(stage_in(ctx, "in.rho", rho, np * 8, &p)); a.rho = (const double*)p;
  FD2D_TRY(stage_in(ctx, "in.dmu", dmu, dmu ? np * 8 : 0, &p)); a.dmu = (const double*)p;
  FD2D_TRY(stage_in(ctx, "in.G_re", G_fft_re, np * 8 * g.K, &p)); a.Gin_re = (const double*)p;
  FD2D_TRY(stage_in(ctx, "in.G_im", G_fft_im, np * 8 * g.K, &p)); a.Gin_im = (const double*)p;
  a.n_G = g.K;
  FD2D_TRY(stage_in(ctx, "in.spectrum", spectrum, (size_t)g.K * n_noise_sources * 8, &p));
  a.spectrum = (const double*)p;
  a.n_src = n_noise_sources;
  FD2D_TRY(stage_in(ctx, "in.source_dist", source_dist, np * 8 * n_dist, &p));
  a.source_dist = (const double*)p;
  a.n_dist = n_dist;
  if (dmu) {
    FD2D_TRY(stage_in(ctx, "in.C_in", C_in, np * 4 * (size_t)g.ntc, &p));
    a.C_in = (const float*)p;
    a.n_C_in = g.ntc;
  }
  // The host copy of spectrum is needed by both drivers (effective spectrum per k).
  void* q;
  if (mode != 0 && nfw > 0) {
    FD2D_TRY(out_buffer(ctx, "out.C_out", C_out, np * 4 * nfw, &q));
    a.C_out = (float*)q;
  }
  FD2D_TRY(out_buffer(ctx, "out.seis", seismograms, (size_t)nr * g.ntc * 8, &q)); a.seis = (double*)q;
  s = ctx->precision == FD2D_PREC_FP64 ? fp64_correlation(ctx, g, a) : fp32_correlation(ctx, g, a);
  if (s != FD2D_OK) return s;
  if (a.C_out) FD2D_TRY(stage_out(ctx, C_out, a.C_out, np * 4 * nfw));
  FD2D_TRY(stage_out(ctx, seismograms, a.seis, (size_t)nr * g.ntc * 8));
  return finish_call(ctx);
}

fd2d_status fd2d_noise_adjoint(fd2d_ctx* ctx, const fd2d_config* cfg, const double* mu,
                               const double* rho, const float* u_fwd, int32_t n_u_fwd,
                               const double* stf_re, const double* stf_im,
                               const int64_t stf_dims[3], const double* src, int32_t ns,
                               const double* rec, int32_t nr, const double* spectrum,
                               int32_t n_noise_sources, const double* source_dist, int32_t n_dist,
                               const double* G_fft_re, const double* G_fft_im, int32_t n_G,
                               int32_t mode, const double* dmu, const float* u_in, int32_t n_u_in,
                               double* K, double* stf_fft_re, double* stf_fft_im, float* u_out,
                               double* seismograms) {
  FD2D_TRY(check_ctx(ctx));
  Geometry g;
  std::string err;
  fd2d_status s = make_geometry(cfg, g, err);
  if (s != FD2D_OK) return set_error(ctx, s, err);
  if (!mu || !rho) return set_error(ctx, FD2D_ERR_ARG, "mu and rho are required");
  if (ns < 0 || nr < 0 || n_G < 0 || n_u_in < 0 || n_u_fwd < 0 || n_dist < 0 || n_noise_sources < 0)
    return set_error(ctx, FD2D_ERR_ARG, "negative count");
  if (!(mode == 0 || mode == 1 || mode == 10 || mode == 11 || mode == 12 || mode == 13))
    return set_error(ctx, FD2D_ERR_ARG, "mode must be 0, 1, 10, 11, 12 or 13");
  if (!K || !stf_fft_re || !stf_fft_im) return set_error(ctx, FD2D_ERR_ARG, "K and stf_fft outputs are required");
  if (nr > 0 && !seismograms) return set_error(ctx, FD2D_ERR_ARG, "seismograms output is required");
  const size_t np = (size_t)g.npts();
  const int nfw = g.ntc / g.fw;
  const bool save_u = mode == 11 || mode == 13;
  if (save_u && nfw > 0 && !u_out) return set_error(ctx, FD2D_ERR_ARG, "u_out output is required for modes 11 and 13");
  SolveArgs a;
  a.mode = mode;
  int64_t d0 = 0, d1 = 0, d2 = 0;
  if (stf_dims) { d0 = stf_dims[0]; d1 = stf_dims[1]; d2 = stf_dims[2]; }
  if (d0 < 0 || d1 < 0 || d2 < 0) return set_error(ctx, FD2D_ERR_ARG, "negative stf dimension");
  const bool stf_empty = !stf_re || d0 * d1 * d2 == 0;
  const int64_t size3 = stf_empty ? 1 : d2;
  if (!stf_empty) {
    if (size3 == 1) {
      if (d0 < ns) return set_error(ctx, FD2D_ERR_INDEX, "stf has fewer rows than adjoint sources");
      int nt_loop = g.ntc;
      if (d1 < nt_loop && ns > 0) return set_error(ctx, FD2D_ERR_INDEX, "stf has fewer columns than time steps");
    } else {
      if (d0 != g.nx || d1 != g.nz) return set_error(ctx, FD2D_ERR_SHAPE, "field stf must be nx-by-nz-by-n_sample");
      if (d2 < g.K) return set_error(ctx, FD2D_ERR_INDEX, "field stf has fewer than n_sample planes");
    }
  }
  const bool have_dist = source_dist && n_dist > 0;
  if (have_dist) {
    if (!spectrum || n_noise_sources < 1) return set_error(ctx, FD2D_ERR_SHAPE, "source_dist needs a spectrum");
    if (g.nb == 0 && n_noise_sources != 1)
      return set_error(ctx, FD2D_ERR_SHAPE, "with n_basis_fct == 0 the reference handles one noise source");
    if (n_dist != (g.nb == 0 ? n_noise_sources : g.nb))
      return set_error(ctx, FD2D_ERR_SHAPE, "source_dist must have n_noise_sources (n_basis_fct == 0) or n_basis_fct planes");
  }
  const bool Gvalid = G_fft_re && n_G == g.K;
  if (Gvalid && (!G_fft_im || !spectrum || n_noise_sources != 1))
    return set_error(ctx, FD2D_ERR_SHAPE, "the source kernel needs G_fft planes and a one-column spectrum");
  // i_ftc is shared by the field-source injection and the stf_fft DFT
  // (code/run_noise_adjoint.m:265,343): both active overruns the table.
  if (!stf_empty && size3 != 1 && (mode == 1 || mode == 12 || mode == 13)) {
    int nt_loop = (mode == 1) ? g.nt : g.ntc;
    int steps = nt_loop / g.fs;
    if (2 * steps > g.ntc / g.fs)
      return set_error(ctx, FD2D_ERR_INDEX, "field source together with stf_fft (modes 1/12/13) overruns fft_coeff, as in the reference");
  }
  std::vector<double> hp;
  FD2D_TRY(host_points(ctx, src, ns, hp));
  FD2D_TRY(point_indices(ctx, g, hp.data(), ns, "src", a.src_idx));
  FD2D_TRY(host_points(ctx, rec, nr, hp));
  FD2D_TRY(point_indices(ctx, g, hp.data(), nr, "rec", a.rec_idx));
  const void* p;
  FD2D_TRY(stage_in(ctx, "in.mu", mu, np * 8, &p)); a.mu = (const double*)p;
  FD2D_TRY(stage_in(ctx, "in.rho", rho, np * 8, &p)); a.rho = (const double*)p;
  const bool born = dmu && u_in && n_u_in == g.ntc;
  if (born) {
    FD2D_TRY(stage_in(ctx, "in.dmu", dmu, np * 8, &p)); a.dmu = (const double*)p;
    FD2D_TRY(stage_in(ctx, "in.C_in", u_in, np * 4 * (size_t)g.ntc, &p)); a.C_in = (const float*)p;
    a.n_C_in = g.ntc;
  }
  if (u_fwd && n_u_fwd > 0) {
    FD2D_TRY(stage_in(ctx, "in.u_fwd", u_fwd, np * 4 * (size_t)n_u_fwd, &p));
    a.u_fwd = (const float*)p;
    a.n_u_fwd = n_u_fwd;
  }
  if (!stf_empty) {
    a.stf_dims[0] = d0; a.stf_dims[1] = d1; a.stf_dims[2] = d2;
    const size_t n_stf = (size_t)(d0 * d1 * d2);
    FD2D_TRY(stage_in(ctx, "in.stf_re", stf_re, n_stf * 8, &p)); a.stf_re = (const double*)p;
    if (stf_im) { FD2D_TRY(stage_in(ctx, "in.stf_im", stf_im, n_stf * 8, &p)); a.stf_im = (const double*)p; }
  }
  if (spectrum && n_noise_sources > 0) {
    FD2D_TRY(stage_in(ctx, "in.spectrum", spectrum, (size_t)g.K * n_noise_sources * 8, &p));
    a.spectrum = (const double*)p;
    a.n_src = n_noise_sources;
  }
  if (have_dist) {
    FD2D_TRY(stage_in(ctx, "in.source_dist", source_dist, np * 8 * n_dist, &p));
    a.source_dist = (const double*)p;
    a.n_dist = n_dist;
  }
  if (Gvalid) {
    FD2D_TRY(stage_in(ctx, "in.G_re", G_fft_re, np * 8 * g.K, &p)); a.Gin_re = (const double*)p;
    FD2D_TRY(stage_in(ctx, "in.G_im", G_fft_im, np * 8 * g.K, &p)); a.Gin_im = (const double*)p;
    a.n_G = g.K;
  }
  const int nkp = g.nb == 0 ? 2 : g.nb + 1;
  void* q;
  FD2D_TRY(out_buffer(ctx, "out.K", K, np * 8 * nkp, &q)); a.Kout = (double*)q;
  FD2D_TRY(out_buffer(ctx, "out.sf_re", stf_fft_re, np * 8 * g.K, &q)); a.sf_re = (double*)q;
  FD2D_TRY(out_buffer(ctx, "out.sf_im", stf_fft_im, np * 8 * g.K, &q)); a.sf_im = (double*)q;
  if (save_u && nfw > 0) {
    FD2D_TRY(out_buffer(ctx, "out.u_out", u_out, np * 4 * nfw, &q));
    a.C_out = (float*)q;
  }
  FD2D_TRY(out_buffer(ctx, "out.seis", seismograms, (size_t)nr * g.ntc * 8, &q)); a.seis = (double*)q;
  s = ctx->precision == FD2D_PREC_FP64 ? fp64_adjoint(ctx, g, a) : fp32_adjoint(ctx, g, a);
  if (s != FD2D_OK) return s;
  FD2D_TRY(stage_out(ctx, K, a.Kout, np * 8 * nkp));
  FD2D_TRY(stage_out(ctx, stf_fft_re, a.sf_re, np * 8 * g.K));
  FD2D_TRY(stage_out(ctx, stf_fft_im, a.sf_im, np * 8 * g.K));
  if (a.C_out) FD2D_TRY(stage_out(ctx, u_out, a.C_out, np * 4 * nfw));
  FD2D_TRY(stage_out(ctx, seismograms, a.seis, (size_t)nr * g.ntc * 8));
  return finish_call(ctx);
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Batches of reference stations (include/fd2d.h: fd2d_correlation_batch)
// ---------------------------------------------------------------------------------
namespace fd2d {
namespace {

struct BatchJob {
  Geometry g;
  SolveArgs green, corr;
  size_t bytes = 0;
  int nr = 0;
  int lane_group = -1, lane = 0;  // jobs of one geometry and receiver count share launches
  double* corr_lane = nullptr;    // the lane's correlations inside the group buffer
};

// Device bytes one FP32 job holds (fields, snapshot chunk, spectra, P and
// injection planes, staged inputs); the FP64 form needs less.
size_t job_footprint(const Geometry& g, int nr, int n_dist, bool host_inputs) {
  const size_t P = (size_t)(g.nx + 31) / 32 * 32;
  const size_t ps = (P * g.nz + 127) / 128 * 128;
  const size_t np = (size_t)g.npts();
  const size_t plane = ps * 4;
  size_t n_dft = 0;
  for (int n = 1; n <= g.nt; ++n) n_dft += ((n + g.nt - 1) % g.fs == 0);
  const size_t T = std::min<size_t>({n_dft, (size_t)DFT_CHUNK_DEFAULT, ((size_t)2 << 30) / plane});
  const size_t n_inj = g.ntc / g.fs;
  const size_t chunk = std::min<size_t>(n_inj, ((size_t)4 << 30) / plane);
  // fields and coefficients, snapshot chunk and its split image (x2), FP64
  // spectra, P planes and their split image (x2), injection planes
  size_t b = 11 * plane + 3 * T * plane + 16 * np * g.K + 3 * 2 * (size_t)g.K * plane + chunk * plane;
  b += (size_t)nr * (g.nt + g.ntc) * 8 + ((size_t)1 << 20);
  if (host_inputs) b += np * 8 * (2 + n_dist) + (size_t)nr * g.ntc * 8;
  return b;
}

}  // namespace
}  // namespace fd2d

extern "C" int32_t fd2d_ctx_last_batch(const fd2d_ctx* ctx, int32_t* lanes, int32_t cap) {
  if (!ctx) return 0;
  const int32_t n = (int32_t)ctx->last_lanes.size();
  for (int32_t i = 0; i < n && i < cap && lanes; ++i) lanes[i] = ctx->last_lanes[i];
  return n;
}

extern "C" fd2d_status fd2d_ctx_set_chunks(fd2d_ctx* ctx, int32_t max_snapshots, int32_t max_injection_planes) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  if (max_snapshots < 0 || max_injection_planes < 0) return set_error(ctx, FD2D_ERR_ARG, "negative chunk size");
  ctx->max_dft_chunk = max_snapshots;
  ctx->max_inj_chunk = max_injection_planes;
  return FD2D_OK;
}

extern "C" fd2d_status fd2d_ctx_set_tile_rows(fd2d_ctx* ctx, int32_t rows) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  if (rows != FD2D_TILE_ROWS_AUTO && rows != FD2D_TILE_ROWS_RULE && rows != 16 && rows != 30 && rows != 32 &&
      rows != 40)
    return set_error(ctx, FD2D_ERR_ARG,
                     "tile rows must be 16, 30, 32, 40, FD2D_TILE_ROWS_AUTO or FD2D_TILE_ROWS_RULE");
  ctx->tile_rows = rows;
  return FD2D_OK;
}

extern "C" int32_t fd2d_ctx_last_tile_rows(const fd2d_ctx* ctx) { return ctx ? ctx->last_tile_rows : 0; }

extern "C" fd2d_status fd2d_ctx_set_time_depth(fd2d_ctx* ctx, int32_t depth) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  if (depth < 0 || depth > 2) return set_error(ctx, FD2D_ERR_ARG, "time depth must be 0 (timed), 1 or 2");
  ctx->time_depth = depth;
  return FD2D_OK;
}

extern "C" int32_t fd2d_ctx_last_time_depth(const fd2d_ctx* ctx) { return ctx ? ctx->last_time_depth : 0; }

extern "C" fd2d_status fd2d_ctx_set_shared_gpu(fd2d_ctx* ctx, int32_t shared) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  ctx->shared_gpu = shared ? 1 : 0;
  return FD2D_OK;
}

extern "C" fd2d_status fd2d_ctx_set_memory_budget(fd2d_ctx* ctx, int64_t bytes) {
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  if (bytes < 0) return set_error(ctx, FD2D_ERR_ARG, "negative memory budget");
  ctx->mem_budget = bytes;
  return FD2D_OK;
}

extern "C" fd2d_status fd2d_correlation_batch(fd2d_ctx* ctx, const fd2d_job* jobs, int32_t n_jobs) {
  FD2D_TRY(check_ctx(ctx));
  if (n_jobs < 0 || (n_jobs > 0 && !jobs)) return set_error(ctx, FD2D_ERR_ARG, "bad job list");
  std::vector<BatchJob> B(n_jobs);
  for (int j = 0; j < n_jobs; ++j) {
    const fd2d_job& J = jobs[j];
    std::string err;
    fd2d_status s = make_geometry(J.cfg, B[j].g, err);
    if (s != FD2D_OK) return set_error(ctx, s, "job " + std::to_string(j) + ": " + err);
    const Geometry& g = B[j].g;
    if (!J.mu || !J.rho || !J.src || (J.nr > 0 && (!J.rec || !J.correlations)) || J.nr < 0)
      return set_error(ctx, FD2D_ERR_ARG, "job " + std::to_string(j) + ": missing array");
    if (!J.spectrum || J.n_noise_sources < 1 || (g.nb == 0 && J.n_noise_sources != 1))
      return set_error(ctx, FD2D_ERR_SHAPE, "job " + std::to_string(j) + ": spectrum");
    if (!J.source_dist || J.n_dist != (g.nb == 0 ? J.n_noise_sources : g.nb))
      return set_error(ctx, FD2D_ERR_SHAPE, "job " + std::to_string(j) + ": source_dist planes");
    B[j].nr = J.nr;
    B[j].bytes = job_footprint(g, J.nr, J.n_dist, ctx->memspace == FD2D_MEM_HOST);
  }
  size_t budget = (size_t)ctx->mem_budget;
  if (budget == 0) {
    size_t free_b = 0, total_b = 0;
    FD2D_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
    // memory the stream-ordered pool holds but no buffer uses is free for us too
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
      uint64_t reserved = 0, used = 0;
      if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
          cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
        free_b += (size_t)(reserved - used);
    }
    cudaGetLastError();
    // the context's own workspace is reused (or regrown) by this batch: count
    // it as available, so that repeated calls see the same budget and split
    // the batch the same way (a different split regrows the named buffers and
    // recaptures the graphs on every call)
    free_b += (size_t)fd2d_ctx_workspace_bytes(ctx);
    budget = free_b / 10 * 8;
  }
  int j0 = 0;
  fd2d_status st = FD2D_OK;
  ctx->last_lanes.clear();
  while (j0 < n_jobs && st == FD2D_OK) {
    int j1 = j0 + 1;
    size_t used = B[j0].bytes;
    // (at most 64 jobs: the solves of one multi-geometry loop)
    while (j1 < n_jobs && j1 - j0 < 64 && used + B[j1].bytes <= budget) used += B[j1++].bytes;
    // lane groups: jobs of one geometry (configuration) and receiver count
    // advance together, one launch per time step for the whole group
    std::vector<std::vector<int>> lanes;
    if (ctx->precision == FD2D_PREC_FP32) {
      for (int j = j0; j < j1; ++j) {
        int gi = -1;
        for (size_t q = 0; q < lanes.size() && gi < 0; ++q) {
          const BatchJob& h = B[lanes[q][0]];
          if (h.g.key && h.g.key == B[j].g.key && h.nr == B[j].nr) gi = (int)q;
        }
        if (gi < 0) {
          gi = (int)lanes.size();
          lanes.emplace_back();
        }
        B[j].lane_group = gi;
        B[j].lane = (int)lanes[gi].size();
        lanes[gi].push_back(j);
      }
    }
    // Several geometries of one FD order and decimation advance together in
    // one multi-geometry launch per time step (FD2D_BATCH_MULTI=0 runs them as
    // parallel graph branches instead, one launch chain per geometry).
    bool multi = ctx->precision == FD2D_PREC_FP32 && lanes.size() > 1;
    for (int j = j0; j < j1 && multi; ++j)
      multi = B[j].g.r == B[j0].g.r && B[j].g.fs == B[j0].g.fs;
    if (multi) {
      const char* e = std::getenv("FD2D_BATCH_MULTI");
      if (e && std::strcmp(e, "0") == 0) multi = false;
    }
    if (lanes.empty())
      for (int j = j0; j < j1; ++j) ctx->last_lanes.push_back(1);
    if (multi)
      ctx->last_lanes.push_back((int32_t)(j1 - j0));  // one launch group of every job
    else
      for (const auto& l : lanes) ctx->last_lanes.push_back((int32_t)l.size());
    // group buffers: spectra, Green seismograms and correlations of all lanes,
    // lane after lane
    std::vector<double*> grp_gre(lanes.size()), grp_gim(lanes.size()), grp_sg(lanes.size()), grp_c(lanes.size());
    for (size_t q = 0; q < lanes.size() && st == FD2D_OK; ++q) {
      const Geometry& g = B[lanes[q][0]].g;
      const size_t S = lanes[q].size(), np = (size_t)g.npts(), nr = (size_t)std::max(B[lanes[q][0]].nr, 1);
      ctx->ws_prefix = "L" + std::to_string(q) + ":";
      void* w;
      if ((st = workspace(ctx, "batch.G_re", S * np * 8 * g.K, &w)) != FD2D_OK) break;
      grp_gre[q] = (double*)w;
      if ((st = workspace(ctx, "batch.G_im", S * np * 8 * g.K, &w)) != FD2D_OK) break;
      grp_gim[q] = (double*)w;
      if ((st = workspace(ctx, "batch.seis_green", S * nr * g.nt * 8, &w)) != FD2D_OK) break;
      grp_sg[q] = (double*)w;
      if ((st = workspace(ctx, "batch.corr", S * nr * g.ntc * 8, &w)) != FD2D_OK) break;
      grp_c[q] = (double*)w;
    }
    // stage the group's inputs and outputs, each job under its own prefix
    for (int j = j0; j < j1 && st == FD2D_OK; ++j) {
      const fd2d_job& J = jobs[j];
      BatchJob& b = B[j];
      const Geometry& g = b.g;
      const size_t np = (size_t)g.npts();
      ctx->ws_prefix = "b" + std::to_string(j - j0) + ":";
      std::vector<double> hp;
      SolveArgs& ga = b.green;
      SolveArgs& ca = b.corr;
      const void* p;
      void* q;
      if ((st = host_points(ctx, J.src, 1, hp)) != FD2D_OK) break;
      if ((st = point_indices(ctx, g, hp.data(), 1, "src", ga.src_idx)) != FD2D_OK) break;
      if ((st = host_points(ctx, J.rec, J.nr, hp)) != FD2D_OK) break;
      if ((st = point_indices(ctx, g, hp.data(), J.nr, "rec", ga.rec_idx)) != FD2D_OK) break;
      ca.rec_idx = ga.rec_idx;
      if ((st = stage_in(ctx, "in.mu", J.mu, np * 8, &p)) != FD2D_OK) break;
      ga.mu = ca.mu = (const double*)p;
      if ((st = stage_in(ctx, "in.rho", J.rho, np * 8, &p)) != FD2D_OK) break;
      ga.rho = ca.rho = (const double*)p;
      if ((st = stage_in(ctx, "in.spectrum", J.spectrum, (size_t)g.K * J.n_noise_sources * 8, &p)) != FD2D_OK) break;
      ca.spectrum = (const double*)p;
      ca.n_src = J.n_noise_sources;
      if ((st = stage_in(ctx, "in.source_dist", J.source_dist, np * 8 * J.n_dist, &p)) != FD2D_OK) break;
      ca.source_dist = (const double*)p;
      ca.n_dist = J.n_dist;
      ca.n_G = g.K;
      if (b.lane_group >= 0) {
        const int q = b.lane_group;
        const size_t nr = (size_t)std::max(J.nr, 1);
        ga.G_re = grp_gre[q] + (size_t)b.lane * np * g.K;
        ga.G_im = grp_gim[q] + (size_t)b.lane * np * g.K;
        ga.seis = grp_sg[q] + (size_t)b.lane * nr * g.nt;
        ca.seis = b.corr_lane = grp_c[q] + (size_t)b.lane * nr * g.ntc;
      } else {
        if ((st = workspace(ctx, "batch.G_re", np * 8 * g.K, &q)) != FD2D_OK) break;
        ga.G_re = (double*)q;
        if ((st = workspace(ctx, "batch.G_im", np * 8 * g.K, &q)) != FD2D_OK) break;
        ga.G_im = (double*)q;
        if ((st = workspace(ctx, "batch.seis_green", (size_t)std::max(J.nr, 1) * g.nt * 8, &q)) != FD2D_OK) break;
        ga.seis = (double*)q;
        if ((st = out_buffer(ctx, "out.corr", J.correlations, (size_t)J.nr * g.ntc * 8, &q)) != FD2D_OK) break;
        if (!q && (st = workspace(ctx, "batch.corr", 8, &q)) != FD2D_OK) break;
        ca.seis = (double*)q;
      }
      ca.Gin_re = ga.G_re;
      ca.Gin_im = ga.G_im;
    }
    if (st != FD2D_OK) break;
    if (ctx->precision == FD2D_PREC_FP64) {
      for (int j = j0; j < j1 && st == FD2D_OK; ++j) {
        ctx->ws_prefix = "b" + std::to_string(j - j0) + ":";
        st = fp64_forward1(ctx, B[j].g, B[j].green);
        if (st == FD2D_OK) st = fp64_correlation(ctx, B[j].g, B[j].corr);
      }
    } else if (multi) {
      std::vector<const Geometry*> gs;
      std::vector<const SolveArgs*> green, corr;
      for (int j = j0; j < j1; ++j) {
        gs.push_back(&B[j].g);
        green.push_back(&B[j].green);
        corr.push_back(&B[j].corr);
      }
      const std::string part = "@" + std::to_string(j0);
      LoopPlan p;
      ctx->ws_prefix.clear();
      st = fp32_multi_forward1_plan(ctx, gs, green, p);
      if (st == FD2D_OK) st = run_captured(ctx, ("batch_green_multi" + part).c_str(), p.key, p.loop);
      if (st == FD2D_OK) st = fp32_multi_correlation_plan(ctx, gs, corr, p);
      if (st == FD2D_OK) st = run_captured(ctx, ("batch_corr_multi" + part).c_str(), p.key, p.loop);
    } else {
      // one plan per lane group; the groups' loops run as parallel graph branches
      std::vector<LoopPlan> plans(lanes.size());
      ctx->concurrent_groups = (int32_t)lanes.size();
      std::vector<SolveArgs> la;
      for (size_t q = 0; q < lanes.size() && st == FD2D_OK; ++q) {
        ctx->ws_prefix = "L" + std::to_string(q) + ":";
        la.clear();
        for (int j : lanes[q]) la.push_back(B[j].green);
        st = fp32_forward1_plan(ctx, B[lanes[q][0]].g, la.data(), (int)la.size(), plans[q]);
      }
      ctx->ws_prefix.clear();
      // graphs cached per sub-batch (the first job's index), so that a batch
      // split by the memory budget replays every part's graphs
      const std::string part = "@" + std::to_string(j0);
      if (st == FD2D_OK) st = run_parallel(ctx, ("batch_green" + part).c_str(), 0x1u, plans);
      for (size_t q = 0; q < lanes.size() && st == FD2D_OK; ++q) {
        ctx->ws_prefix = "L" + std::to_string(q) + ":";
        la.clear();
        for (int j : lanes[q]) la.push_back(B[j].corr);
        st = fp32_correlation_plan(ctx, B[lanes[q][0]].g, la.data(), (int)la.size(), plans[q]);
      }
      ctx->ws_prefix.clear();
      ctx->concurrent_groups = 0;
      if (st == FD2D_OK) st = run_parallel(ctx, ("batch_corr" + part).c_str(), 0x2u, plans);
    }
    for (int j = j0; j < j1 && st == FD2D_OK; ++j) {
      const size_t bytes = (size_t)jobs[j].nr * B[j].g.ntc * 8;
      if (B[j].corr_lane) {
        if (bytes && jobs[j].correlations)
        {
          const cudaError_t e =
              cudaMemcpyAsync(jobs[j].correlations, B[j].corr_lane, bytes, cudaMemcpyDefault, ctx->stream);
          if (e != cudaSuccess) st = set_error(ctx, FD2D_ERR_CUDA, std::string("copy correlations: ") + cudaGetErrorString(e));
        }
      } else {
        st = stage_out(ctx, jobs[j].correlations, B[j].corr.seis, bytes);
      }
    }
    if (st == FD2D_OK && j1 < n_jobs && ctx->memspace == FD2D_MEM_DEVICE)
      st = FD2D_OK;  // device outputs are already in place
    j0 = j1;
  }
  ctx->ws_prefix.clear();
  ctx->concurrent_groups = 0;
  if (st != FD2D_OK) return st;
  return finish_call(ctx);
}
