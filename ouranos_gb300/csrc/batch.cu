// Many independent problems behind one handle.  No counterpart in the
// reference, which solves one problem per MPI job (src/ouranos.cc:43-209).
//
// A batched Apply does, on the batch's stream:
//   per problem   the scattering source of its slice of x (and the source
//                 expansion when its sweep reads expanded sources),
//   per class     ONE persistent sweep launch over the tasks of all problems of
//                 that class (class = dimension, FE order, fused-moment form),
//                 warps taking (problem, task) pairs in ticket order,
//   per problem   the moment reduction and y = x - phi.
// The edge-word epoch lives in device memory and is advanced by a kernel, the
// tickets are reset by memset nodes, and every pointer is fixed once the
// buffers have been sized, so the whole Apply is captured into a CUDA graph on
// its second use for a given (precision, problem set) and replayed after.
//
// The member handles are used only through this batch: all their sweeps share
// the batch's epoch sequence (a handle's own sweeps number theirs separately,
// and an edge word left by one sequence could carry a tag that the other
// sequence is waiting for).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "internal.h"

using namespace ouranos;

namespace {

constexpr int kMaxClasses = 16;
constexpr int kStatus = kMaxClasses;      // d_ctrl[kStatus]: sticky timeout flag
constexpr int kEpoch = kMaxClasses + 1;   // d_ctrl[kEpoch]: edge-word epoch
constexpr size_t kMaxGraphs = 64;         // captured Apply graphs kept per batch
constexpr size_t kMaxTicketMaps = 256;

struct TicketMap {
  // classes present in the set: (dim, p1, fm), first ticket-map entry, count
  struct Cls { int dim, p1, fm, lpc; long first, count; };
  std::vector<Cls> cls;
  DevBuf d;  // int2 (problem, task) entries of all classes
};

struct GraphEntry {
  int precision = 0;
  bool sources = false;
  std::vector<char> mask;
  int uses = 0;
  cudaGraphExec_t exec = nullptr;
};

}  // namespace

struct ouranos_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev0 = nullptr, ev1 = nullptr;
  std::string err;
  int sms = 0;
  std::vector<ouranos_rt*> rt;
  std::vector<long> off;  // slice offsets in the concatenated layout (count + 1)
  DevBuf d_X, d_Y, d_ctrl;
  // sweep arguments per (precision, with sources): pinned host copies and their
  // device images.  The content for one such pair never changes once the
  // buffers are sized, so a captured copy that replays it, or an eager call
  // that rewrites it before an earlier copy has run, always moves the same bytes.
  DevBuf d_args64[2], d_args32[2];
  SweepArgs<double>* h_args64[2] = {nullptr, nullptr};
  SweepArgs<float>* h_args32[2] = {nullptr, nullptr};
  std::vector<int> fm;                    // fused-moment form per problem
  std::map<std::vector<char>, TicketMap> tmaps;
  std::vector<GraphEntry> graphs;
  bool use_graphs = true;
  int graph_launches = 0;
  double last_ms = 0.0;
  DsaBatchScratch dsa;  // the members' diffusion solves in one launch
};

namespace {

int bfail(ouranos_batch* b, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  b->err = buf;
  return OURANOS_ERR_CUDA;
}
int bbad(ouranos_batch* b, const char* what) {
  b->err = what;
  return OURANOS_ERR_BAD_INPUT;
}
#define BC(expr, what)                                   \
  do {                                                   \
    cudaError_t _e = (expr);                             \
    if (_e != cudaSuccess) return bfail(b, _e, what);    \
  } while (0)
#define BR(expr)                                         \
  do {                                                   \
    int _rc = (expr);                                    \
    if (_rc != OURANOS_OK) return _rc;                   \
  } while (0)

// a member handle's failure, reported through the batch
int member(ouranos_batch* b, int p, int rc) {
  if (rc == OURANOS_OK) return rc;
  char buf[512];
  std::snprintf(buf, sizeof buf, "problem %d: %s", p, b->rt[p]->err.c_str());
  b->err = buf;
  return rc;
}

// Tickets of the problems in `mask`, per class.  Within a class the entries
// are sorted by (task index / task count of its problem, problem), which
// keeps every problem's own level-major order -- all a waiting warp needs --
// and interleaves the problems' wavefronts.
void drop_graphs(ouranos_batch* b);

int ticket_map(ouranos_batch* b, const std::vector<char>& mask, TicketMap** out) {
  auto it = b->tmaps.find(mask);
  if (it != b->tmaps.end()) {
    *out = &it->second;
    return OURANOS_OK;
  }
  if (b->tmaps.size() >= kMaxTicketMaps) {  // graphs hold ticket-map addresses: both go
    BC(cudaStreamSynchronize(b->stream), "ticket maps");
    drop_graphs(b);
    b->tmaps.clear();
  }
  TicketMap tm;
  std::vector<int2> all;
  std::vector<int> done(b->rt.size(), 0);
  for (size_t p = 0; p < b->rt.size(); ++p) {
    if (!mask[p] || done[p]) continue;
    const ouranos_rt* r = b->rt[p];
    const int dim = r->dim, p1 = r->p1, fm = b->fm[p], lpc = r->lpc;
    struct Key { double f; int p, t; };
    std::vector<Key> keys;
    for (size_t q = p; q < b->rt.size(); ++q) {
      const ouranos_rt* s = b->rt[q];
      if (!mask[q] || done[q] || s->dim != dim || s->p1 != p1 || b->fm[q] != fm || s->lpc != lpc) continue;
      done[q] = 1;
      for (int t = 0; t < s->n_tasks; ++t) keys.push_back({(double)t / s->n_tasks, (int)q, t});
    }
    std::sort(keys.begin(), keys.end(), [](const Key& x, const Key& y) {
      return x.f != y.f ? x.f < y.f : (x.p != y.p ? x.p < y.p : x.t < y.t);
    });
    if ((int)tm.cls.size() == kMaxClasses) return bbad(b, "too many problem classes in one batch");
    tm.cls.push_back({dim, p1, fm, lpc, (long)all.size(), (long)keys.size()});
    for (const Key& k : keys) all.push_back(make_int2(k.p, k.t));
  }
  BC(tm.d.alloc(sizeof(int2) * std::max<size_t>(all.size(), 1)), "ticket map");
  BC(cudaMemcpy(tm.d.p, all.data(), sizeof(int2) * all.size(), cudaMemcpyHostToDevice), "ticket map");
  auto res = b->tmaps.emplace(mask, std::move(tm));
  *out = &res.first->second;
  return OURANOS_OK;
}

// Enqueue one batched Apply of the problems in `mask` (no synchronisation):
// y = x - D L^-1 M2D S x per slice, or with sources, y = D L^-1 (q + inflow).
template <typename real>
int apply_body(ouranos_batch* b, const std::vector<char>& mask, bool sources, TicketMap* tm) {
  const bool f64 = sizeof(real) == 8;
  SweepArgs<real>* h_args =
      (SweepArgs<real>*)(f64 ? (void*)b->h_args64[sources] : (void*)b->h_args32[sources]);
  DevBuf& d_args = f64 ? b->d_args64[sources] : b->d_args32[sources];
  const double* X = b->d_X.as<double>();
  double* Y = b->d_Y.as<double>();
  int* ctrl = b->d_ctrl.as<int>();
  for (size_t p = 0; p < b->rt.size(); ++p) {
    if (!mask[p]) continue;
    int fm = 0;
    BR(member(b, (int)p, rt_batch_prepare(b->rt[p], sources ? nullptr : X + b->off[p], &h_args[p], &fm,
                                          sources)));
    if (fm != b->fm[p]) return bbad(b, "fused-moment form changed");
    h_args[p].ticket = ctrl;
    h_args[p].status = ctrl + kStatus;
  }
  BC(cudaMemcpyAsync(d_args.p, h_args, sizeof(SweepArgs<real>) * b->rt.size(), cudaMemcpyHostToDevice,
                     b->stream),
     "sweep arguments");
  BC(launch_bump_epoch((unsigned*)(ctrl + kEpoch), b->stream), "epoch");
  BC(cudaMemsetAsync(ctrl, 0, sizeof(int) * kMaxClasses, b->stream), "tickets");
  // while capturing, external records: in the graph they stay timing records
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  BC(cudaStreamIsCapturing(b->stream, &cap), "capture status");
  const unsigned rec = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
  BC(cudaEventRecordWithFlags(b->ev0, b->stream, rec), "event");
  for (size_t c = 0; c < tm->cls.size(); ++c) {
    const TicketMap::Cls& k = tm->cls[c];
    const int grid = (int)std::min<long>((k.count + 3) / 4, (long)std::max(1, b->sms * 8));
    BC(launch_sweep_batch<real>(k.dim, k.p1, k.fm, k.lpc, d_args.as<SweepArgs<real>>(),
                                tm->d.as<int2>() + k.first, (int)k.count, ctrl + c, ctrl + kStatus,
                                (const unsigned*)(ctrl + kEpoch), grid, 128, b->stream),
       "batched sweep");
  }
  BC(cudaEventRecordWithFlags(b->ev1, b->stream, rec), "event");
  for (size_t p = 0; p < b->rt.size(); ++p) {
    if (!mask[p]) continue;
    BR(member(b, (int)p, rt_batch_finish(b->rt[p], sources ? nullptr : X + b->off[p], Y + b->off[p], sources)));
  }
  return OURANOS_OK;
}

int apply_any(ouranos_batch* b, int precision, const std::vector<char>& mask, bool sources, TicketMap* tm) {
  return precision == OURANOS_FP64 ? apply_body<double>(b, mask, sources, tm)
                                   : apply_body<float>(b, mask, sources, tm);
}

// One batched Apply of d_X into d_Y: eager on the first use of a (precision,
// sources, set), captured into a graph on the second and replayed after.
int batched_apply(ouranos_batch* b, int precision, const std::vector<char>& mask, bool sources) {
  TicketMap* tm = nullptr;
  BR(ticket_map(b, mask, &tm));
  if (!b->use_graphs) return apply_any(b, precision, mask, sources, tm);
  GraphEntry* g = nullptr;
  for (GraphEntry& e : b->graphs)
    if (e.precision == precision && e.sources == sources && e.mask == mask) g = &e;
  if (!g) {
    if (b->graphs.size() >= kMaxGraphs) {  // oldest first
      BC(cudaStreamSynchronize(b->stream), "graphs");
      if (b->graphs.front().exec) cudaGraphExecDestroy(b->graphs.front().exec);
      b->graphs.erase(b->graphs.begin());
    }
    b->graphs.push_back(GraphEntry{precision, sources, mask, 0, nullptr});
    g = &b->graphs.back();
  }
  if (g->exec) {
    BC(cudaGraphLaunch(g->exec, b->stream), "graph launch");
    ++b->graph_launches;
    return OURANOS_OK;
  }
  if (g->uses++ == 0) return apply_any(b, precision, mask, sources, tm);  // sizes every buffer
  cudaGraph_t graph = nullptr;
  BC(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
  const int rc = apply_any(b, precision, mask, sources, tm);
  const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
  if (rc != OURANOS_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  BC(ec, "graph capture");
  const cudaError_t ei = cudaGraphInstantiate(&g->exec, graph, 0);
  cudaGraphDestroy(graph);
  BC(ei, "graph instantiate");
  BC(cudaGraphLaunch(g->exec, b->stream), "graph launch");
  ++b->graph_launches;
  return OURANOS_OK;
}

void drop_graphs(ouranos_batch* b) {
  for (GraphEntry& e : b->graphs)
    if (e.exec) cudaGraphExecDestroy(e.exec);
  b->graphs.clear();
}

// the caller's earlier work on the legacy default stream comes first
int order_after_caller(ouranos_batch* b) {
  BC(cudaEventRecord(b->ev_in, cudaStreamLegacy), "order");
  BC(cudaStreamWaitEvent(b->stream, b->ev_in, 0), "order");
  BC(cudaMemsetAsync(b->d_ctrl.as<int>() + kStatus, 0, sizeof(int), b->stream), "status");
  return OURANOS_OK;
}

int check_status(ouranos_batch* b) {
  BC(cudaStreamSynchronize(b->stream), "batch");
  int st = 0;
  BC(cudaMemcpy(&st, b->d_ctrl.as<int>() + kStatus, sizeof(int), cudaMemcpyDeviceToHost), "status");
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, b->ev0, b->ev1) == cudaSuccess) b->last_ms = ms;
  else cudaGetLastError();  // not recorded yet: leave no error for the next launch check
  if (st) {
    b->err = (st & 2) ? "diffusion acceleration: grid barrier wait timed out" : "sweep dependency wait timed out";
    return OURANOS_ERR_TIMEOUT;
  }
  return OURANOS_OK;
}

std::vector<char> all_of(const ouranos_batch* b) { return std::vector<char>(b->rt.size(), 1); }

}  // namespace

namespace {

bool is_device(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

long total_len(const ouranos_batch* b) { return b->off.back(); }

int copy_in(ouranos_batch* b, const double* x) {
  BC(cudaMemcpyAsync(b->d_X.p, x, sizeof(double) * total_len(b),
                     is_device(x) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream),
     "copy in");
  return OURANOS_OK;
}
int copy_out(ouranos_batch* b, double* y) {
  BC(cudaMemcpyAsync(y, b->d_Y.p, sizeof(double) * total_len(b),
                     is_device(y) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->stream),
     "copy out");
  return OURANOS_OK;
}

// Size every buffer the batched Apply touches (FP64 first: the angular flux
// and expanded-source buffers are shared by both precisions and must reach
// their FP64 size before any graph holds their addresses).
int size_buffers(ouranos_batch* b) {
  BC(cudaMemsetAsync(b->d_X.p, 0, sizeof(double) * total_len(b), b->stream), "zero");
  const std::vector<char> all = all_of(b);
  TicketMap* tm = nullptr;
  BR(ticket_map(b, all, &tm));
  BR(apply_any(b, OURANOS_FP64, all, true, tm));
  BR(apply_any(b, OURANOS_FP64, all, false, tm));
  BR(apply_any(b, OURANOS_FP32, all, false, tm));
  return check_status(b);
}

// process-wide cache of tuned tilings: (dim, p1, directions, cells, precision) -> tiling
std::mutex g_tune_mutex;
std::map<std::vector<long>, std::vector<int>> g_tune_cache;

}  // namespace

extern "C" {

int ouranos_batch_create(const ouranos_problem_desc* descs, int count, int device, ouranos_batch** out) {
  if (!out) return OURANOS_ERR_BAD_INPUT;
  *out = nullptr;
  if (!descs || count < 1) return OURANOS_ERR_BAD_INPUT;
  ouranos_batch* b = new ouranos_batch();
  *out = b;  // kept on failure so the caller can read the message; it must destroy it
  for (int p = 0; p < count; ++p) {
    ouranos_rt* r = nullptr;
    const int rc = ouranos_rt_create(&descs[p], device, &r);
    if (rc != OURANOS_OK) {
      char buf[512];
      std::snprintf(buf, sizeof buf, "problem %d: %s", p, r ? r->err.c_str() : "creation failed");
      b->err = buf;
      if (r) ouranos_rt_destroy(r);
      return rc;
    }
    b->rt.push_back(r);
    if (r->lpc == 32) {
      char buf[256];
      std::snprintf(buf, sizeof buf,
                    "problem %d: the batched launch covers the per-lane sweep orders (2-D Q1..Q4, 3-D Q1..Q2)", p);
      b->err = buf;
      return OURANOS_ERR_UNSUPPORTED;
    }
  }
  b->device = b->rt[0]->device;
  for (ouranos_rt* r : b->rt)
    if (r->device != b->device) return bbad(b, "all problems of a batch must be on one device");
  cudaSetDevice(b->device);
  BC(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
  BC(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming), "event");
  BC(cudaEventCreate(&b->ev0), "event");
  BC(cudaEventCreate(&b->ev1), "event");
  BC(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device), "device query");
  b->off.assign(1, 0);
  for (ouranos_rt* r : b->rt) {
    BR(ouranos_rt_set_stream(r, b->stream));
    b->off.push_back(b->off.back() + (long)r->n_mom * r->n_dofs);
  }
  BC(b->d_X.alloc(sizeof(double) * total_len(b)), "batch vectors");
  BC(b->d_Y.alloc(sizeof(double) * total_len(b)), "batch vectors");
  BC(b->d_ctrl.alloc(sizeof(int) * (kMaxClasses + 8)), "batch control");
  BC(cudaMemset(b->d_ctrl.p, 0, sizeof(int) * (kMaxClasses + 8)), "batch control");
  for (int s = 0; s < 2; ++s) {
    BC(cudaMallocHost((void**)&b->h_args64[s], sizeof(SweepArgs<double>) * count), "pinned arguments");
    BC(cudaMallocHost((void**)&b->h_args32[s], sizeof(SweepArgs<float>) * count), "pinned arguments");
    BC(b->d_args64[s].alloc(sizeof(SweepArgs<double>) * count), "arguments");
    BC(b->d_args32[s].alloc(sizeof(SweepArgs<float>) * count), "arguments");
  }
  // edge words start unwritten (epoch 0), whatever the handles did before
  for (ouranos_rt* r : b->rt) {
    BC(cudaMemsetAsync(r->d_edge_x.p, 0, r->d_edge_x.bytes, b->stream), "edge buffers");
    if (r->d_edge_y.p) BC(cudaMemsetAsync(r->d_edge_y.p, 0, r->d_edge_y.bytes, b->stream), "edge buffers");
  }
  // the sweep form of each problem, from a preparation on zeros
  BC(cudaMemsetAsync(b->d_X.p, 0, sizeof(double) * total_len(b), b->stream), "zero");
  b->fm.assign(count, 0);
  for (int p = 0; p < count; ++p)
    BR(member(b, p, rt_batch_prepare(b->rt[p], b->d_X.as<double>() + b->off[p], &b->h_args64[0][p], &b->fm[p],
                                     false)));
  return size_buffers(b);
}

int ouranos_batch_destroy(ouranos_batch* b) {
  if (!b) return OURANOS_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  b->tmaps.clear();
  for (ouranos_rt* r : b->rt) {
    ouranos_rt_set_stream(r, nullptr);
    ouranos_rt_destroy(r);
  }
  for (int s = 0; s < 2; ++s) {
    if (b->h_args64[s]) cudaFreeHost(b->h_args64[s]);
    if (b->h_args32[s]) cudaFreeHost(b->h_args32[s]);
  }
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return OURANOS_OK;
}

int ouranos_batch_layout(const ouranos_batch* b, int* count, long* total_length, long* offsets) {
  if (!b) return OURANOS_ERR_BAD_INPUT;
  if (count) *count = (int)b->rt.size();
  if (total_length) *total_length = total_len(b);
  if (offsets)
    for (size_t p = 0; p < b->off.size(); ++p) offsets[p] = b->off[p];
  return OURANOS_OK;
}

int ouranos_batch_apply(ouranos_batch* b, int precision, const double* x, double* y) {
  if (!b || !x || !y) return OURANOS_ERR_BAD_INPUT;
  if (precision != OURANOS_FP64 && precision != OURANOS_FP32) return bbad(b, "unknown precision");
  cudaSetDevice(b->device);
  BR(order_after_caller(b));
  BR(copy_in(b, x));
  BR(batched_apply(b, precision, all_of(b), false));
  BR(copy_out(b, y));
  return check_status(b);
}

int ouranos_batch_rhs(ouranos_batch* b, double* rhs) {
  if (!b || !rhs) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(b->device);
  BR(order_after_caller(b));
  BR(batched_apply(b, OURANOS_FP64, all_of(b), true));
  BR(copy_out(b, rhs));
  return check_status(b);
}

int ouranos_batch_set_graphs(ouranos_batch* b, int enable) {
  if (!b) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(b->device);
  BC(cudaStreamSynchronize(b->stream), "graphs");
  if (!enable) drop_graphs(b);
  b->use_graphs = enable != 0;
  return OURANOS_OK;
}

int ouranos_batch_stats(const ouranos_batch* b, double* last_sweep_ms, int* graph_launches) {
  if (!b) return OURANOS_ERR_BAD_INPUT;
  if (last_sweep_ms) *last_sweep_ms = b->last_ms;
  if (graph_launches) *graph_launches = b->graph_launches;
  return OURANOS_OK;
}

int ouranos_batch_last_error(const ouranos_batch* b, char* buf, size_t len) {
  if (!b || !buf || !len) return OURANOS_ERR_BAD_INPUT;
  std::snprintf(buf, len, "%s", b->err.c_str());
  return OURANOS_OK;
}

// Per problem, time each tiling whose lanes cover one warp (2-D: 32x1 cells
// by 1 direction down to 4x1 by 8; 3-D: 8x4 x 1 down to 2x2 x 8; for cells of
// 9 or more dofs also two lanes per cell, 16 cells per warp) on its own
// sweep kernel in `precision`, keep the fastest.  Results are cached per
// (dim, order, directions, cells, precision) for the process.  tiling_out
// (may be NULL) receives count x 3 ints.
int ouranos_batch_autotune(ouranos_batch* b, int precision, int reps, int* tiling_out) {
  if (!b) return OURANOS_ERR_BAD_INPUT;
  if (precision != OURANOS_FP64 && precision != OURANOS_FP32) return bbad(b, "unknown precision");
  cudaSetDevice(b->device);
  BC(cudaStreamSynchronize(b->stream), "autotune");
  reps = std::max(1, std::min(reps, 20));
  drop_graphs(b);
  b->tmaps.clear();
  DevBuf tx, ty;
  for (size_t p = 0; p < b->rt.size(); ++p) {
    ouranos_rt* r = b->rt[p];
    const std::vector<long> key = {r->dim, r->p1, r->n_dir, r->nx[0], r->nx[1], r->nx[2], precision};
    std::vector<int> best;
    {
      std::lock_guard<std::mutex> lk(g_tune_mutex);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) best = it->second;
    }
    if (best.empty()) {
      std::vector<std::vector<int>> cand;
      if (r->dim == 2) cand = {{32, 1, 1}, {16, 1, 2}, {8, 1, 4}, {4, 1, 8}};
      else cand = {{8, 4, 1}, {4, 4, 2}, {4, 2, 4}, {2, 2, 8}};
      if (r->n >= 9) {  // two lanes per cell
        if (r->dim == 2) cand.insert(cand.end(), {{16, 1, 1}, {8, 1, 2}, {4, 1, 4}});
        else cand.insert(cand.end(), {{4, 4, 1}, {4, 2, 2}, {2, 2, 4}});
      }
      const long len = (long)r->n_mom * r->n_dofs;
      BC(tx.alloc(sizeof(double) * len), "autotune");
      BC(ty.alloc(sizeof(double) * len), "autotune");
      BC(cudaMemsetAsync(tx.p, 0, sizeof(double) * len, b->stream), "autotune");
      double best_ms = 1e30;
      for (const auto& c : cand) {
        BR(member(b, (int)p, ouranos_rt_set_tiling(r, c[0], c[1], c[2])));
        r->precision = precision;
        double t = 1e30;
        for (int k = 0; k <= reps; ++k) {  // first run warms up
          BR(member(b, (int)p, rt_apply_device(r, tx.as<double>(), ty.as<double>())));
          BR(member(b, (int)p, rt_check_status(r)));
          if (k) t = std::min(t, r->last_ms);
        }
        if (t < best_ms) {
          best_ms = t;
          best = c;
        }
      }
      std::lock_guard<std::mutex> lk(g_tune_mutex);
      g_tune_cache[key] = best;
    }
    // rebuilding the schedule also clears the edge buffers of the single-
    // problem sweeps timed above
    BR(member(b, (int)p, ouranos_rt_set_tiling(r, best[0], best[1], best[2])));
    if (tiling_out)
      for (int k = 0; k < 3; ++k) tiling_out[3 * p + k] = best[k];
  }
  return size_buffers(b);
}

}  // extern "C"

// ------------------------------------------------------------ batched solve
namespace {

// One problem's restarted GMRES inside the batched solve.  Its Krylov basis,
// right-hand side and solution live in one device block; the Gram-Schmidt
// coefficients stay on the device (the axpy reads them there) and reach the
// host through a pinned block, once per step for all problems together.
struct Solve {
  enum { kIter, kRestart, kDone };
  long len = 0;
  int m = 0, k = 0, phase = kDone, total = 0, cycles = 0;
  double bnorm = 0, rel = 0;
  bool converged = false;
  DevBuf mem;
  double *B = nullptr, *Xs = nullptr, *dres = nullptr, *partial = nullptr, *ycoef = nullptr;
  double** dptrs = nullptr;  // [0, m] basis V, [32, 32 + m) the preconditioned Z (flexible form)
  std::vector<double*> V, Z;
  bool flexible = false;
  double* hb = nullptr;  // pinned: [0,32) pass 1, [32,64) pass 2, [64] |w|^2, [65] |r|^2, [66,98) y
  Givens gv{1};
};

int solve_setup(ouranos_batch* b, Solve& S, long len, int m, bool flexible) {
  S.len = len;
  S.m = m;
  S.flexible = flexible;
  const size_t vb = sizeof(double) * (size_t)len;
  const size_t nvec = (size_t)m + 3 + (flexible ? (size_t)m : 0);  // V[0..m], B, Xs (, Z[0..m))
  const size_t extra = sizeof(double*) * 64 + sizeof(double) * (64 + 64 * (size_t)kDotGrid + 64) + 256;
  BC(S.mem.alloc(vb * nvec + extra), "solver workspace");
  char* p = (char*)S.mem.p;
  S.V.resize(m + 1);
  for (int j = 0; j <= m; ++j) S.V[j] = (double*)(p + vb * j);
  S.B = (double*)(p + vb * (m + 1));
  S.Xs = (double*)(p + vb * (m + 2));
  S.Z.assign(flexible ? m : 0, nullptr);
  for (int j = 0; j < (int)S.Z.size(); ++j) S.Z[j] = (double*)(p + vb * (m + 3 + j));
  p += vb * nvec;
  S.dptrs = (double**)p;
  p += sizeof(double*) * 64;
  S.dres = (double*)p;
  S.partial = S.dres + 64;
  S.ycoef = S.partial + 64 * (size_t)kDotGrid;
  BC(cudaMemcpyAsync(S.dptrs, S.V.data(), sizeof(double*) * (m + 1), cudaMemcpyHostToDevice, b->stream),
     "solver workspace");
  if (flexible)
    BC(cudaMemcpyAsync(S.dptrs + 32, S.Z.data(), sizeof(double*) * m, cudaMemcpyHostToDevice, b->stream),
       "solver workspace");
  BC(cudaMemsetAsync(S.Xs, 0, vb, b->stream), "solver workspace");
  BC(cudaMallocHost((void**)&S.hb, sizeof(double) * 128), "pinned solver block");
  return OURANOS_OK;
}

// |v|^2 of S.V[j] into dres[0] and host slot hb[slot]; then v /= |v| on the device
int norm_and_scale(ouranos_batch* b, Solve& S, int j, int slot) {
  BC(launch_dots((const double* const*)(S.dptrs + j), S.V[j], 1, S.len, S.dres, S.partial, b->stream),
     "norm");
  BC(cudaMemcpyAsync(S.hb + slot, S.dres, sizeof(double), cudaMemcpyDeviceToHost, b->stream), "norm");
  BC(launch_scale_inv_norm(S.dres, S.V[j], S.len, b->stream), "normalise");
  return OURANOS_OK;
}

// V[k+1] -= sum_j h_j V[j], j <= k, twice; the two passes' h to hb[0..] and hb[32..]
int gram_schmidt(ouranos_batch* b, Solve& S) {
  const int n = S.k + 1;
  for (int pass = 0; pass < 2; ++pass) {
    BC(launch_dots((const double* const*)S.dptrs, S.V[S.k + 1], n, S.len, S.dres, S.partial, b->stream),
       "orthogonalise");
    BC(cudaMemcpyAsync(S.hb + 32 * pass, S.dres, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream),
       "orthogonalise");
    BC(launch_multi_axpy((const double* const*)S.dptrs, n, S.dres, -1.0, S.V[S.k + 1], S.len, b->stream),
       "orthogonalise");
  }
  return norm_and_scale(b, S, S.k + 1, 64);
}

int batch_solve(ouranos_batch* b, int inner, bool dsa, int m, int max_it, double tol, std::vector<Solve>& S) {
  const int P = (int)b->rt.size();
  const double drop = inner == OURANOS_FP32 ? 1e-5 : 0.0;  // FP32 operator accuracy
  double* X = b->d_X.as<double>();
  double* Y = b->d_Y.as<double>();
  // right-hand sides (FP64) and their norms; x = 0 so r = b
  BR(batched_apply(b, OURANOS_FP64, all_of(b), true));
  for (int p = 0; p < P; ++p) {
    BR(solve_setup(b, S[p], b->off[p + 1] - b->off[p], m, dsa));
    BC(cudaMemcpyAsync(S[p].B, Y + b->off[p], sizeof(double) * S[p].len, cudaMemcpyDeviceToDevice, b->stream),
       "rhs");
    BC(cudaMemcpyAsync(S[p].V[0], S[p].B, sizeof(double) * S[p].len, cudaMemcpyDeviceToDevice, b->stream),
       "rhs");
    BR(norm_and_scale(b, S[p], 0, 65));
  }
  BR(check_status(b));
  for (Solve& s : S) {
    s.bnorm = std::sqrt(std::max(s.hb[65], 0.0));
    s.rel = s.bnorm > 0 ? 1.0 : 0.0;
    s.converged = s.bnorm == 0.0;
    s.phase = s.converged ? Solve::kDone : Solve::kIter;
    if (!s.converged) {
      s.gv = Givens(m);
      s.gv.g[0] = s.bnorm;
      s.cycles = 1;
    }
  }
  std::vector<char> mi(P), mr(P);
  for (;;) {
    bool any_i = false, any_r = false;
    for (int p = 0; p < P; ++p) {
      mi[p] = S[p].phase == Solve::kIter;
      mr[p] = S[p].phase == Solve::kRestart;
      any_i |= mi[p] != 0;
      any_r |= mr[p] != 0;
    }
    if (!any_i && !any_r) break;
    if (any_i) {  // one Arnoldi step: w = A v_k (or A P v_k) in the inner precision, orthogonalised
      if (dsa) {  // z_k = P v_k: every iterating member's diffusion correction, one launch
        std::vector<ouranos_rt*> rts;
        std::vector<const double*> vin;
        std::vector<double*> zout;
        for (int p = 0; p < P; ++p)
          if (mi[p]) {
            rts.push_back(b->rt[p]);
            vin.push_back(S[p].V[S[p].k]);
            zout.push_back(S[p].Z[S[p].k]);
          }
        const int rc = rt_dsa_apply_batch(rts.data(), vin.data(), zout.data(), (int)rts.size(), b->stream,
                                          b->d_ctrl.as<int>() + kStatus, b->dsa, b->err);
        if (rc) return rc;
      }
      for (int p = 0; p < P; ++p)
        if (mi[p]) {
          const double* in = dsa ? S[p].Z[S[p].k] : S[p].V[S[p].k];
          BC(cudaMemcpyAsync(X + b->off[p], in, sizeof(double) * S[p].len, cudaMemcpyDeviceToDevice, b->stream),
             "arnoldi");
        }
      BR(batched_apply(b, inner, mi, false));
      for (int p = 0; p < P; ++p)
        if (mi[p]) {
          BC(cudaMemcpyAsync(S[p].V[S[p].k + 1], Y + b->off[p], sizeof(double) * S[p].len,
                             cudaMemcpyDeviceToDevice, b->stream),
             "arnoldi");
          BR(gram_schmidt(b, S[p]));
        }
    }
    if (any_r) {  // true residual r = b - A x in FP64 starts the next cycle
      for (int p = 0; p < P; ++p)
        if (mr[p])
          BC(cudaMemcpyAsync(X + b->off[p], S[p].Xs, sizeof(double) * S[p].len, cudaMemcpyDeviceToDevice,
                             b->stream),
             "restart");
      BR(batched_apply(b, OURANOS_FP64, mr, false));
      for (int p = 0; p < P; ++p)
        if (mr[p]) {
          BC(launch_axpby(1.0, S[p].B, -1.0, Y + b->off[p], S[p].len, b->stream), "restart");
          BC(cudaMemcpyAsync(S[p].V[0], Y + b->off[p], sizeof(double) * S[p].len, cudaMemcpyDeviceToDevice,
                             b->stream),
             "restart");
          BR(norm_and_scale(b, S[p], 0, 65));
        }
    }
    BR(check_status(b));  // the step's one synchronisation
    for (int p = 0; p < P; ++p) {
      Solve& s = S[p];
      if (mi[p]) {
        std::vector<double> col(s.k + 2);
        for (int j = 0; j <= s.k; ++j) col[j] = s.hb[j] + s.hb[32 + j];
        col[s.k + 1] = std::sqrt(std::max(s.hb[64], 0.0));
        const double est = s.gv.add_column(s.k, col.data()) / s.bnorm;
        ++s.total;
        ++s.k;
        if (est < tol || est < s.rel * drop || s.k == s.m || col[s.k] == 0.0 || s.total >= max_it) {
          // x += V y: the cycle's correction; the true residual decides what next
          const std::vector<double> y = s.gv.solve(s.k);
          std::memcpy(s.hb + 66, y.data(), sizeof(double) * s.k);
          BC(cudaMemcpyAsync(s.ycoef, s.hb + 66, sizeof(double) * s.k, cudaMemcpyHostToDevice, b->stream),
             "update");
          BC(launch_multi_axpy((const double* const*)(s.flexible ? s.dptrs + 32 : s.dptrs), s.k, s.ycoef, 1.0,
                               s.Xs, s.len, b->stream),
             "update");
          s.phase = Solve::kRestart;
        }
      } else if (mr[p]) {
        s.rel = std::sqrt(std::max(s.hb[65], 0.0)) / s.bnorm;
        if (s.rel < tol || s.total >= max_it) {
          s.converged = s.rel < tol;
          s.phase = Solve::kDone;
        } else {
          s.gv = Givens(m);
          s.gv.g[0] = s.rel * s.bnorm;
          s.k = 0;
          ++s.cycles;
          s.phase = Solve::kIter;
        }
      }
    }
  }
  // solutions into d_Y in the concatenated layout
  for (int p = 0; p < P; ++p)
    BC(cudaMemcpyAsync(Y + b->off[p], S[p].Xs, sizeof(double) * S[p].len, cudaMemcpyDeviceToDevice, b->stream),
       "solution");
  return OURANOS_OK;
}

}  // namespace

extern "C" {

// Diffusion synthetic acceleration for every problem of the batch (the
// members' ouranos_rt_set_dsa): used by ouranos_batch_solve with
// OURANOS_SOLVER_DSA OR'ed into `inner`.
int ouranos_batch_set_dsa(ouranos_batch* b, int cg_iterations) {
  if (!b) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(b->device);
  for (size_t p = 0; p < b->rt.size(); ++p) BR(member(b, (int)p, ouranos_rt_set_dsa(b->rt[p], cg_iterations)));
  return OURANOS_OK;
}

// z = P x for every member (concatenated layout, host or device): each
// member's diffusion correction, all in one cooperative launch
int ouranos_batch_dsa_apply(ouranos_batch* b, const double* x, double* z) {
  if (!b || !x || !z) return OURANOS_ERR_BAD_INPUT;
  for (ouranos_rt* r : b->rt)
    if (r->dsa_iters < 1) return bbad(b, "diffusion acceleration is off (ouranos_batch_set_dsa)");
  cudaSetDevice(b->device);
  BR(order_after_caller(b));
  BR(copy_in(b, x));
  const int P = (int)b->rt.size();
  std::vector<const double*> vin(P);
  std::vector<double*> zout(P);
  for (int p = 0; p < P; ++p) {
    vin[p] = b->d_X.as<double>() + b->off[p];
    zout[p] = b->d_Y.as<double>() + b->off[p];
  }
  const int rc = rt_dsa_apply_batch(b->rt.data(), vin.data(), zout.data(), P, b->stream,
                                    b->d_ctrl.as<int>() + kStatus, b->dsa, b->err);
  if (rc) return rc;
  BR(copy_out(b, z));
  return check_status(b);
}

// Restarted GMRES on every problem of the batch at once (right-hand side from
// each problem's fixed source and inflow): inner = OURANOS_FP32 for FP32
// Arnoldi sweeps with FP64 restarts (a cycle also ends once its estimate has
// dropped 1e-5 below the cycle's start), OURANOS_FP64 for the plain method;
// with OURANOS_SOLVER_DSA OR'ed in, FGMRES with each problem's diffusion
// correction as the right preconditioner (x += Z y).
// x (concatenated, host or device) receives the solutions, info[count] the
// per-problem results; seconds is the batch's wall time.
int ouranos_batch_solve(ouranos_batch* b, int inner, int restart, int max_it, double tol, double* x,
                        ouranos_solve_info* info) {
  if (!b || !x || !info || max_it < 1 || !(tol > 0)) return OURANOS_ERR_BAD_INPUT;
  const bool dsa = (inner & OURANOS_SOLVER_DSA) != 0;
  inner &= ~OURANOS_SOLVER_DSA;
  if (inner != OURANOS_FP64 && inner != OURANOS_FP32) return bbad(b, "unknown inner precision");
  if (dsa)
    for (ouranos_rt* r : b->rt)
      if (r->dsa_iters < 1) return bbad(b, "diffusion acceleration is off (ouranos_batch_set_dsa)");
  cudaSetDevice(b->device);
  const auto t0 = std::chrono::steady_clock::now();
  BR(order_after_caller(b));
  const int m = std::max(1, std::min(restart, 30));
  std::vector<Solve> S(b->rt.size());
  int rc = batch_solve(b, inner, dsa, m, max_it, tol, S);
  if (rc == OURANOS_OK) rc = copy_out(b, x);
  if (rc == OURANOS_OK) rc = check_status(b);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (size_t p = 0; p < S.size(); ++p) {
    info[p].iterations = S[p].total;
    info[p].restarts = S[p].cycles;
    info[p].residual = S[p].rel;
    info[p].seconds = secs;
    info[p].converged = S[p].converged ? 1 : 0;
    if (S[p].hb) cudaFreeHost(S[p].hb);
  }
  if (rc != OURANOS_OK) return rc;
  for (const Solve& s : S)
    if (!s.converged) return OURANOS_ERR_NOT_CONVERGED;
  return OURANOS_OK;
}

}  // extern "C"
