// Batched box reconstructions replayed as one CUDA graph (no reference
// counterpart; the reference runs one mock per run! call).
//
// Mocks are grouped by (mesh, box): one context per group, whose buffers and
// cuFFT plans every mock of the group reuses.  At creation the whole batch —
// per mock: paint (CIC or TSC, wrap), Gaussian smoothing with that mock's
// radius, normalisation, n_iter iterative-FFT steps, displacement and the
// shifted positions — is captured once, each group on its own stream forked
// from and joined back into the launch stream, so groups of different mesh
// sizes run concurrently inside the graph.  A launch replays every kernel of
// the batch with one host call; the caller may refill the input arrays (same
// addresses, same counts) between launches.
#include <map>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

struct baorec_batch {
  std::vector<baorec_ctx*> groups;
  std::vector<baorec_batch_item> items;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaEvent_t> events;
  int64_t launches_per_replay = 0;
  char msg[512] = {0};
};

namespace {

int bfail(baorec_batch* b, int code, const char* what) {
  if (b) snprintf(b->msg, sizeof(b->msg), "%s", what);
  return code;
}

#define BK(call)                                                                   \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess) {                                                       \
      cudaGetLastError();                                                          \
      snprintf(b->msg, sizeof(b->msg), "%s: %s", #call, cudaGetErrorString(_e));   \
      return BAOREC_ERR_CUDA;                                                      \
    }                                                                              \
  } while (0)

int check_item(baorec_batch* b, const baorec_batch_item& it, int i) {
  char buf[256];
  if (it.n < 0 || (it.n > 0 && (!it.x || !it.y || !it.z || !it.w)) || !it.out_x || !it.out_y || !it.out_z) {
    snprintf(buf, sizeof(buf), "batch item %d: missing particle or output arrays", i);
    return bfail(b, BAOREC_ERR_ARG, buf);
  }
  if (it.mesh < 4 || it.mesh % 2 || !(it.box_size > 0.0f) || (it.mas != BAOREC_MAS_CIC && it.mas != BAOREC_MAS_TSC) ||
      !(it.smoothing_radius >= 0.0f) || it.field < BAOREC_FIELD_DISP || it.field > BAOREC_FIELD_SUM) {
    snprintf(buf, sizeof(buf), "batch item %d: bad mesh, box, mas, radius or field", i);
    return bfail(b, BAOREC_ERR_ARG, buf);
  }
  return BAOREC_OK;
}

// the captured work of one group, on the group context's stream
int record_group(baorec_batch* b, baorec_ctx* ctx, const std::vector<int>& members) {
  for (int i : members) {
    const baorec_batch_item& it = b->items[i];
    ctx->cfg.mas = it.mas;
    ctx->cfg.smoothing_radius = it.smoothing_radius;
    int st = baorec::reconstruct_iterative_device(ctx, it.x, it.y, it.z, it.w, it.n);
    if (st == BAOREC_OK) st = baorec::positions_device(ctx, it.x, it.y, it.z, it.n, it.field, it.out_x, it.out_y, it.out_z);
    if (st != BAOREC_OK) {
      snprintf(b->msg, sizeof(b->msg), "batch item %d: %s", i, ctx->msg);
      return st;
    }
  }
  return BAOREC_OK;
}

}  // namespace

extern "C" int baorec_batch_create(const baorec_config* base, const baorec_batch_item* items, int count,
                                   baorec_batch** out) {
  if (!base || !items || count <= 0 || !out) return BAOREC_ERR_ARG;
  *out = nullptr;
  baorec_batch* b = new (std::nothrow) baorec_batch();
  if (!b) return BAOREC_ERR_NOMEM;
  *out = b;   // the caller destroys it on failure too, and reads the message
  b->items.assign(items, items + count);
  for (int i = 0; i < count; ++i) CKS(check_item(b, b->items[i], i));
  if (base->method != BAOREC_ITERATIVE) return bfail(b, BAOREC_ERR_ARG, "batch: only the iterative method is batched");
  // group by (mesh, box size)
  std::map<std::pair<int, float>, std::vector<int>> groups;
  for (int i = 0; i < count; ++i) groups[{b->items[i].mesh, b->items[i].box_size}].push_back(i);
  std::vector<std::vector<int>> members;
  for (auto& g : groups) {
    baorec_config c = *base;
    for (int a = 0; a < 3; ++a) {
      c.n[a] = g.first.first;
      c.box_size[a] = g.first.second;
      c.box_min[a] = 0.0f;
    }
    baorec_ctx* ctx = nullptr;
    int st = baorec_create(&c, &ctx);
    if (st != BAOREC_OK) {
      snprintf(b->msg, sizeof(b->msg), "batch: context for mesh %d: %s", g.first.first, baorec_last_error(nullptr));
      return st;
    }
    b->groups.push_back(ctx);
    members.push_back(g.second);
  }
  BK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  b->events.resize(2 * b->groups.size() + 1);
  for (auto& e : b->events) BK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // one eager pass first: lazy allocations and per-kernel attributes happen
  // outside the capture, and the pass checks every item
  int64_t l0 = 0;
  for (size_t g = 0; g < b->groups.size(); ++g) {
    l0 += b->groups[g]->launches;
    CKS(record_group(b, b->groups[g], members[g]));
    BK(cudaStreamSynchronize(b->groups[g]->stream));
  }
  int64_t l1 = 0;
  for (auto* ctx : b->groups) l1 += ctx->launches;
  b->launches_per_replay = l1 - l0;
  // capture: fork every group stream from the launch stream, join them back
  BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int st = BAOREC_OK;
  cudaError_t e = cudaEventRecord(b->events[0], b->stream);
  for (size_t g = 0; g < b->groups.size() && e == cudaSuccess && st == BAOREC_OK; ++g) {
    e = cudaStreamWaitEvent(b->groups[g]->stream, b->events[0], 0);
    if (e == cudaSuccess) st = record_group(b, b->groups[g], members[g]);
    if (e == cudaSuccess && st == BAOREC_OK) e = cudaEventRecord(b->events[1 + g], b->groups[g]->stream);
    if (e == cudaSuccess && st == BAOREC_OK) e = cudaStreamWaitEvent(b->stream, b->events[1 + g], 0);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(b->stream, &graph);
  if (st != BAOREC_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  BK(e);
  BK(ee);
  b->graph = graph;
  BK(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return BAOREC_OK;
}

extern "C" int baorec_batch_launch(baorec_batch* b, void* stream) {
  if (!b || !b->exec) return BAOREC_ERR_ARG;
  BK(cudaGraphLaunch(b->exec, stream ? (cudaStream_t)stream : b->stream));
  return BAOREC_OK;
}

extern "C" int baorec_batch_sync(baorec_batch* b, void* stream) {
  if (!b) return BAOREC_ERR_ARG;
  BK(cudaStreamSynchronize(stream ? (cudaStream_t)stream : b->stream));
  for (auto* ctx : b->groups) {
    int st = baorec::finish(ctx, 0);
    if (st != BAOREC_OK) {
      snprintf(b->msg, sizeof(b->msg), "%s", ctx->msg);
      return st;
    }
  }
  return BAOREC_OK;
}

extern "C" void* baorec_batch_stream(baorec_batch* b) { return b ? (void*)b->stream : nullptr; }

extern "C" int64_t baorec_batch_kernel_launches(const baorec_batch* b) { return b ? b->launches_per_replay : 0; }

extern "C" const char* baorec_batch_last_error(const baorec_batch* b) { return b ? b->msg : "null batch"; }

extern "C" int baorec_batch_destroy(baorec_batch* b) {
  if (!b) return BAOREC_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto e : b->events)
    if (e) cudaEventDestroy(e);
  for (auto* ctx : b->groups) baorec_destroy(ctx);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return BAOREC_OK;
}
