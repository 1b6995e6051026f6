// Batched runs: many plans (signals with their own n, k and parameters) in
// one call.  The batch forks the caller's stream into a fixed set of internal
// streams, runs plan i's pipeline on stream i mod S, and joins them back, so
// the small transforms of different signals fill the GPU together instead of
// one after the other.  Plans keep their own buffers (nothing is shared
// between concurrently running pipelines), so the results of a batched run
// are identical to running each plan alone.
//
// Graph form: gsfft_batch_capture records one batched run (draws fixed at
// capture time) into a CUDA graph; each gsfft_batch_launch replays it with one
// launch, on whatever signals the captured d_x buffers hold by then.  Every
// run's first kernel advances its plan's device epoch, so replays count votes
// afresh; the host mirrors the epoch and clears a vote table before a replay
// would wrap it.
#include "engine.cuh"

#include <vector>

namespace gsfft {

static_assert(GSFFT_MAX_LOOPS == MAX_LOOPS && GSFFT_MAX_RLFC_LOOPS == MAX_RLFC_LOOPS,
              "draw strides of gsfft_run_batched");

struct Batch {
  std::vector<Plan *> plans;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  BatchTail *tail = nullptr;        // persistent tail of every plan (or none)
  cudaEvent_t fork2 = nullptr;      // fork after the persistent tail
};

void batch_destroy(Batch *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->fork2) cudaEventDestroy(b->fork2);
  batch_tail_free(b->tail);
  delete b;
}

int batch_create(Plan *const *plans, int count, int nstreams, Batch **out) {
  if (!plans || count < 1 || !out) return GSFFT_ERR_PARAM;
  for (int i = 0; i < count; i++)
    if (!plans[i]) return GSFFT_ERR_PARAM;
  Batch *b = new Batch();
  b->plans.assign(plans, plans + count);
  const int S = nstreams < 1 ? 1 : (nstreams > count ? count : nstreams);
  int s = GSFFT_OK;
  for (int i = 0; i < S && s == GSFFT_OK; i++) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      if (st) cudaStreamDestroy(st);
      set_last_error("gsfft_batch_create: %s", cudaGetErrorString(cudaGetLastError()));
      s = GSFFT_ERR_CUDA;
      break;
    }
    b->streams.push_back(st);
    b->joins.push_back(ev);
  }
  if (s == GSFFT_OK && (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&b->fork2, cudaEventDisableTiming) != cudaSuccess))
    s = GSFFT_ERR_CUDA;
  if (s != GSFFT_OK) {
    batch_destroy(b);
    return s;
  }
  *out = b;
  return GSFFT_OK;
}

int batch_run(Batch *b, const void *const *d_x, const int *offs, const int *a, const int *ai,
              cudaStream_t st, bool capturing) {
  if (!b || !d_x || !offs || !a || !ai) return GSFFT_ERR_PARAM;
  const int S = (int)b->streams.size();
  GS_CUDA(cudaEventRecord(b->fork, st));
  for (int i = 0; i < S; i++) GS_CUDA(cudaStreamWaitEvent(b->streams[i], b->fork, 0));
  const int n = (int)b->plans.size();
  int s = GSFFT_OK;
  auto join = [&]() {
    // join every internal stream back into the caller's stream, also on error
    for (int i = 0; i < S; i++) {
      if (cudaEventRecord(b->joins[i], b->streams[i]) != cudaSuccess ||
          cudaStreamWaitEvent(st, b->joins[i], 0) != cudaSuccess) {
        set_last_error("gsfft_run_batched: join: %s", cudaGetErrorString(cudaGetLastError()));
        if (s == GSFFT_OK) s = GSFFT_ERR_CUDA;
      }
    }
  };
  if (!b->tail) {
    for (int i = 0; i < n && s == GSFFT_OK; i++)
      s = plan_run(b->plans[i], d_x[i], offs + (size_t)i * MAX_RLFC_LOOPS, a + (size_t)i * MAX_LOOPS,
                   ai + (size_t)i * MAX_LOOPS, b->streams[i % S], capturing);
    join();
    return s;
  }
  // fronts on the streams, every plan's voting in one persistent launch, then
  // estimation and top-k on the streams
  for (int i = 0; i < n && s == GSFFT_OK; i++)
    s = plan_run(b->plans[i], d_x[i], offs + (size_t)i * MAX_RLFC_LOOPS, a + (size_t)i * MAX_LOOPS,
                 ai + (size_t)i * MAX_LOOPS, b->streams[i % S], capturing, PH_FRONT);
  join();
  if (s == GSFFT_OK) s = batch_tail_launch(b->tail, st);
  if (s == GSFFT_OK) {
    GS_CUDA(cudaEventRecord(b->fork2, st));
    for (int i = 0; i < S; i++) GS_CUDA(cudaStreamWaitEvent(b->streams[i], b->fork2, 0));
  }
  for (int i = 0; i < n && s == GSFFT_OK; i++)
    s = plan_run(b->plans[i], nullptr, nullptr, nullptr, nullptr, b->streams[i % S], capturing,
                 PH_EST | PH_TOPK);
  join();
  return s;
}

int batch_capture(Batch *b, const void *const *d_x, const int *offs, const int *a, const int *ai) {
  if (!b || !d_x || !offs || !a || !ai) return GSFFT_ERR_PARAM;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaStream_t cs = nullptr;
  GS_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  int s = GSFFT_OK;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    set_last_error("gsfft_batch_capture: %s", cudaGetErrorString(cudaGetLastError()));
    s = GSFFT_ERR_CUDA;
  } else {
    s = batch_run(b, d_x, offs, a, ai, cs, true);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cs, &g);
    if (s == GSFFT_OK && e != cudaSuccess) {
      set_last_error("gsfft_batch_capture: end capture: %s", cudaGetErrorString(e));
      s = GSFFT_ERR_UNSUPPORTED;
    }
    if (s == GSFFT_OK) {
      const cudaError_t ei = cudaGraphInstantiate(&b->exec, g, 0);
      if (ei != cudaSuccess) {
        set_last_error("gsfft_batch_capture: instantiate: %s", cudaGetErrorString(ei));
        s = GSFFT_ERR_UNSUPPORTED;
        cudaGraphDestroy(g);
      } else {
        b->graph = g;
      }
    } else if (g) {
      cudaGraphDestroy(g);
    }
  }
  cudaGetLastError();  // a failed capture leaves its error behind
  cudaStreamDestroy(cs);
  return s;
}

int batch_set_persistent_tail(Batch *b, bool on) {
  if (!b) return GSFFT_ERR_PARAM;
  if (b->exec) {  // a captured graph holds the other form
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  batch_tail_free(b->tail);
  b->tail = nullptr;
  if (!on) return GSFFT_OK;
  return batch_tail_create(b->plans.data(), (int)b->plans.size(), &b->tail);
}

int batch_launch(Batch *b, cudaStream_t st) {
  if (!b) return GSFFT_ERR_PARAM;
  if (!b->exec) return GSFFT_ERR_STATE;
  for (Plan *P : b->plans) GS_CHECK(plan_epoch_advance(P, st));
  GS_CUDA(cudaGraphLaunch(b->exec, st));
  return GSFFT_OK;
}

}  // namespace gsfft
