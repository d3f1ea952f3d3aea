// batch.cpp -- the batched sweep behind dmsim_batch_* (include/dmsim_gb300.h):
// many independent circuits of uneven qubit counts, each planned like a single
// circuit, run together by the persistent work-queue kernel of batch.cu from
// one captured CUDA graph (reset states -> queue -> per-circuit diagonal and
// <Z_i Z_{i+1}>).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dmsim_gb300.h"
#include "batch.h"
#include "costmodel.h"
#include "gates.h"
#include "kernels.h"
#include "plan.h"

using namespace dmg;

struct dmsim_batch {
  std::vector<uint32_t> nq;
  std::vector<std::vector<GateRec>> circ;
  int mode = 1, maxk = 4, planner = 0;
  int device = 0, sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<BatchCircuit> circs;
  uint64_t total_entries = 0, diag_total = 0, zz_total = 0;
  double *d_re = nullptr, *d_im = nullptr, *d_diag = nullptr, *d_zz = nullptr;
  BatchCircuit* d_circs = nullptr;
  unsigned char* d_blob = nullptr;
  BatchRange* d_ranges = nullptr;
  unsigned long long* d_next = nullptr;
  unsigned* d_done = nullptr;
  int* d_err = nullptr;
  int nranges = 0;
  unsigned long long nitems = 0;
  unsigned grid = 0;
  cudaGraphExec_t gexec = nullptr;
  bool uploaded = false;
  uint64_t n_passes = 0, n_basic = 0;
  double bytes = 0, last_ms = 0;
  std::vector<std::vector<PassSpec>> plans;
  // tile shape: circuits of at most small_n qubits get log2(groups per tile)
  // reduced by g_shift (smaller tiles, more blocks on a small state)
  int small_n = 0, g_shift = 0;
  unsigned wait_limit = 1u << 25;  // polls (128 ns naps) before a dependency wait gives up: ~4 s
  int test_stall = 0;              // test hook: the last pass of circuit 0 waits for a tile that never comes
  std::string err;
};

namespace {

struct BErr {
  int code;
  std::string msg;
};

#define B_CUDA(call)                                                                                  \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess)                                                                            \
      throw BErr{e_ == cudaErrorMemoryAllocation ? DMSIM_ERR_OOM : DMSIM_ERR_CUDA,                    \
                 std::string(#call) + ": " + cudaGetErrorString(e_)};                                 \
  } while (0)

template <typename F>
int guard(dmsim_batch* b, F&& f) {
  if (!b) return DMSIM_ERR_ARG;
  try {
    f();
  } catch (const BErr& e) {
    b->err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    b->err = "host allocation failed";
    return DMSIM_ERR_OOM;
  }
  b->err.clear();
  return DMSIM_OK;
}

void free_plan(dmsim_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  cudaFree(b->d_blob);
  cudaFree(b->d_ranges);
  cudaFree(b->d_done);
  b->d_blob = nullptr;
  b->d_ranges = nullptr;
  b->d_done = nullptr;
  b->uploaded = false;
}

// Descriptors (per circuit, per pass, with the current tile shape),
// layer-major ranges, and the captured graph.
void build(dmsim_batch* b) {
  const int nc = (int)b->nq.size();
  const std::vector<std::vector<PassSpec>>& plans = b->plans;
  // descriptors (per circuit, per pass) and layer-major ranges
  size_t maxp = 0;
  for (auto& p : plans) maxp = std::max(maxp, p.size());
  std::vector<unsigned char> blob;
  std::vector<BatchRange> ranges;
  std::vector<std::vector<int>> range_of(nc);
  for (int c = 0; c < nc; c++) range_of[c].assign(plans[c].size(), -1);
  unsigned long long item = 0;
  double bytes = 0;
  for (size_t p = 0; p < maxp; p++)
    for (int c = 0; c < nc; c++) {
      if (p >= plans[c].size()) continue;
      const PassSpec& ps = plans[c][p];
      const size_t off = blob.size();
      blob.resize(off + ((desc_size(ps.K) + 255) & ~(size_t)255));
      uint64_t ntiles = 0;
      int tile = 0;
      const int g_cap = (int)b->nq[c] <= b->small_n ? std::max(0, 8 - ps.K - b->g_shift) : 8;
      const uint64_t entries = build_desc(ps, (int)b->nq[c], blob.data() + off, nullptr, &ntiles, &tile, g_cap);
      bytes += 16.0 * (double)entries;
      BatchRange r;
      std::memset(&r, 0, sizeof r);
      r.desc_off = off;
      r.state_off = b->circs[c].state_off;
      r.item_begin = item;
      r.ntiles = (uint32_t)ntiles;
      r.K = ps.K;
      r.cls = ps.cls;
      r.dep = p == 0 ? -1 : range_of[c][p - 1];
      r.dep_expected = p == 0 ? 0 : ranges[range_of[c][p - 1]].ntiles;
      range_of[c][p] = (int)ranges.size();
      ranges.push_back(r);
      item += ntiles;
    }
  if (b->test_stall && plans[0].size() >= 2) ranges[range_of[0].back()].dep_expected += 1;
  b->nranges = (int)ranges.size();
  b->nitems = item;
  b->bytes = bytes;
  B_CUDA(cudaMalloc(&b->d_blob, std::max<size_t>(blob.size(), 256)));
  B_CUDA(cudaMalloc(&b->d_ranges, std::max<size_t>(ranges.size(), 1) * sizeof(BatchRange)));
  B_CUDA(cudaMalloc(&b->d_done, std::max<size_t>(ranges.size(), 1) * sizeof(unsigned)));
  if (!blob.empty()) B_CUDA(cudaMemcpy(b->d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice));
  if (!ranges.empty())
    B_CUDA(cudaMemcpy(b->d_ranges, ranges.data(), ranges.size() * sizeof(BatchRange), cudaMemcpyHostToDevice));
  b->grid = (unsigned)(b->sms * batch_blocks_per_sm(b->mode == 1));
  // one graph: reset -> queue -> epilogue
  BatchLaunch a;
  a.re = b->d_re;
  a.im = b->d_im;
  a.total_entries = b->total_entries;
  a.blob = b->d_blob;
  a.ranges = b->d_ranges;
  a.nranges = b->nranges;
  a.nitems = b->nitems;
  a.circs = b->d_circs;
  a.ncirc = nc;
  a.next = b->d_next;
  a.done = b->d_done;
  a.err = b->d_err;
  a.diag = b->d_diag;
  a.zz = b->d_zz;
  a.grid = b->grid;
  a.spin_limit = b->wait_limit;
  a.df64_arith = b->mode == 1;  // fused batches compute in double-float, plain ones in FP64
  cudaGraph_t graph = nullptr;
  B_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = launch_batch(a, b->stream);
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    throw BErr{DMSIM_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2)};
  }
  e = cudaGraphInstantiate(&b->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->gexec = nullptr;
    throw BErr{DMSIM_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)};
  }
}

void upload(dmsim_batch* b) {
  if (b->uploaded) throw BErr{DMSIM_ERR_STATE, "upload() called twice"};
  const int nc = (int)b->nq.size();
  // plan every circuit
  std::vector<std::vector<PassSpec>> plans(nc);
  b->n_passes = b->n_basic = 0;
  for (int c = 0; c < nc; c++) {
    std::vector<Basic> basics;
    for (const GateRec& g : b->circ[c]) decompose(g, basics);
    bool rlin = false;
    for (const Basic& x : basics) rlin |= x.kind == BK_RLIN;
    if (rlin) throw BErr{DMSIM_ERR_UNSUPPORTED, "the batched sweep does not take SRN (run such circuits singly)"};
    if (b->mode == 0) plans[c] = plan_plain(basics);
    else if (b->planner == 1) {
      std::lock_guard<std::mutex> lock(cost_model_mutex());
      CostModel& m = global_cost_model();
      if (!m.ready) throw BErr{DMSIM_ERR_STATE, "the learned planner needs a trained or loaded cost model"};
      std::string err;
      plans[c] = plan_learned(basics, (int)b->nq[c], b->maxk, AR_DF64, false, m, nullptr, err);
      if (!err.empty()) throw BErr{DMSIM_ERR_CUDA, err};
    } else plans[c] = plan_greedy(basics, b->maxk);
    b->n_passes += plans[c].size();
    b->n_basic += basics.size();
  }
  b->plans = std::move(plans);
  build(b);
  b->uploaded = true;
}

}  // namespace

extern "C" {

int dmsim_batch_create(uint32_t n_circuits, const uint32_t* n_qubits, dmsim_batch_handle* out) {
  if (!out || !n_qubits || n_circuits == 0) return DMSIM_ERR_ARG;
  *out = nullptr;
  for (uint32_t c = 0; c < n_circuits; c++)
    if (n_qubits[c] < 1 || n_qubits[c] > (uint32_t)kBatchMaxQubits) return DMSIM_ERR_ARG;
  dmsim_batch* b = new (std::nothrow) dmsim_batch;
  if (!b) return DMSIM_ERR_OOM;
  const int st = guard(b, [&] {
    b->nq.assign(n_qubits, n_qubits + n_circuits);
    b->circ.resize(n_circuits);
    B_CUDA(cudaGetDevice(&b->device));
    B_CUDA(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
    B_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    B_CUDA(cudaEventCreate(&b->ev0));
    B_CUDA(cudaEventCreate(&b->ev1));
    uint64_t off = 0, doff = 0, zoff = 0;
    for (uint32_t c = 0; c < n_circuits; c++) {
      BatchCircuit bc;
      std::memset(&bc, 0, sizeof bc);
      bc.n = (int)n_qubits[c];
      bc.state_off = off;
      bc.diag_off = doff;
      bc.zz_off = zoff;
      off += std::max<uint64_t>(1ull << (2 * n_qubits[c]), 32);  // keep every state 256-byte aligned
      doff += 1ull << n_qubits[c];
      zoff += n_qubits[c] > 1 ? n_qubits[c] - 1 : 0;
      b->circs.push_back(bc);
    }
    b->total_entries = off;
    b->diag_total = doff;
    b->zz_total = std::max<uint64_t>(zoff, 1);
    B_CUDA(cudaMalloc(&b->d_re, off * sizeof(double)));
    B_CUDA(cudaMalloc(&b->d_im, off * sizeof(double)));
    B_CUDA(cudaMalloc(&b->d_diag, doff * sizeof(double)));
    B_CUDA(cudaMalloc(&b->d_zz, b->zz_total * sizeof(double)));
    B_CUDA(cudaMalloc(&b->d_circs, n_circuits * sizeof(BatchCircuit)));
    B_CUDA(cudaMemcpy(b->d_circs, b->circs.data(), n_circuits * sizeof(BatchCircuit), cudaMemcpyHostToDevice));
    B_CUDA(cudaMalloc(&b->d_next, sizeof(unsigned long long)));
    B_CUDA(cudaMalloc(&b->d_err, sizeof(int)));
  });
  if (st != DMSIM_OK) {
    dmsim_batch_destroy(b);
    return st;
  }
  *out = b;
  return DMSIM_OK;
}

int dmsim_batch_destroy(dmsim_batch_handle b) {
  if (!b) return DMSIM_ERR_ARG;
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_plan(b);
  cudaFree(b->d_re);
  cudaFree(b->d_im);
  cudaFree(b->d_diag);
  cudaFree(b->d_zz);
  cudaFree(b->d_circs);
  cudaFree(b->d_next);
  cudaFree(b->d_err);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return DMSIM_OK;
}

int dmsim_batch_set_option(dmsim_batch_handle b, int key, int64_t v) {
  return guard(b, [&] {
    if (b->uploaded) throw BErr{DMSIM_ERR_STATE, "set options before upload()"};
    switch (key) {
      case DMSIM_OPT_MODE: b->mode = v != 0; break;
      case DMSIM_OPT_MAX_K:
        if (v < 1 || v > kMaxK) throw BErr{DMSIM_ERR_ARG, "max_k must be 1..4"};
        b->maxk = (int)v;
        break;
      case DMSIM_OPT_PLANNER: b->planner = v != 0; break;
      case DMSIM_BATCH_OPT_WAIT_LIMIT:
        if (v < 1 || v > (int64_t)1 << 30) throw BErr{DMSIM_ERR_ARG, "wait limit must be 1..2^30 polls"};
        b->wait_limit = (unsigned)v;
        break;
      case DMSIM_BATCH_OPT_TEST_STALL: b->test_stall = v != 0; break;
      default: throw BErr{DMSIM_ERR_ARG, "unsupported batch option"};
    }
  });
}

int dmsim_batch_append(dmsim_batch_handle b, uint32_t circuit, int op, const uint32_t qb[5], double theta, double phi,
                       double lambda) {
  return guard(b, [&] {
    if (!qb || circuit >= b->nq.size()) throw BErr{DMSIM_ERR_ARG, "bad circuit index or null qubits"};
    if (b->uploaded) throw BErr{DMSIM_ERR_STATE, "append after upload()"};
    const int ar = gate_arity(op);
    if (op < 0 || op >= N_REF_OPS || ar == 0) throw BErr{DMSIM_ERR_ARG, "unknown gate id"};
    GateRec g;
    std::memset(&g, 0, sizeof g);
    g.op = op;
    for (int i = 0; i < 5; i++) {
      g.qb[i] = qb[i];
      if (qb[i] >= b->nq[circuit]) throw BErr{DMSIM_ERR_ARG, "qubit index out of range"};
    }
    for (int i = 0; i < ar; i++)
      for (int j = i + 1; j < ar; j++)
        if (qb[i] == qb[j]) throw BErr{DMSIM_ERR_ARG, "a gate's qubits must be distinct"};
    g.theta = theta;
    g.phi = phi;
    g.lambda = lambda;
    b->circ[circuit].push_back(g);
  });
}

int dmsim_batch_upload(dmsim_batch_handle b) { return guard(b, [&] { upload(b); }); }

int dmsim_batch_run(dmsim_batch_handle b) {
  return guard(b, [&] {
    if (!b->uploaded) throw BErr{DMSIM_ERR_STATE, "run() before upload()"};
    B_CUDA(cudaEventRecord(b->ev0, b->stream));
    B_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    B_CUDA(cudaEventRecord(b->ev1, b->stream));
    B_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0;
    B_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    int err = 0;
    B_CUDA(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
      // Items after the expired wait ran on partly updated states: make every
      // output NaN (all-ones bytes) rather than leave plausible values behind.
      B_CUDA(cudaMemsetAsync(b->d_diag, 0xFF, b->diag_total * sizeof(double), b->stream));
      B_CUDA(cudaMemsetAsync(b->d_zz, 0xFF, b->zz_total * sizeof(double), b->stream));
      B_CUDA(cudaMemsetAsync(b->d_re, 0xFF, b->total_entries * sizeof(double), b->stream));
      B_CUDA(cudaMemsetAsync(b->d_im, 0xFF, b->total_entries * sizeof(double), b->stream));
      B_CUDA(cudaStreamSynchronize(b->stream));
      throw BErr{DMSIM_ERR_TIMEOUT, "a work-queue dependency wait ran out; every output of this run is NaN"};
    }
  });
}

int dmsim_batch_autotune(dmsim_batch_handle b, double* best_ms) {
  return guard(b, [&] {
    if (!b->uploaded) throw BErr{DMSIM_ERR_STATE, "autotune() before upload()"};
    struct Cfg {
      int small_n, g_shift;
    };
    const Cfg cands[] = {{0, 0}, {8, 1}, {8, 2}, {10, 1}, {10, 2}, {12, 1}};
    double best = 1e30;
    Cfg pick = cands[0];
    for (const Cfg& c : cands) {
      free_plan(b);
      b->small_n = c.small_n;
      b->g_shift = c.g_shift;
      build(b);
      b->uploaded = true;
      double t = 1e30;
      for (int r = 0; r < 2; r++) {
        B_CUDA(cudaEventRecord(b->ev0, b->stream));
        B_CUDA(cudaGraphLaunch(b->gexec, b->stream));
        B_CUDA(cudaEventRecord(b->ev1, b->stream));
        B_CUDA(cudaEventSynchronize(b->ev1));
        float ms = 0;
        B_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        t = std::min(t, (double)ms);
      }
      if (t < best) {
        best = t;
        pick = c;
      }
    }
    free_plan(b);
    b->small_n = pick.small_n;
    b->g_shift = pick.g_shift;
    build(b);
    b->uploaded = true;
    if (best_ms) *best_ms = best;
  });
}

int dmsim_batch_get_diag(dmsim_batch_handle b, uint32_t circuit, double* out) {
  return guard(b, [&] {
    if (!out || circuit >= b->nq.size()) throw BErr{DMSIM_ERR_ARG, "bad circuit index or null output"};
    B_CUDA(cudaMemcpy(out, b->d_diag + b->circs[circuit].diag_off, (1ull << b->nq[circuit]) * sizeof(double),
                      cudaMemcpyDeviceToHost));
  });
}

int dmsim_batch_get_zz(dmsim_batch_handle b, uint32_t circuit, double* out) {
  return guard(b, [&] {
    if (!out || circuit >= b->nq.size()) throw BErr{DMSIM_ERR_ARG, "bad circuit index or null output"};
    if (b->nq[circuit] > 1)
      B_CUDA(cudaMemcpy(out, b->d_zz + b->circs[circuit].zz_off, (b->nq[circuit] - 1) * sizeof(double),
                        cudaMemcpyDeviceToHost));
  });
}

int dmsim_batch_get_dm(dmsim_batch_handle b, uint32_t circuit, double* re, double* im) {
  return guard(b, [&] {
    if (!re || !im || circuit >= b->nq.size()) throw BErr{DMSIM_ERR_ARG, "bad circuit index or null output"};
    const uint64_t N = 1ull << (2 * b->nq[circuit]);
    B_CUDA(cudaMemcpy(re, b->d_re + b->circs[circuit].state_off, N * sizeof(double), cudaMemcpyDeviceToHost));
    B_CUDA(cudaMemcpy(im, b->d_im + b->circs[circuit].state_off, N * sizeof(double), cudaMemcpyDeviceToHost));
    if (b->mode == 1) {  // fused batches hold double-float pairs (hi, lo): widen on the host
      for (double* p : {re, im})
        for (uint64_t i = 0; i < N; i++) {
          float hl[2];
          std::memcpy(hl, p + i, sizeof hl);
          p[i] = (double)hl[0] + (double)hl[1];
        }
    }
  });
}

int dmsim_batch_stats(dmsim_batch_handle b, double out[8]) {
  return guard(b, [&] {
    if (!out) throw BErr{DMSIM_ERR_ARG, "null output"};
    out[0] = b->last_ms;
    out[1] = (double)b->n_passes;
    out[2] = (double)b->n_basic;
    out[3] = (double)b->nitems;
    out[4] = b->bytes;
    out[5] = (double)b->grid;
    out[6] = (double)b->small_n;
    out[7] = (double)b->g_shift;
  });
}

const char* dmsim_batch_last_error(dmsim_batch_handle b) { return b ? b->err.c_str() : "null handle"; }

}  // extern "C"
