// batch.cpp -- the batched sweep behind dmsim_batch_* (include/dmsim_gb300.h):
// many independent circuits of uneven qubit counts, each planned like a single
// circuit, run together from one captured CUDA graph with two kinds of branch:
//   * narrow circuits (fewer than wide_n qubits, most of a sweep by count and
//     little of its work): one persistent work-queue kernel (batch.cu) over
//     all of them -- reset states -> queue -> per-circuit diagonal and
//     <Z_i Z_{i+1}>;
//   * wide circuits (at least wide_n qubits, nearly all of the work): each
//     held by an internal engine handle whose own pass kernels (tensor-core,
//     register and tiled passes, the same as a single run) are captured on
//     one of a few side streams, so wide circuits run concurrently with each
//     other and with the queue; then the circuit's diagonal and <ZZ>.
// The autotuner times a few (wide_n, tile shape) choices and keeps the best.
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
#include "engine_internal.h"
#include "plan.h"

using namespace dmg;

struct dmsim_batch {
  std::vector<uint32_t> nq;
  std::vector<std::vector<GateRec>> circ;
  int mode = 1, maxk = 4, planner = 0;
  int fused_arith = 0;  // fused batches: 0 = FP64 width (the engine's default), 1 = double-float
  int wide_n = 10;      // circuits of at least wide_n qubits run on the engine's own pass kernels
  std::vector<dmsim_handle> sims;       // per circuit: the engine handle of a wide circuit, else null
  std::vector<cudaStream_t> side;       // side streams of the wide circuits' graph branches
  std::vector<cudaEvent_t> join;        // one per side stream
  cudaEvent_t fork = nullptr;
  std::vector<int> narrow;              // the circuits run by the work-queue kernel
  uint64_t narrow_alloc = 0;            // entries allocated for the narrow states
  int device = 0, sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<BatchCircuit> circs;
  uint64_t total_entries = 0, diag_total = 0, zz_total = 0;
  double *d_re = nullptr, *d_im = nullptr, *d_diag = nullptr, *d_zz = nullptr;
  BatchCircuit* d_circs = nullptr;     // the narrow circuits' records
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

bool df64_queue(const dmsim_batch* b) { return b->mode == 1 && b->fused_arith == 1; }

// The engine handle of wide circuit c, created and uploaded on first use and
// kept (it owns its state and descriptors).
dmsim_handle wide_sim(dmsim_batch* b, int c) {
  if (b->sims[c]) return b->sims[c];
  dmsim_handle h = nullptr;
  int st = dmsim_create(b->nq[c], 1, &h);
  auto chk = [&](int code, const char* what) {
    if (code != DMSIM_OK) {
      std::string msg = std::string("wide circuit ") + std::to_string(c) + ": " + what + ": " +
                        (h ? dmsim_last_error(h) : dmsim_status_string(code));
      if (h) dmsim_destroy(h);
      throw BErr{code, msg};
    }
  };
  chk(st, "create");
  chk(dmsim_set_option(h, DMSIM_OPT_MODE, b->mode), "mode");
  chk(dmsim_set_option(h, DMSIM_OPT_MAX_K, b->maxk), "max_k");
  chk(dmsim_set_option(h, DMSIM_OPT_PLANNER, b->planner), "planner");
  chk(dmsim_set_option(h, DMSIM_OPT_FUSED_ARITH, b->fused_arith), "arithmetic");
  chk(dmsim_set_option(h, DMSIM_OPT_PLAIN_ARITH, 0), "arithmetic");
  chk(dmsim_set_option(h, DMSIM_OPT_GRAPH, 0), "graph");  // its passes are captured into the batch's graph
  for (const GateRec& g : b->circ[c]) chk(dmsim_append(h, g.op, g.qb, g.theta, g.phi, g.lambda), "append");
  chk(dmsim_upload(h), "upload");
  b->sims[c] = h;
  return h;
}

// The narrow circuits' states (contiguous, 256-byte aligned), records and
// descriptors (per circuit, per pass, with the current tile shape) in
// layer-major ranges; the wide circuits' engine handles; and the captured
// graph of both branches.
void build(dmsim_batch* b) {
  const int nc = (int)b->nq.size();
  const std::vector<std::vector<PassSpec>>& plans = b->plans;
  // ---- narrow circuits: states and records
  b->narrow.clear();
  uint64_t off = 0;
  for (int c = 0; c < nc; c++) {
    b->circs[c].state_off = 0;
    if ((int)b->nq[c] >= b->wide_n) continue;
    b->narrow.push_back(c);
    b->circs[c].state_off = off;
    off += std::max<uint64_t>(1ull << (2 * b->nq[c]), 32);
  }
  if (off > b->narrow_alloc) {
    cudaFree(b->d_re);
    cudaFree(b->d_im);
    b->d_re = b->d_im = nullptr;
    b->narrow_alloc = 0;
    B_CUDA(cudaMalloc(&b->d_re, off * sizeof(double)));
    B_CUDA(cudaMalloc(&b->d_im, off * sizeof(double)));
    b->narrow_alloc = off;
  }
  b->total_entries = off;
  std::vector<BatchCircuit> nrec;
  for (int c : b->narrow) nrec.push_back(b->circs[c]);
  if (!nrec.empty())
    B_CUDA(cudaMemcpy(b->d_circs, nrec.data(), nrec.size() * sizeof(BatchCircuit), cudaMemcpyHostToDevice));
  // ---- narrow circuits: descriptors and layer-major ranges
  size_t maxp = 0;
  for (int c : b->narrow) maxp = std::max(maxp, plans[c].size());
  std::vector<unsigned char> blob;
  std::vector<BatchRange> ranges;
  std::vector<std::vector<int>> range_of(nc);
  for (int c = 0; c < nc; c++) range_of[c].assign(plans[c].size(), -1);
  unsigned long long item = 0;
  double bytes = 0;
  for (size_t p = 0; p < maxp; p++)
    for (int c : b->narrow) {
      if (p >= plans[c].size()) continue;
      const PassSpec& ps = plans[c][p];
      const size_t doff = blob.size();
      blob.resize(doff + ((desc_size(ps.K) + 255) & ~(size_t)255));
      uint64_t ntiles = 0;
      int tile = 0;
      const int g_cap = (int)b->nq[c] <= b->small_n ? std::max(0, 8 - ps.K - b->g_shift) : 8;
      const uint64_t entries = build_desc(ps, (int)b->nq[c], blob.data() + doff, nullptr, &ntiles, &tile, g_cap);
      bytes += 16.0 * (double)entries;
      BatchRange r;
      std::memset(&r, 0, sizeof r);
      r.desc_off = doff;
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
  if (b->test_stall && !b->narrow.empty() && b->narrow[0] == 0 && plans[0].size() >= 2)
    ranges[range_of[0].back()].dep_expected += 1;
  b->nranges = (int)ranges.size();
  b->nitems = item;
  B_CUDA(cudaMalloc(&b->d_blob, std::max<size_t>(blob.size(), 256)));
  B_CUDA(cudaMalloc(&b->d_ranges, std::max<size_t>(ranges.size(), 1) * sizeof(BatchRange)));
  B_CUDA(cudaMalloc(&b->d_done, std::max<size_t>(ranges.size(), 1) * sizeof(unsigned)));
  if (!blob.empty()) B_CUDA(cudaMemcpy(b->d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice));
  if (!ranges.empty())
    B_CUDA(cudaMemcpy(b->d_ranges, ranges.data(), ranges.size() * sizeof(BatchRange), cudaMemcpyHostToDevice));
  b->grid = (unsigned)(b->sms * batch_blocks_per_sm(df64_queue(b)));
  // ---- wide circuits: engine handles, their passes and bytes
  b->n_passes = 0;
  for (int c : b->narrow) b->n_passes += plans[c].size();
  for (int c = 0; c < nc; c++) {
    if ((int)b->nq[c] < b->wide_n) continue;
    dmsim_handle h = wide_sim(b, c);
    uint32_t np = 0, nb = 0;
    dmsim_plan_stats(h, &np, &nb);
    b->n_passes += np;
    bytes += sim_plan_bytes(h);
  }
  b->bytes = bytes;
  // ---- one graph: the queue branch on the batch stream, the wide circuits
  // round-robin on the side streams
  BatchLaunch a;
  a.re = b->d_re;
  a.im = b->d_im;
  a.total_entries = b->total_entries;
  a.blob = b->d_blob;
  a.ranges = b->d_ranges;
  a.nranges = b->nranges;
  a.nitems = b->nitems;
  a.circs = b->d_circs;
  a.ncirc = (int)b->narrow.size();
  a.next = b->d_next;
  a.done = b->d_done;
  a.err = b->d_err;
  a.diag = b->d_diag;
  a.zz = b->d_zz;
  a.grid = b->grid;
  a.spin_limit = b->wait_limit;
  a.df64_arith = df64_queue(b);
  cudaGraph_t graph = nullptr;
  std::string werr;
  B_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaEventRecord(b->fork, b->stream);
  std::vector<char> used(b->side.size(), 0);
  int k = 0;
  for (int c = 0; c < nc && e == cudaSuccess; c++) {
    if ((int)b->nq[c] < b->wide_n) continue;
    const int sidx = k++ % (int)b->side.size();
    cudaStream_t st = b->side[sidx];
    if (!used[sidx]) {
      e = cudaStreamWaitEvent(st, b->fork, 0);
      used[sidx] = 1;
    }
    void *re = nullptr, *im = nullptr;
    if (e == cudaSuccess) e = dmsim_device_state(b->sims[c], &re, &im) == DMSIM_OK ? cudaSuccess : cudaErrorUnknown;
    if (e == cudaSuccess) e = sim_enqueue(b->sims[c], st, werr);
    if (e == cudaSuccess)
      e = launch_circuit_epilogue(static_cast<const double*>(re), (int)b->nq[c], b->d_diag + b->circs[c].diag_off,
                                  b->d_zz + b->circs[c].zz_off, st);
  }
  if (e == cudaSuccess) e = launch_batch(a, b->stream);
  for (size_t i = 0; i < b->side.size() && e == cudaSuccess; i++) {
    if (!used[i]) continue;
    e = cudaEventRecord(b->join[i], b->side[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->join[i], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    throw BErr{DMSIM_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2) +
                                   (werr.empty() ? "" : " (" + werr + ")")};
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
  // plan every circuit (the wide ones are planned again by their engine handles)
  std::vector<std::vector<PassSpec>> plans(nc);
  b->n_basic = 0;
  const int arith = df64_queue(b) ? AR_DF64 : AR_FP64;
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
      plans[c] = plan_learned(basics, (int)b->nq[c], b->maxk, arith, false, m, nullptr, err);
      if (!err.empty()) throw BErr{DMSIM_ERR_CUDA, err};
    } else plans[c] = plan_greedy(basics, b->maxk);
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
    uint64_t doff = 0, zoff = 0;
    for (uint32_t c = 0; c < n_circuits; c++) {
      BatchCircuit bc;
      std::memset(&bc, 0, sizeof bc);
      bc.n = (int)n_qubits[c];
      bc.diag_off = doff;
      bc.zz_off = zoff;
      doff += 1ull << n_qubits[c];
      zoff += n_qubits[c] > 1 ? n_qubits[c] - 1 : 0;
      b->circs.push_back(bc);
    }
    b->sims.assign(n_circuits, nullptr);
    b->diag_total = doff;
    b->zz_total = std::max<uint64_t>(zoff, 1);
    constexpr int kSideStreams = 8;
    for (int i = 0; i < kSideStreams; i++) {
      cudaStream_t st = nullptr;
      cudaEvent_t ev = nullptr;
      B_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      b->side.push_back(st);
      B_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      b->join.push_back(ev);
    }
    B_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    B_CUDA(cudaMalloc(&b->d_diag, doff * sizeof(double)));
    B_CUDA(cudaMalloc(&b->d_zz, b->zz_total * sizeof(double)));
    B_CUDA(cudaMalloc(&b->d_circs, n_circuits * sizeof(BatchCircuit)));
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
  for (dmsim_handle h : b->sims)
    if (h) dmsim_destroy(h);
  for (cudaStream_t st : b->side) cudaStreamDestroy(st);
  for (cudaEvent_t ev : b->join) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
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
      case DMSIM_OPT_FUSED_ARITH: b->fused_arith = v != 0; break;
      case DMSIM_BATCH_OPT_WIDE_QUBITS:
        if (v < 1 || v > kBatchMaxQubits + 1) throw BErr{DMSIM_ERR_ARG, "wide circuits start at 1..17 qubits"};
        b->wide_n = (int)v;
        break;
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
    for (dmsim_handle h : b->sims) {  // a wide circuit's tensor pass whose bounded wait ran out
      int f = 0;
      if (h) B_CUDA(sim_take_error(h, &f));
      err |= f;
    }
    if (err) {
      // Work after the expired wait ran on partly updated states: make every
      // output NaN (all-ones bytes) rather than leave plausible values behind.
      B_CUDA(cudaMemsetAsync(b->d_diag, 0xFF, b->diag_total * sizeof(double), b->stream));
      B_CUDA(cudaMemsetAsync(b->d_zz, 0xFF, b->zz_total * sizeof(double), b->stream));
      if (b->total_entries) {
        B_CUDA(cudaMemsetAsync(b->d_re, 0xFF, b->total_entries * sizeof(double), b->stream));
        B_CUDA(cudaMemsetAsync(b->d_im, 0xFF, b->total_entries * sizeof(double), b->stream));
      }
      for (size_t c = 0; c < b->sims.size(); c++) {
        void *re = nullptr, *im = nullptr;
        if (!b->sims[c] || dmsim_device_state(b->sims[c], &re, &im) != DMSIM_OK) continue;
        const size_t N = 1ull << (2 * b->nq[c]);
        B_CUDA(cudaMemsetAsync(re, 0xFF, N * sizeof(double), b->stream));
        B_CUDA(cudaMemsetAsync(im, 0xFF, N * sizeof(double), b->stream));
      }
      B_CUDA(cudaStreamSynchronize(b->stream));
      throw BErr{DMSIM_ERR_TIMEOUT, "a bounded device wait ran out; every output of this run is NaN"};
    }
  });
}

int dmsim_batch_autotune(dmsim_batch_handle b, double* best_ms) {
  return guard(b, [&] {
    if (!b->uploaded) throw BErr{DMSIM_ERR_STATE, "autotune() before upload()"};
    struct Cfg {
      int wide_n, small_n, g_shift;
    };
    // where the engine's own kernels take over from the queue, and the
    // queue's tile shape for its smallest circuits
    const int w = b->wide_n;
    const Cfg cands[] = {{w, 0, 0}, {w - 1, 0, 0}, {w + 1, 0, 0}, {w, 8, 1}, {w, 8, 2}};
    double best = 1e30;
    Cfg pick = cands[0];
    for (const Cfg& c : cands) {
      if (c.wide_n < 1 || c.wide_n > kBatchMaxQubits + 1) continue;
      free_plan(b);
      b->wide_n = c.wide_n;
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
    b->wide_n = pick.wide_n;
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
    if ((int)b->nq[circuit] >= b->wide_n && b->sims[circuit]) {  // a wide circuit: its engine handle's state
      const int st = dmsim_get_dm(b->sims[circuit], re, im);
      if (st != DMSIM_OK) throw BErr{st, dmsim_last_error(b->sims[circuit])};
      return;
    }
    const uint64_t N = 1ull << (2 * b->nq[circuit]);
    B_CUDA(cudaMemcpy(re, b->d_re + b->circs[circuit].state_off, N * sizeof(double), cudaMemcpyDeviceToHost));
    B_CUDA(cudaMemcpy(im, b->d_im + b->circs[circuit].state_off, N * sizeof(double), cudaMemcpyDeviceToHost));
    if (df64_queue(b)) {  // double-float queues hold (hi, lo) pairs: widen on the host
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
