// engine.cpp -- the Simulation object behind the C ABI (include/dmsim_gb300.h).
//
// Life cycle as DM-Sim's Simulation (src/dmsim_nvgpu_omp.cuh:193-814):
// append() collects gates, upload() decomposes them into basic gates, plans
// the passes (one per basic gate in plain mode, fused k<=4 operators in fused
// mode), writes all pass descriptors to the device in one copy and captures
// the launch sequence in a CUDA graph; run() replays it.  rho stays resident
// in HBM across runs (chained circuits), in the reference's result layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <sstream>
#include <string>
#include <vector>

#include <dlfcn.h>

#include <random>

#include "../../include/dmsim_gb300.h"
#include "costmodel.h"
#include "engine_internal.h"
#include "gates.h"
#include "kernels.h"
#include "metrics.h"
#include "plan.h"

using namespace dmg;

namespace {

struct DmError {
  int code;
  std::string msg;
};

#define DM_CUDA(call)                                                                         \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      throw DmError{e_ == cudaErrorMemoryAllocation ? DMSIM_ERR_OOM : DMSIM_ERR_CUDA,         \
                    std::string(#call) + ": " + cudaGetErrorString(e_)};                      \
  } while (0)

}  // namespace

struct dmsim_sim {
  uint32_t n = 0;
  uint64_t dim = 0, N = 0;
  int device = 0, sms = 0;
  bool fp32 = false;
  void* d_re = nullptr;
  void* d_im = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double* d_diag = nullptr;
  double* d_acc = nullptr;
  int* d_err = nullptr;  // set by a tensor pass whose bounded wait ran out

  std::vector<GateRec> circuit;
  std::vector<Channel> channels;  // superoperators of the circuit's noise channels
  bool uploaded = false;
  std::vector<PassInfo> passes;
  void* d_desc = nullptr;
  size_t desc_bytes = 0;
  uint32_t n_basic = 0;
  cudaGraphExec_t gexec = nullptr;

  int mode = 0, maxk = 4, planner = 0, record = 0, graph_on = 1, verbose = 0;
  int fused_arith = 0;  // fused FP64 runs: FP64 width (0: FP64-width tensor passes, FP64 elsewhere) or double-float (1)
  int plain_arith = 0;  // plain FP64 runs compute in FP64 (0: FP64-pipe-bound) or double-float (1: HBM-bound)
  int renorm = 64;      // complex64: renormalise every renorm passes (0 = never)
  int tensor = 1;       // K = 3, 4 dense/sparse passes on the tensor cores (DMSIM_OPT_TENSOR)
  int direct1 = 1;      // 1-qubit passes on the register kernel (DMSIM_OPT_DIRECT1)
  int arith = 0;        // arithmetic of the uploaded plan (kernels.h Arith)
  int64_t seed = -1;

  double last_ms = 0, last_bytes = 0, predicted_ms = 0;
  std::vector<PassRecord> records;
  std::string err;
};

namespace {

size_t esize(const dmsim_sim* s) { return s->fp32 ? 4 : 8; }

void free_plan(dmsim_sim* s) {
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  s->gexec = nullptr;
  if (s->d_desc) cudaFree(s->d_desc);
  s->d_desc = nullptr;
  s->desc_bytes = 0;
  s->passes.clear();
  s->n_basic = 0;
  s->uploaded = false;
}

void free_state(dmsim_sim* s) {
  if (s->d_re) cudaFree(s->d_re);
  if (s->d_im) cudaFree(s->d_im);
  s->d_re = s->d_im = nullptr;
}

void ensure_state(dmsim_sim* s) {
  if (s->d_re) return;
  const size_t bytes = s->N * esize(s);
  DM_CUDA(cudaSetDevice(s->device));
  if (cudaMalloc(&s->d_re, bytes) != cudaSuccess) {
    s->d_re = nullptr;
    cudaGetLastError();
    throw DmError{DMSIM_ERR_OOM, "device allocation of rho (real part) failed"};
  }
  if (cudaMalloc(&s->d_im, bytes) != cudaSuccess) {
    cudaFree(s->d_re);
    s->d_re = nullptr;
    s->d_im = nullptr;
    cudaGetLastError();
    throw DmError{DMSIM_ERR_OOM, "device allocation of rho (imaginary part) failed"};
  }
  DM_CUDA(launch_set_zero_state(s->d_re, s->d_im, s->N, s->fp32, s->stream));
  DM_CUDA(cudaStreamSynchronize(s->stream));
}

void check_qubits(const dmsim_sim* s, const GateRec& g) {
  const int ar = g.op == OP_CHANNEL ? g.nq : gate_arity(g.op);
  if (ar == 0) throw DmError{DMSIM_ERR_ARG, "unknown gate id " + std::to_string(g.op)};
  // the reference asserts every qubit slot < n_qubits (:334-338)
  for (int i = 0; i < 5; i++)
    if (g.qb[i] >= s->n) throw DmError{DMSIM_ERR_ARG, "qubit index out of range"};
  for (int i = 0; i < ar; i++)
    for (int j = i + 1; j < ar; j++)
      if (g.qb[i] == g.qb[j]) throw DmError{DMSIM_ERR_ARG, "a gate's qubits must be distinct"};
}

// Launch the planned passes on stream st (captured or direct).
void enqueue_passes(dmsim_sim* s, bool timed, cudaStream_t st) {
  for (size_t i = 0; i < s->passes.size(); i++) {
    PassInfo& p = s->passes[i];
    if (p.renorm) {
      if (timed) DM_CUDA(cudaEventRecord(p.ev0, st));
      DM_CUDA(launch_renormalise(s->d_re, s->d_im, (int)s->n, s->fp32, s->d_acc + 4, p.grid, st));
      if (timed) DM_CUDA(cudaEventRecord(p.ev1, st));
      continue;
    }
    if (p.conv) {
      if (timed) DM_CUDA(cudaEventRecord(p.ev0, st));
      if (p.conv == 1) DM_CUDA(launch_to_df64(s->d_re, s->d_im, s->N, p.grid, st));
      else DM_CUDA(launch_from_df64(s->d_re, s->d_im, s->N, p.grid, st));
      if (timed) DM_CUDA(cudaEventRecord(p.ev1, st));
      continue;
    }
    if (p.transpose) {
      if (timed) DM_CUDA(cudaEventRecord(p.ev0, st));
      DM_CUDA(launch_conj_transpose(s->d_re, s->d_im, (int)s->n, s->fp32, p.grid, st));
      if (timed) DM_CUDA(cudaEventRecord(p.ev1, st));
      continue;
    }
    LaunchArgs a;
    a.re = s->d_re;
    a.im = s->d_im;
    a.desc = static_cast<const char*>(s->d_desc) + p.desc_off;
    a.K = p.K;
    a.cls = p.cls;
    a.fp32 = s->fp32;
    a.arith = s->arith;
    a.grid = p.grid;
    a.tile_entries = p.tile_entries;
    a.tc = p.tc;
    a.real = p.real;
    a.err = s->d_err;
    a.direct1 = p.direct1;
    a.q0 = p.q0;
    a.n = (int)s->n;
    if (timed) DM_CUDA(cudaEventRecord(p.ev0, st));
    DM_CUDA(launch_pass(a, st));
    if (timed) DM_CUDA(cudaEventRecord(p.ev1, st));
  }
}

// The cost model shipped with the library: $DMSIM_COST_MODEL, else
// <library dir>/../model/cost_mlp.bin.
void load_default_cost_model() {
  std::string path;
  if (const char* e = getenv("DMSIM_COST_MODEL")) path = e;
  if (path.empty()) {
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&dmsim_create), &info) && info.dli_fname) {
      std::string lib = info.dli_fname;
      const size_t cut = lib.find_last_of('/');
      path = (cut == std::string::npos ? std::string(".") : lib.substr(0, cut)) + "/../model/cost_mlp.bin";
    }
  }
  if (!path.empty()) cost_model_load(global_cost_model(), path);
}

// Arithmetic of a run: complex64 state -> FP32; a fused FP64 run ->
// double-float unless the option asks for FP64; a plain run -> FP64 unless the
// option asks for double-float; the reference's order for SRN -> FP64.
int run_arith(const dmsim_sim* s, bool reference_order) {
  if (s->fp32) return AR_FP32;
  if (reference_order) return AR_FP64;
  if (s->mode == 1 && s->fused_arith) return AR_DF64;
  if (s->mode == 0 && s->plain_arith) return AR_DF64;
  return AR_FP64;
}

// Plain: one pass per basic gate.  Fused: the greedy (fixed-width) or the
// learned planner.  A circuit holding a real-linear gate (SRN) runs in the
// reference's own order in either mode, the only order that reproduces it.
std::vector<PassSpec> make_plan(dmsim_sim* s, const std::vector<Basic>& basics) {
  bool has_rlin = false;
  for (const Basic& b : basics) has_rlin |= b.kind == BK_RLIN;
  if (has_rlin) return plan_reference_order(basics);
  if (s->mode == 0) return plan_plain(basics);
  if (s->planner == 1) {
    std::lock_guard<std::mutex> lock(cost_model_mutex());
    CostModel& m = global_cost_model();
    if (!m.ready) load_default_cost_model();
    if (!m.ready)
      throw DmError{DMSIM_ERR_STATE, "the learned planner needs a cost model: train one (dmsim_cost_train) or load one "
                                     "(dmsim_cost_load, or set DMSIM_COST_MODEL)"};
    std::string err;
    std::vector<PassSpec> p =
        plan_learned(basics, (int)s->n, s->maxk, run_arith(s, false), s->tensor != 0, m, &s->predicted_ms, err);
    if (!err.empty()) throw DmError{DMSIM_ERR_CUDA, "learned planner: " + err};
    return p;
  }
  return plan_greedy(basics, s->maxk);
}

void upload_specs(dmsim_sim* s, const std::vector<PassSpec>& specs, uint32_t n_basic, int arith);

bool use_tensor(const dmsim_sim* s, const PassSpec& p, int arith) {
  return tc_choose(p, (int)s->n, s->tensor, arith);
}

void upload(dmsim_sim* s) {
  if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "upload() called twice without clear_circuit() (:347-350)"};
  ensure_state(s);
  std::vector<Basic> basics;
  for (const GateRec& g : s->circuit) decompose(g, basics, &s->channels);
  bool rlin = false, chan = false;
  for (const Basic& b : basics) {
    rlin |= b.kind == BK_RLIN;
    chan |= b.kind == BK_SUPER;
  }
  if (rlin && chan)
    throw DmError{DMSIM_ERR_UNSUPPORTED, "a circuit with SRN runs in the reference's order, which has no noise channels"};
  upload_specs(s, make_plan(s, basics), (uint32_t)basics.size(), run_arith(s, rlin));
}

// Write the descriptors of a plan to the device and capture its launches.
void upload_specs(dmsim_sim* s, const std::vector<PassSpec>& specs, uint32_t n_basic, int arith) {
  ensure_state(s);
  s->n_basic = n_basic;
  s->arith = arith;
  // descriptors, 256-byte aligned, one host blob, one copy
  std::vector<size_t> offs;
  std::vector<char> tcs;
  size_t total = 0;
  for (const PassSpec& p : specs) {
    offs.push_back(total);
    const bool tc = use_tensor(s, p, arith);
    tcs.push_back(tc);
    if (!p.transpose) total += ((tc ? tc_desc_bytes(p.K, arith) : desc_size(p.K)) + 255) & ~(size_t)255;
  }
  std::vector<unsigned char> blob(std::max<size_t>(total, 256));
  s->passes.clear();
  const double conv_bytes = 2.0 * 2.0 * (double)s->N * 8.0;
  if (arith == AR_DF64) {
    PassInfo pi;
    std::memset(&pi, 0, sizeof pi);
    pi.conv = 1;
    pi.grid = (unsigned)s->sms * 8;
    pi.bytes = conv_bytes;
    s->passes.push_back(pi);
  }
  for (size_t i = 0; i < specs.size(); i++) {
    PassInfo pi;
    std::memset(&pi, 0, sizeof pi);
    if (specs[i].transpose) {
      pi.transpose = true;
      pi.K = 0;
      pi.grid = (unsigned)s->sms * 8;
      pi.bytes = 2.0 * 2.0 * (double)s->N * (double)esize(s);
      s->passes.push_back(pi);
      continue;
    }
    uint64_t ntiles = 0;
    int tile = 0;
    pi.tc = tcs[i] != 0;
    const uint64_t entries =
        pi.tc ? build_tc_desc(specs[i], (int)s->n, blob.data() + offs[i], &pi.feat, &ntiles, &tile, true, arith)
              : build_desc(specs[i], (int)s->n, blob.data() + offs[i], &pi.feat, &ntiles, &tile);
    pi.feat.tc = pi.tc ? 1 : 0;
    pi.real = !pi.tc && pi.feat.real;
    pi.K = specs[i].K;
    pi.cls = specs[i].cls;
    pi.desc_off = offs[i];
    pi.tile_entries = tile;
    pi.bytes = (double)entries * 2.0 * (double)esize(s);
    pi.nbasic = specs[i].nbasic;
    pi.feat.arith = arith;
    const int bps = pi.tc ? tc_blocks_per_sm(pi.K, arith) : pass_blocks_per_sm(pi.K, pi.cls, arith);
    const uint64_t cap = (uint64_t)s->sms * (uint64_t)bps;
    pi.grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ntiles, cap));
    // 1-qubit passes (n >= 2): one register-resident group of 4 entries per thread
    pi.q0 = specs[i].q[0];
    pi.direct1 = s->direct1 && !pi.tc && pi.K == 1 && s->n >= 2 && direct1_class(pi.cls);
    if (pi.direct1) {
      const uint64_t groups = 1ull << (2 * s->n - 2);
      pi.grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((groups + 255) / 256, (uint64_t)s->sms * 8));
    }
    s->passes.push_back(pi);
    // complex64: FP64 trace + Hermitian renormalisation every renorm passes and at the end
    if (s->fp32 && s->renorm > 0 && ((i + 1) % (size_t)s->renorm == 0 || i + 1 == specs.size())) {
      PassInfo rn;
      std::memset(&rn, 0, sizeof rn);
      rn.renorm = true;
      rn.grid = (unsigned)s->sms * 8;
      rn.bytes = 2.0 * 2.0 * (double)s->N * (double)esize(s);
      s->passes.push_back(rn);
    }
  }
  if (arith == AR_DF64) {
    PassInfo pi;
    std::memset(&pi, 0, sizeof pi);
    pi.conv = 2;
    pi.grid = (unsigned)s->sms * 8;
    pi.bytes = conv_bytes;
    s->passes.push_back(pi);
  }
  if (total > 0) {
    DM_CUDA(cudaMalloc(&s->d_desc, total));
    DM_CUDA(cudaMemcpyAsync(s->d_desc, blob.data(), total, cudaMemcpyHostToDevice, s->stream));
    DM_CUDA(cudaStreamSynchronize(s->stream));
  }
  s->desc_bytes = total;
  // capture the pass sequence once; run() replays it
  if (s->graph_on && !s->passes.empty()) {
    cudaGraph_t graph = nullptr;
    DM_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue_passes(s, false, s->stream);
    } catch (...) {
      cudaStreamEndCapture(s->stream, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    DM_CUDA(cudaStreamEndCapture(s->stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&s->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      s->gexec = nullptr;
      throw DmError{DMSIM_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)};
    }
  }
  s->uploaded = true;
}

void run(dmsim_sim* s) {
  if (!s->uploaded) throw DmError{DMSIM_ERR_STATE, "run() before upload()"};
  ensure_state(s);
  const bool timed = s->record != 0;
  if (timed) {
    for (PassInfo& p : s->passes) {
      if (!p.ev0) DM_CUDA(cudaEventCreate(&p.ev0));
      if (!p.ev1) DM_CUDA(cudaEventCreate(&p.ev1));
    }
  }
  DM_CUDA(cudaEventRecord(s->ev0, s->stream));
  if (timed || !s->gexec) enqueue_passes(s, timed, s->stream);
  else DM_CUDA(cudaGraphLaunch(s->gexec, s->stream));
  DM_CUDA(cudaEventRecord(s->ev1, s->stream));
  DM_CUDA(cudaEventSynchronize(s->ev1));
  DM_CUDA(cudaGetLastError());
  bool any_tc = false;
  for (const PassInfo& p : s->passes) any_tc |= p.tc;
  if (any_tc) {
    int flag = 0;
    DM_CUDA(cudaMemcpy(&flag, s->d_err, sizeof flag, cudaMemcpyDeviceToHost));
    if (flag) {
      DM_CUDA(cudaMemset(s->d_err, 0, sizeof flag));
      throw DmError{DMSIM_ERR_TIMEOUT, "a tensor-core pass did not see its MMAs complete in time"};
    }
  }
  float ms = 0;
  DM_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
  s->last_ms = ms;
  double bytes = 0;
  for (const PassInfo& p : s->passes) bytes += p.bytes;
  s->last_bytes = bytes;
  if (timed) {
    s->records.clear();
    for (const PassInfo& p : s->passes) {
      float pms = 0;
      DM_CUDA(cudaEventElapsedTime(&pms, p.ev0, p.ev1));
      PassRecord r;
      r.feat = p.feat;
      if (p.conv) r.feat.cls = kRecConvert;
      else if (p.transpose) r.feat.cls = kRecTranspose;
      else if (p.renorm) r.feat.cls = kRecRenorm;
      r.ms = pms;
      r.bytes = p.bytes;
      r.grid = p.grid;
      s->records.push_back(r);
    }
  }
  if (s->verbose) {
    // the reference's per-run banner (PRINT_MEA_PER_CIRCUIT, :484-490)
    const double mem = 2.0 * (double)s->N * (double)esize(s) / 1024.0 / 1024.0;
    printf("\n============== DM-Sim ===============\n");
    printf("nqubits:%u, ngates:%zu, ngpus:1, comp:%.3lf ms, comm:%.3lf ms, sim:%.3lf ms, mem:%.3lf MB, mem_per_gpu:%.3lf MB\n",
           s->n, s->circuit.size(), (double)ms, 0.0, (double)ms, mem, mem);
    printf("=====================================\n");
  }
}

void clear_circuit(dmsim_sim* s) {
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (PassInfo& p : s->passes) {
    if (p.ev0) cudaEventDestroy(p.ev0);
    if (p.ev1) cudaEventDestroy(p.ev1);
  }
  free_plan(s);
  s->circuit.clear();
  s->channels.clear();
}

void reset_dm(dmsim_sim* s) {
  ensure_state(s);
  DM_CUDA(launch_set_zero_state(s->d_re, s->d_im, s->N, s->fp32, s->stream));
  DM_CUDA(cudaStreamSynchronize(s->stream));
}

std::vector<double> host_diag(dmsim_sim* s) {
  ensure_state(s);
  std::vector<double> d(s->dim);
  DM_CUDA(launch_get_diag(s->d_re, s->dim, s->fp32, s->d_diag, s->stream));
  DM_CUDA(cudaMemcpyAsync(d.data(), s->d_diag, s->dim * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  DM_CUDA(cudaStreamSynchronize(s->stream));
  return d;
}

int fail(dmsim_sim* s, const DmError& e) {
  if (s) s->err = e.msg;
  return e.code;
}

}  // namespace

// ============================================================================ C ABI
#define DM_TRY(h, ...)                                                \
  do {                                                                \
    if (!(h)) return DMSIM_ERR_ARG;                                   \
    try {                                                             \
      __VA_ARGS__;                                                    \
    } catch (const DmError& e_) {                                     \
      return fail((h), e_);                                           \
    } catch (const std::bad_alloc&) {                                 \
      return fail((h), DmError{DMSIM_ERR_OOM, "host allocation failed"}); \
    } catch (...) {                                                   \
      return fail((h), DmError{DMSIM_ERR_ARG, "unexpected exception"}); \
    }                                                                 \
    (h)->err.clear();                                                 \
    return DMSIM_OK;                                                  \
  } while (0)

extern "C" {

int dmsim_create(uint32_t n_qubits, uint32_t n_gpus, dmsim_handle* out) {
  if (!out) return DMSIM_ERR_ARG;
  *out = nullptr;
  // the reference requires n_gpus to be a power of 2 (:218-229); this engine
  // is one GPU by design
  if (n_gpus != 1) return DMSIM_ERR_UNSUPPORTED;
  if (n_qubits < 1 || n_qubits > 17) return DMSIM_ERR_ARG;
  dmsim_sim* s = new (std::nothrow) dmsim_sim;
  if (!s) return DMSIM_ERR_OOM;
  s->n = n_qubits;
  s->dim = 1ull << n_qubits;
  s->N = s->dim * s->dim;
  try {
    DM_CUDA(cudaGetDevice(&s->device));
    DM_CUDA(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device));
    DM_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    DM_CUDA(cudaEventCreate(&s->ev0));
    DM_CUDA(cudaEventCreate(&s->ev1));
    DM_CUDA(cudaMalloc(&s->d_diag, s->dim * sizeof(double)));
    DM_CUDA(cudaMalloc(&s->d_acc, 8 * sizeof(double)));
    DM_CUDA(cudaMalloc(&s->d_err, 16));
    DM_CUDA(cudaMemset(s->d_err, 0, 16));
    // rho is allocated on first use so that complex64 can be chosen first
    // (17 qubits fit only in complex64); FP64 up to 16 qubits is allocated now
    if (n_qubits <= 16) ensure_state(s);
  } catch (const DmError& e) {
    int code = e.code;
    dmsim_destroy(s);
    return code;
  }
  *out = s;
  return DMSIM_OK;
}

int dmsim_destroy(dmsim_handle s) {
  if (!s) return DMSIM_ERR_ARG;
  if (s->stream) cudaStreamSynchronize(s->stream);
  clear_circuit(s);
  free_state(s);
  if (s->d_diag) cudaFree(s->d_diag);
  if (s->d_acc) cudaFree(s->d_acc);
  if (s->d_err) cudaFree(s->d_err);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return DMSIM_OK;
}

int dmsim_set_option(dmsim_handle s, int key, int64_t v) {
  DM_TRY(s, {
    switch (key) {
      case DMSIM_OPT_MODE:
        if (v != 0 && v != 1) throw DmError{DMSIM_ERR_ARG, "mode must be 0 or 1"};
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set the mode before upload()"};
        s->mode = (int)v;
        break;
      case DMSIM_OPT_PRECISION: {
        if (v != 0 && v != 1) throw DmError{DMSIM_ERR_ARG, "precision must be 0 (FP64) or 1 (complex64)"};
        if (s->uploaded || !s->circuit.empty())
          throw DmError{DMSIM_ERR_STATE, "set the precision before appending gates"};
        if ((v == 1) != s->fp32) {
          free_state(s);
          s->fp32 = v == 1;
        }
        break;
      }
      case DMSIM_OPT_MAX_K:
        if (v < 1 || v > kMaxK) throw DmError{DMSIM_ERR_ARG, "max_k must be 1..4"};
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set max_k before upload()"};
        s->maxk = (int)v;
        break;
      case DMSIM_OPT_PLANNER:
        if (v != 0 && v != 1) throw DmError{DMSIM_ERR_ARG, "planner must be 0 or 1"};
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set the planner before upload()"};
        s->planner = (int)v;
        break;
      case DMSIM_OPT_RECORD: s->record = v != 0; break;
      case DMSIM_OPT_SEED: s->seed = v; break;
      case DMSIM_OPT_GRAPH:
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set graph replay before upload()"};
        s->graph_on = v != 0;
        break;
      case DMSIM_OPT_VERBOSE: s->verbose = v != 0; break;
      case DMSIM_OPT_FUSED_ARITH:
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set the fused arithmetic before upload()"};
        s->fused_arith = v != 0;
        break;
      case DMSIM_OPT_PLAIN_ARITH:
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set the plain arithmetic before upload()"};
        s->plain_arith = v != 0;
        break;
      case DMSIM_OPT_DIRECT1:
        if (v != 0 && v != 1) throw DmError{DMSIM_ERR_ARG, "direct1 must be 0 or 1"};
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set the 1-qubit kernel option before upload()"};
        s->direct1 = (int)v;
        break;
      case DMSIM_OPT_TENSOR:
        if (v < 0 || v > 2) throw DmError{DMSIM_ERR_ARG, "tensor must be 0, 1 or 2"};
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set the tensor-core option before upload()"};
        s->tensor = (int)v;
        break;
      case DMSIM_OPT_RENORM:
        if (v < 0) throw DmError{DMSIM_ERR_ARG, "renorm interval must be >= 0"};
        if (s->uploaded) throw DmError{DMSIM_ERR_STATE, "set the renormalisation interval before upload()"};
        s->renorm = (int)v;
        break;
      default: throw DmError{DMSIM_ERR_ARG, "unknown option"};
    }
  });
}

int dmsim_get_option(dmsim_handle s, int key, int64_t* v) {
  DM_TRY(s, {
    if (!v) throw DmError{DMSIM_ERR_ARG, "null output"};
    switch (key) {
      case DMSIM_OPT_MODE: *v = s->mode; break;
      case DMSIM_OPT_PRECISION: *v = s->fp32 ? 1 : 0; break;
      case DMSIM_OPT_MAX_K: *v = s->maxk; break;
      case DMSIM_OPT_PLANNER: *v = s->planner; break;
      case DMSIM_OPT_RECORD: *v = s->record; break;
      case DMSIM_OPT_SEED: *v = s->seed; break;
      case DMSIM_OPT_GRAPH: *v = s->graph_on; break;
      case DMSIM_OPT_VERBOSE: *v = s->verbose; break;
      case DMSIM_OPT_FUSED_ARITH: *v = s->fused_arith; break;
      case DMSIM_OPT_RENORM: *v = s->renorm; break;
      case DMSIM_OPT_PLAIN_ARITH: *v = s->plain_arith; break;
      case DMSIM_OPT_TENSOR: *v = s->tensor; break;
      case DMSIM_OPT_DIRECT1: *v = s->direct1; break;
      default: throw DmError{DMSIM_ERR_ARG, "unknown option"};
    }
  });
}

int dmsim_append(dmsim_handle s, int op, const uint32_t qb[5], double theta, double phi, double lambda) {
  DM_TRY(s, {
    if (!qb) throw DmError{DMSIM_ERR_ARG, "null qubit array"};
    if (op < 0 || op >= N_REF_OPS) throw DmError{DMSIM_ERR_ARG, "unknown gate id " + std::to_string(op)};
    GateRec g;
    std::memset(&g, 0, sizeof g);
    g.op = op;
    for (int i = 0; i < 5; i++) g.qb[i] = qb[i];
    g.theta = theta;
    g.phi = phi;
    g.lambda = lambda;
    check_qubits(s, g);
    s->circuit.push_back(g);
  });
}

int dmsim_append_c1(dmsim_handle s, uint32_t q, const double m[8]) {
  DM_TRY(s, {
    if (!m) throw DmError{DMSIM_ERR_ARG, "null matrix"};
    GateRec g;
    std::memset(&g, 0, sizeof g);
    g.op = OP_C1;
    g.qb[0] = q;
    std::memcpy(g.m, m, 8 * sizeof(double));
    check_qubits(s, g);
    s->circuit.push_back(g);
  });
}

int dmsim_append_c2(dmsim_handle s, uint32_t q1, uint32_t q2, const double m[32]) {
  DM_TRY(s, {
    if (!m) throw DmError{DMSIM_ERR_ARG, "null matrix"};
    GateRec g;
    std::memset(&g, 0, sizeof g);
    g.op = OP_C2;
    g.qb[0] = q1;
    g.qb[1] = q2;
    std::memcpy(g.m, m, 32 * sizeof(double));
    check_qubits(s, g);
    s->circuit.push_back(g);
  });
}

namespace {
// Kraus operators -> the superoperator S = sum_i K_i (x) conj(K_i) in the pass
// sub-index order (bit i <-> qubit q[i]); the caller's 2-qubit matrices use the
// C2 basis order (index 2*bit(q1) + bit(q2)), so the two bits are swapped here.
void append_kraus(dmsim_sim* s, uint32_t nq, const uint32_t q[2], uint32_t nk, const cplx* kraus) {
  if (nq < 1 || nq > 2) throw DmError{DMSIM_ERR_ARG, "channels act on 1 or 2 qubits"};
  if (nk < 1 || nk > 16) throw DmError{DMSIM_ERR_ARG, "1 to 16 Kraus operators"};
  GateRec g;
  std::memset(&g, 0, sizeof g);
  g.op = OP_CHANNEL;
  g.nq = (int)nq;
  if (nq == 1) g.qb[0] = q[0];
  else {
    g.qb[0] = q[1];  // pass sub-index bit 0 <-> the caller's second qubit
    g.qb[1] = q[0];
  }
  check_qubits(s, g);
  const int D = 1 << nq, DD = D * D;
  auto sub = [&](int idx) {  // caller's index -> pass sub-index
    if (nq == 1) return idx;
    return ((idx >> 1) & 1) | ((idx & 1) << 1);
  };
  Channel ch;
  std::memset(&ch, 0, sizeof ch);
  ch.K = (int)nq;
  for (uint32_t i = 0; i < nk; i++) {
    const cplx* Km = kraus + (size_t)i * DD;
    for (int a = 0; a < D; a++)
      for (int c = 0; c < D; c++)
        for (int b = 0; b < D; b++)
          for (int e = 0; e < D; e++) {
            const int A = sub(a), C = sub(c), B = sub(b), E = sub(e);
            ch.S[(A * D + B) * DD + (C * D + E)] += Km[a * D + c] * std::conj(Km[b * D + e]);
          }
  }
  g.chan = (int32_t)s->channels.size();
  s->channels.push_back(ch);
  s->circuit.push_back(g);
}
}  // namespace

int dmsim_append_channel(dmsim_handle s, uint32_t nq, const uint32_t q[2], uint32_t n_kraus, const double* kraus) {
  DM_TRY(s, {
    if (!q || !kraus) throw DmError{DMSIM_ERR_ARG, "null argument"};
    const int D = 1 << nq;
    std::vector<cplx> K((size_t)n_kraus * D * D);
    for (size_t i = 0; i < K.size(); i++) K[i] = cplx(kraus[2 * i], kraus[2 * i + 1]);
    append_kraus(s, nq, q, n_kraus, K.data());
  });
}

int dmsim_append_noise(dmsim_handle s, int kind, const uint32_t q[2], double p) {
  DM_TRY(s, {
    if (!q) throw DmError{DMSIM_ERR_ARG, "null qubits"};
    if (!(p >= 0.0 && p <= 1.0)) throw DmError{DMSIM_ERR_ARG, "noise strength must be in [0, 1]"};
    const cplx I(0, 1);
    const cplx id[4] = {1, 0, 0, 1}, X[4] = {0, 1, 1, 0}, Y[4] = {0, -I, I, 0}, Z[4] = {1, 0, 0, -1};
    std::vector<cplx> K;
    uint32_t nq = 1, nk = 0;
    auto add = [&](const cplx* m, double w) {
      for (int i = 0; i < 4; i++) K.push_back(std::sqrt(w) * m[i]);
      nk++;
    };
    switch (kind) {
      case DMSIM_NOISE_DEPOLARIZING:  // rho -> (1-p) rho + p I/2
        add(id, 1 - 3 * p / 4);
        add(X, p / 4);
        add(Y, p / 4);
        add(Z, p / 4);
        break;
      case DMSIM_NOISE_AMPLITUDE_DAMPING: {
        const cplx k0[4] = {1, 0, 0, std::sqrt(1 - p)}, k1[4] = {0, std::sqrt(p), 0, 0};
        add(k0, 1);
        add(k1, 1);
        break;
      }
      case DMSIM_NOISE_PHASE_DAMPING: {
        const cplx k0[4] = {1, 0, 0, std::sqrt(1 - p)}, k1[4] = {0, 0, 0, std::sqrt(p)};
        add(k0, 1);
        add(k1, 1);
        break;
      }
      case DMSIM_NOISE_BIT_FLIP:
        add(id, 1 - p);
        add(X, p);
        break;
      case DMSIM_NOISE_PHASE_FLIP:
        add(id, 1 - p);
        add(Z, p);
        break;
      case DMSIM_NOISE_DEPOLARIZING2: {  // rho -> (1-p) rho + p I/4 on two qubits
        nq = 2;
        const cplx* P[4] = {id, X, Y, Z};
        for (int i = 0; i < 4; i++)
          for (int j = 0; j < 4; j++) {
            const double w = (i == 0 && j == 0) ? 1 - 15 * p / 16 : p / 16;
            for (int a = 0; a < 4; a++)
              for (int c = 0; c < 4; c++) K.push_back(std::sqrt(w) * P[i][(a >> 1) * 2 + (c >> 1)] * P[j][(a & 1) * 2 + (c & 1)]);
            nk++;
          }
        break;
      }
      default: throw DmError{DMSIM_ERR_ARG, "unknown noise kind"};
    }
    append_kraus(s, nq, q, nk, K.data());
  });
}

int dmsim_upload(dmsim_handle s) { DM_TRY(s, upload(s)); }
int dmsim_run(dmsim_handle s) { DM_TRY(s, run(s)); }
int dmsim_clear_circuit(dmsim_handle s) { DM_TRY(s, clear_circuit(s)); }
int dmsim_reset_dm(dmsim_handle s) { DM_TRY(s, reset_dm(s)); }
int dmsim_reset(dmsim_handle s) {
  DM_TRY(s, {
    clear_circuit(s);
    reset_dm(s);
  });
}

int dmsim_measure(dmsim_handle s, uint32_t rep, const double* uniforms, uint64_t* out) {
  DM_TRY(s, {
    if (!out && rep) throw DmError{DMSIM_ERR_ARG, "null output"};
    const std::vector<double> d = host_diag(s);
    // sequential FP64 prefix of |Re rho_ii| (:527-533)
    std::vector<double> scan(s->dim + 1);
    scan[0] = 0;
    for (uint64_t i = 1; i < s->dim + 1; i++) scan[i] = scan[i - 1] + std::fabs(d[i - 1]);
    std::vector<double> u(rep);
    if (uniforms) {
      std::memcpy(u.data(), uniforms, rep * sizeof(double));
    } else {
      // srand(RAND_SEED) + rand()/RAND_MAX (:534-538), RAND_SEED = time(0) by default
      srand(s->seed >= 0 ? (unsigned)s->seed : (unsigned)time(0));
      for (uint32_t i = 0; i < rep; i++) u[i] = (double)rand() / (double)RAND_MAX;
    }
    for (uint32_t i = 0; i < rep; i++) {
      // the reference's linear search returns the j with scan[j] <= r <
      // scan[j+1] (0 if none); scan is non-decreasing, so that j is the one
      // before the first entry greater than r.
      const double r = u[i];
      const auto it = std::upper_bound(scan.begin(), scan.end(), r);
      uint64_t res = 0;
      if (it != scan.begin() && it != scan.end()) res = (uint64_t)(it - scan.begin()) - 1;
      out[i] = res;
    }
    if (std::fabs(scan[s->dim] - 1.0) > 1e-3)  // ERROR_BAR (src/config.hpp:53)
      fprintf(stderr, "Sum of probability along diag is far from 1.0 with %lf\n", scan[s->dim]);
  });
}

int dmsim_get_dm(dmsim_handle s, double* re, double* im) {
  DM_TRY(s, {
    if (!re || !im) throw DmError{DMSIM_ERR_ARG, "null buffer"};
    ensure_state(s);
    if (!s->fp32) {
      DM_CUDA(cudaMemcpyAsync(re, s->d_re, s->N * 8, cudaMemcpyDeviceToHost, s->stream));
      DM_CUDA(cudaMemcpyAsync(im, s->d_im, s->N * 8, cudaMemcpyDeviceToHost, s->stream));
      DM_CUDA(cudaStreamSynchronize(s->stream));
    } else {
      std::vector<float> tmp(s->N);
      DM_CUDA(cudaMemcpy(tmp.data(), s->d_re, s->N * 4, cudaMemcpyDeviceToHost));
      for (uint64_t i = 0; i < s->N; i++) re[i] = tmp[i];
      DM_CUDA(cudaMemcpy(tmp.data(), s->d_im, s->N * 4, cudaMemcpyDeviceToHost));
      for (uint64_t i = 0; i < s->N; i++) im[i] = tmp[i];
    }
  });
}

int dmsim_set_dm(dmsim_handle s, const double* re, const double* im) {
  DM_TRY(s, {
    if (!re || !im) throw DmError{DMSIM_ERR_ARG, "null buffer"};
    ensure_state(s);
    if (!s->fp32) {
      DM_CUDA(cudaMemcpyAsync(s->d_re, re, s->N * 8, cudaMemcpyHostToDevice, s->stream));
      DM_CUDA(cudaMemcpyAsync(s->d_im, im, s->N * 8, cudaMemcpyHostToDevice, s->stream));
      DM_CUDA(cudaStreamSynchronize(s->stream));
    } else {
      std::vector<float> tmp(s->N);
      for (uint64_t i = 0; i < s->N; i++) tmp[i] = (float)re[i];
      DM_CUDA(cudaMemcpy(s->d_re, tmp.data(), s->N * 4, cudaMemcpyHostToDevice));
      for (uint64_t i = 0; i < s->N; i++) tmp[i] = (float)im[i];
      DM_CUDA(cudaMemcpy(s->d_im, tmp.data(), s->N * 4, cudaMemcpyHostToDevice));
    }
  });
}

int dmsim_get_diag(dmsim_handle s, double* diag) {
  DM_TRY(s, {
    if (!diag) throw DmError{DMSIM_ERR_ARG, "null buffer"};
    const std::vector<double> d = host_diag(s);
    std::memcpy(diag, d.data(), s->dim * sizeof(double));
  });
}

int dmsim_dump(dmsim_handle s, char* buf, size_t len, size_t* needed) {
  DM_TRY(s, {
    // Gate::dump (:170-176): NAME(qb0,qb1,qb2,qb3,qb4,theta,phi,lambda);
    std::stringstream ss;
    for (const GateRec& g : s->circuit) {
      const char* name = g.op == OP_C1 ? "C1" : g.op == OP_C2 ? "C2" : g.op == OP_CHANNEL ? "CHANNEL" : kOpNames[g.op];
      ss << name << "(" << g.qb[0] << "," << g.qb[1] << "," << g.qb[2] << "," << g.qb[3] << "," << g.qb[4] << ","
         << g.theta << "," << g.phi << "," << g.lambda << ");" << std::endl;
    }
    const std::string str = ss.str();
    if (needed) *needed = str.size() + 1;
    if (buf && len > 0) {
      const size_t c = std::min(len - 1, str.size());
      std::memcpy(buf, str.data(), c);
      buf[c] = 0;
    }
  });
}

int dmsim_n_qubits(dmsim_handle s, uint32_t* n) {
  DM_TRY(s, {
    if (!n) throw DmError{DMSIM_ERR_ARG, "null output"};
    *n = s->n;
  });
}

int dmsim_n_gates(dmsim_handle s, uint32_t* n) {
  DM_TRY(s, {
    if (!n) throw DmError{DMSIM_ERR_ARG, "null output"};
    *n = (uint32_t)s->circuit.size();
  });
}

int dmsim_plan_stats(dmsim_handle s, uint32_t* n_passes, uint32_t* n_basic) {
  DM_TRY(s, {
    if (n_passes) *n_passes = (uint32_t)s->passes.size();
    if (n_basic) *n_basic = s->n_basic;
  });
}

int dmsim_upload_bytes(dmsim_handle s, uint64_t* bytes) {
  DM_TRY(s, {
    if (!bytes) throw DmError{DMSIM_ERR_ARG, "null output"};
    *bytes = (uint64_t)s->desc_bytes;
  });
}

int dmsim_last_timings(dmsim_handle s, double out[3]) {
  DM_TRY(s, {
    if (!out) throw DmError{DMSIM_ERR_ARG, "null output"};
    out[0] = s->last_ms;
    out[1] = (double)s->passes.size();
    out[2] = s->last_bytes;
  });
}

int dmsim_pass_records(dmsim_handle s, double* out, uint32_t cap, uint32_t* count) {
  DM_TRY(s, {
    if (count) *count = (uint32_t)s->records.size();
    if (out)
      for (uint32_t i = 0; i < cap && i < s->records.size(); i++) {
        const PassRecord& r = s->records[i];
        double* o = out + DMSIM_PASS_RECORD * i;
        o[0] = r.feat.K;
        o[1] = r.feat.cls;
        o[2] = r.feat.nnz;
        o[3] = r.feat.max_lo_bit;
        o[4] = r.feat.min_hi_bit;
        o[5] = r.feat.n;
        o[6] = r.ms;
        o[7] = r.bytes;
        o[8] = r.feat.tc;
        o[9] = r.grid;
      }
  });
}

int dmsim_pure_metrics(dmsim_handle s, const double* psi_re, const double* psi_im, double out[4]) {
  DM_TRY(s, {
    if (!psi_re || !psi_im || !out) throw DmError{DMSIM_ERR_ARG, "null buffer"};
    ensure_state(s);
    double* d_psi = nullptr;
    DM_CUDA(cudaMalloc(&d_psi, 2 * s->dim * sizeof(double)));
    cudaError_t e = cudaMemcpyAsync(d_psi, psi_re, s->dim * 8, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_psi + s->dim, psi_im, s->dim * 8, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = launch_pure_metrics(s->d_re, s->d_im, s->fp32, d_psi, d_psi + s->dim, (int)s->n, s->d_acc, s->sms, s->stream);
    double acc[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(acc, s->d_acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d_psi);
    if (e != cudaSuccess) throw DmError{DMSIM_ERR_CUDA, std::string("pure_metrics: ") + cudaGetErrorString(e)};
    out[0] = acc[0];
    out[1] = acc[1];
    out[2] = std::sqrt(acc[2]);
    out[3] = std::sqrt(acc[3]);
  });
}

int dmsim_compare_states(dmsim_handle a, dmsim_handle b, double out[2]) {
  DM_TRY(a, {
    if (!b || !out) throw DmError{DMSIM_ERR_ARG, "null argument"};
    if (a->N != b->N) throw DmError{DMSIM_ERR_ARG, "states differ in size"};
    ensure_state(a);
    ensure_state(b);
    DM_CUDA(cudaStreamSynchronize(b->stream));
    DM_CUDA(launch_compare(a->d_re, a->d_im, b->d_re, b->d_im, a->fp32, b->fp32, a->N, a->d_acc, a->sms, a->stream));
    double acc[2] = {0, 0};
    DM_CUDA(cudaMemcpyAsync(acc, a->d_acc, 2 * sizeof(double), cudaMemcpyDeviceToHost, a->stream));
    DM_CUDA(cudaStreamSynchronize(a->stream));
    out[0] = std::sqrt(acc[0]);
    out[1] = std::sqrt(acc[1]);
  });
}

int dmsim_alloc_host(size_t bytes, void** out) {
  if (!out) return DMSIM_ERR_ARG;
  *out = nullptr;
  cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    *out = nullptr;
    return e == cudaErrorMemoryAllocation ? DMSIM_ERR_OOM : DMSIM_ERR_CUDA;
  }
  return DMSIM_OK;
}

int dmsim_free_host(void* p) {
  if (!p) return DMSIM_ERR_ARG;
  return cudaFreeHost(p) == cudaSuccess ? DMSIM_OK : DMSIM_ERR_CUDA;
}

int dmsim_pure_metrics_noalloc(dmsim_handle s, const double* psi_re, const double* psi_im, double out[4]) {
  if (!s) return DMSIM_ERR_ARG;
  if (!psi_re || !psi_im || !out) {
    s->err = "dmsim_pure_metrics_noalloc: null argument";
    return DMSIM_ERR_ARG;
  }
  if (s->n > (uint32_t)kNoAllocMaxQubits) {
    s->err = "dmsim_pure_metrics_noalloc: the state has more than 16 qubits, beyond its static scratch of 2^16 "
             "amplitudes; use dmsim_pure_metrics";
    return DMSIM_ERR_ARG;
  }
  if (!s->d_re) {  // allocating rho here would defeat the purpose
    s->err = "dmsim_pure_metrics_noalloc: rho is not allocated yet";
    return DMSIM_ERR_STATE;
  }
  cudaError_t e = cudaSetDevice(s->device);
  if (e == cudaSuccess) e = pure_metrics_noalloc(s->d_re, s->d_im, s->fp32, psi_re, psi_im, (int)s->n, s->sms, s->stream, out);
  if (e != cudaSuccess) {
    s->err = std::string("dmsim_pure_metrics_noalloc: ") + cudaGetErrorString(e);
    return DMSIM_ERR_CUDA;
  }
  s->err.clear();
  return DMSIM_OK;
}

int dmsim_device_state(dmsim_handle s, void** re, void** im) {
  DM_TRY(s, {
    ensure_state(s);
    if (re) *re = s->d_re;
    if (im) *im = s->d_im;
  });
}

int dmsim_plan_inspect(uint32_t n_qubits, const int32_t* ops, const uint32_t* qubits, const double* params,
                       const double* mats, uint32_t ngates, int mode, int max_k, int planner, double* out, uint32_t cap,
                       uint32_t* npasses) {
  if (!ops || !qubits || !params || n_qubits < 1 || n_qubits > 30 || max_k < 1 || max_k > kMaxK) return DMSIM_ERR_ARG;
  try {
    std::vector<Basic> basics;
    for (uint32_t i = 0; i < ngates; i++) {
      GateRec g;
      std::memset(&g, 0, sizeof g);
      g.op = ops[i];
      for (int k = 0; k < 5; k++) g.qb[k] = qubits[5 * i + k];
      g.theta = params[3 * i];
      g.phi = params[3 * i + 1];
      g.lambda = params[3 * i + 2];
      if (mats) std::memcpy(g.m, mats + 32 * i, 32 * sizeof(double));
      const int ar = gate_arity(g.op);
      if (ar == 0) return DMSIM_ERR_ARG;
      for (int k = 0; k < ar; k++)
        if (g.qb[k] >= n_qubits) return DMSIM_ERR_ARG;
      decompose(g, basics);
    }
    bool has_rlin = false;
    for (const Basic& b : basics) has_rlin |= b.kind == BK_RLIN;
    std::vector<PassSpec> specs;
    if (has_rlin) specs = plan_reference_order(basics);
    else if (mode == 0) specs = plan_plain(basics);
    else if (planner == 1) {
      std::lock_guard<std::mutex> lock(cost_model_mutex());
      CostModel& m = global_cost_model();
      if (!m.ready) load_default_cost_model();
      if (!m.ready) return DMSIM_ERR_STATE;
      std::string err;
      specs = plan_learned(basics, (int)n_qubits, max_k, AR_DF64, true, m, nullptr, err);
      if (!err.empty()) return DMSIM_ERR_CUDA;
    } else specs = plan_greedy(basics, max_k);
    if (npasses) *npasses = (uint32_t)specs.size();
    if (out)
      for (uint32_t i = 0; i < cap && i < specs.size(); i++) {
        const PassSpec& p = specs[i];
        double* o = out + (size_t)DMSIM_PASS_REC * i;
        std::memset(o, 0, DMSIM_PASS_REC * sizeof(double));
        o[0] = p.K;
        o[1] = p.cls;
        o[2] = p.nbasic;
        o[3] = p.nnz;
        for (int k = 0; k < p.K; k++) o[4 + k] = p.q[k];
        o[10] = (mode == 1 && tc_choose(p, (int)n_qubits, 1, AR_DF64)) ? 1 : 0;
        o[8] = p.ket_only ? 1 : 0;
        o[9] = p.transpose ? 1 : 0;
        if (p.transpose) continue;
        if (p.rlin) {
          std::memcpy(o + 16, p.rl, 16 * sizeof(double));
          std::memcpy(o + 528, p.rlb, 16 * sizeof(double));
        } else {
          const int D = 1 << p.K;
          for (int j = 0; j < D * D; j++) {
            o[16 + 2 * j] = p.U[j].real();
            o[16 + 2 * j + 1] = p.U[j].imag();
            o[528 + 2 * j] = p.V[j].real();
            o[528 + 2 * j + 1] = p.V[j].imag();
          }
        }
      }
  } catch (...) {
    return DMSIM_ERR_ARG;
  }
  return DMSIM_OK;
}

// ---------------------------------------------------------------- cost model
namespace {
// Random circuit from the 29-entry mixed table (mt19937_64), in engine form.
void random_table_circuit(uint32_t n, uint32_t ngates, std::mt19937_64& rng, std::vector<GateRec>& out) {
  static const int table[] = {2, 1, 0, 13, 14, 15, 8, 9, 11, 5, 6, 7, 3, 17, 16, 19, 18, 22, 23, 24, 25, 26, 27, 37, 28,
                              20, 21, 31, 33};
  std::uniform_int_distribution<int> pick(0, (int)(sizeof(table) / sizeof(table[0])) - 1);
  std::uniform_real_distribution<double> ang(0.0, 6.283185307179586);
  for (uint32_t i = 0; i < ngates; i++) {
    GateRec g;
    std::memset(&g, 0, sizeof g);
    int op = table[pick(rng)];
    while (gate_arity(op) > (int)n) op = table[pick(rng)];
    g.op = op;
    std::vector<uint32_t> qs(n);
    for (uint32_t q = 0; q < n; q++) qs[q] = q;
    std::shuffle(qs.begin(), qs.end(), rng);
    for (int k = 0; k < gate_arity(op); k++) g.qb[k] = qs[k];
    g.theta = ang(rng);
    g.phi = ang(rng);
    g.lambda = ang(rng);
    out.push_back(g);
  }
}
}  // namespace

int dmsim_cost_collect(uint32_t n, uint32_t n_circuits, uint32_t gates, uint64_t seed, int arith, double* feats,
                       double* ms, uint32_t cap, uint32_t* count) {
  if (!count || n < 2 || n > 16 || arith < AR_FP64 || arith > AR_DF64) return DMSIM_ERR_ARG;
  *count = 0;
  dmsim_handle h = nullptr;
  int st = dmsim_create(n, 1, &h);
  if (st == DMSIM_OK && arith == AR_FP32) st = dmsim_set_option(h, DMSIM_OPT_PRECISION, 1);  // complex64 state
  if (st != DMSIM_OK) {
    dmsim_destroy(h);
    return st;
  }
  std::mt19937_64 rng(seed);
  uint32_t got = 0;
  try {
    h->record = 1;
    h->graph_on = 0;
    const int widths[] = {1, 2, 3, 4};
    const int caps[] = {kMaxD, 8, 4, 2};
    for (uint32_t c = 0; c < n_circuits; c++) {
      std::vector<GateRec> circ;
      random_table_circuit(n, gates, rng, circ);
      std::vector<Basic> basics;
      for (const GateRec& g : circ) decompose(g, basics);
      for (int k : widths)
        for (int rc : caps) {
          if (rc != kMaxD && rc >= (1 << k)) continue;
          std::vector<PassSpec> specs = k == 1 ? plan_plain(basics) : plan_greedy(basics, k, rc);
          bool any_tc = false;
          for (const PassSpec& p : specs) any_tc |= tc_eligible(p, (int)n);
          // double-float plans are timed on the FP32 pipe and, where passes
          // can run there, on the tensor cores
          const int variants = any_tc ? 2 : 1;
          for (int v = 0; v < variants; v++) {
            h->tensor = v == 1 ? 2 : 0;
            upload_specs(h, specs, (uint32_t)basics.size(), arith);
            h->uploaded = true;
            run(h);
            for (const PassRecord& r : h->records) {
              if (r.feat.K == 0) continue;  // format conversions are not passes
              if (v == 1 && !r.feat.tc) continue;  // already timed in the first variant
              if (got < cap && feats && ms) {
                float x[kMlpIn];
                pass_features(r.feat, x);
                for (int i = 0; i < kMlpIn; i++) feats[(size_t)got * kMlpIn + i] = x[i];
                ms[got] = r.ms;
              }
              got++;
            }
            clear_circuit(h);
          }
          h->circuit.clear();
          if (k == 1) break;
        }
    }
  } catch (const DmError& e) {
    dmsim_destroy(h);
    return e.code;
  }
  dmsim_destroy(h);
  *count = got;
  return DMSIM_OK;
}

int dmsim_cost_train(const double* feats, const double* ms, uint32_t count, uint32_t steps, double lr, uint64_t seed,
                     double loss[2]) {
  if (!feats || !ms || count == 0) return DMSIM_ERR_ARG;
  std::vector<float> X((size_t)count * kMlpIn), Y(count);
  for (size_t i = 0; i < X.size(); i++) X[i] = (float)feats[i];
  for (uint32_t i = 0; i < count; i++) Y[i] = (float)ms[i];
  std::lock_guard<std::mutex> lock(cost_model_mutex());
  CostModel& m = global_cost_model();
  cost_model_init(m, seed);
  float l[2] = {0, 0};
  std::string err;
  if (!cost_model_train(m, X, Y, (int)steps, (float)lr, l, err)) {
    fprintf(stderr, "dmsim_cost_train: %s\n", err.c_str());
    return DMSIM_ERR_CUDA;
  }
  if (loss) {
    loss[0] = l[0];
    loss[1] = l[1];
  }
  return DMSIM_OK;
}

int dmsim_cost_predict(const double* feats, uint32_t count, double* out_ms) {
  if (!feats || !out_ms) return DMSIM_ERR_ARG;
  std::lock_guard<std::mutex> lock(cost_model_mutex());
  CostModel& m = global_cost_model();
  if (!m.ready) load_default_cost_model();
  if (!m.ready) return DMSIM_ERR_STATE;
  std::vector<float> X((size_t)count * kMlpIn), Y;
  for (size_t i = 0; i < X.size(); i++) X[i] = (float)feats[i];
  std::string err;
  if (!cost_model_predict(m, X, Y, err)) return DMSIM_ERR_CUDA;
  for (uint32_t i = 0; i < count; i++) out_ms[i] = Y[i];
  return DMSIM_OK;
}

int dmsim_cost_save(const char* path) {
  std::lock_guard<std::mutex> lock(cost_model_mutex());
  if (!path || !global_cost_model().ready) return DMSIM_ERR_STATE;
  return cost_model_save(global_cost_model(), path) ? DMSIM_OK : DMSIM_ERR_ARG;
}

int dmsim_cost_load(const char* path) {
  if (!path) return DMSIM_ERR_ARG;
  std::lock_guard<std::mutex> lock(cost_model_mutex());
  return cost_model_load(global_cost_model(), path) ? DMSIM_OK : DMSIM_ERR_ARG;
}

int dmsim_mlp_forward(const float* params, const float* X, uint32_t B, float* y) {
  if (!params || !X || !y) return DMSIM_ERR_ARG;
  float *dp = nullptr, *dX = nullptr, *dy = nullptr;
  cudaError_t e = cudaMalloc(&dp, kMlpParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dX, (size_t)std::max<uint32_t>(B, 1) * kMlpIn * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dy, (size_t)std::max<uint32_t>(B, 1) * 4);
  if (e == cudaSuccess) e = cudaMemcpy(dp, params, kMlpParams * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dX, X, (size_t)B * kMlpIn * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = mlp_forward(dp, dX, (int)B, dy, 0);
  if (e == cudaSuccess) e = cudaMemcpy(y, dy, (size_t)B * 4, cudaMemcpyDeviceToHost);
  cudaFree(dp);
  cudaFree(dX);
  cudaFree(dy);
  return e == cudaSuccess ? DMSIM_OK : DMSIM_ERR_CUDA;
}

int dmsim_mlp_grad(const float* params, const float* X, const float* T, uint32_t B, float* grad, float* loss) {
  if (!params || !X || !T || !grad || !loss) return DMSIM_ERR_ARG;
  float *dp = nullptr, *dX = nullptr, *dT = nullptr, *dg = nullptr, *dl = nullptr;
  cudaError_t e = cudaMalloc(&dp, kMlpParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dX, (size_t)std::max<uint32_t>(B, 1) * kMlpIn * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dT, (size_t)std::max<uint32_t>(B, 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dg, kMlpParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dl, 4);
  if (e == cudaSuccess) e = cudaMemcpy(dp, params, kMlpParams * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dX, X, (size_t)B * kMlpIn * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dT, T, (size_t)B * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = mlp_grad(dp, dX, dT, (int)B, dg, dl, 0);
  if (e == cudaSuccess) e = cudaMemcpy(grad, dg, kMlpParams * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(loss, dl, 4, cudaMemcpyDeviceToHost);
  cudaFree(dp);
  cudaFree(dX);
  cudaFree(dT);
  cudaFree(dg);
  cudaFree(dl);
  return e == cudaSuccess ? DMSIM_OK : DMSIM_ERR_CUDA;
}

int dmsim_plan_predicted_ms(dmsim_handle s, double* ms) {
  DM_TRY(s, {
    if (!ms) throw DmError{DMSIM_ERR_ARG, "null output"};
    *ms = s->predicted_ms;
  });
}

const char* dmsim_last_error(dmsim_handle s) { return s ? s->err.c_str() : "null handle"; }

const char* dmsim_status_string(int st) {
  switch (st) {
    case DMSIM_OK: return "ok";
    case DMSIM_ERR_ARG: return "invalid argument";
    case DMSIM_ERR_STATE: return "call out of order";
    case DMSIM_ERR_OOM: return "out of memory";
    case DMSIM_ERR_CUDA: return "CUDA error";
    case DMSIM_ERR_TIMEOUT: return "device wait timed out";
    case DMSIM_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

}  // extern "C"

namespace dmg {

cudaError_t sim_enqueue(dmsim_handle s, cudaStream_t st, std::string& err) {
  if (!s || !s->uploaded) {
    err = "sim_enqueue: no uploaded plan";
    return cudaErrorInvalidValue;
  }
  try {
    DM_CUDA(launch_set_zero_state(s->d_re, s->d_im, s->N, s->fp32, st));
    enqueue_passes(s, false, st);
  } catch (const DmError& e) {
    err = e.msg;
    return cudaErrorUnknown;
  }
  return cudaSuccess;
}

double sim_plan_bytes(dmsim_handle s) {
  double t = 0;
  for (const PassInfo& p : s->passes) t += p.bytes;
  return t;
}

cudaError_t sim_take_error(dmsim_handle s, int* flag) {
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h) e = cudaMemset(s->d_err, 0, sizeof(int));
  *flag = h;
  return e;
}

}  // namespace dmg
