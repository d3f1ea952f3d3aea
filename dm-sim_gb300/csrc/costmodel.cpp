// costmodel.cpp -- the learned pass-time model (host side) and the planner that
// uses it.  Training and inference run on the GPU through mlp.cu; the host only
// builds feature vectors, moves them and reads the loss.
#include "costmodel.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <thread>

namespace dmg {

void pass_features(const PassFeatures& f, float* x) {
  const double nb = 2.0 * f.n;
  for (int i = 0; i < kMlpIn; i++) x[i] = 0.f;
  x[0] = f.K / 4.0f;
  // x[1..6] class one-hot (a channel pass counts as dense)
  const int cls = f.cls == CLS_SUPER ? CLS_DENSE : f.cls;
  if (cls >= 0 && cls <= CLS_RLIN) x[1 + cls] = 1.f;
  const int D = 1 << f.K;
  x[7] = (float)f.nnz / (float)(D * D);           // density of U
  x[8] = (float)f.nnz / (float)D / 16.f;          // nonzeros per row
  x[9] = (float)f.ld_frac;
  x[10] = (float)f.st_frac;
  x[11] = (float)((f.max_lo_bit + 1) / nb);
  x[12] = (float)(f.min_hi_bit / nb);
  x[13] = (float)(nb / 34.0);                     // log2 of the entry count
  x[14] = f.arith == 1 ? 1.f : (f.arith == 2 ? 0.5f : 0.f);  // FP32 / double-float / FP64
  // arithmetic volume (real operators need half the multiply-adds)
  x[15] = (float)((f.nnz / (double)D) * f.ld_frac * std::ldexp(1.0, (int)nb - 28) * (f.real && !f.tc ? 0.5 : 1.0));
  x[16] = f.tc ? 1.f : 0.f;                       // on the tensor cores (cost independent of the density)
}

// ln(4^n) of a pass from its features (x[13] = 2n / 34)
double log_entries(const float* x) { return std::nearbyint(x[13] * 34.0) * std::log(2.0); }

CostModel& global_cost_model() {
  static CostModel m;
  return m;
}

std::mutex& cost_model_mutex() {
  static std::mutex mu;
  return mu;
}

namespace {
constexpr uint32_t kMagic = 0x434d4d44;  // "DMMC"
constexpr uint32_t kVersion = 3;  // 3: targets are log time per state entry
}  // namespace

bool cost_model_save(const CostModel& m, const std::string& path) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  const uint32_t hdr[4] = {kMagic, kVersion, (uint32_t)kMlpIn, (uint32_t)kMlpParams};
  bool ok = fwrite(hdr, sizeof hdr, 1, f) == 1;
  ok = ok && fwrite(&m.y_mean, sizeof(float), 1, f) == 1 && fwrite(&m.y_std, sizeof(float), 1, f) == 1;
  ok = ok && fwrite(m.params, sizeof(float), kMlpParams, f) == (size_t)kMlpParams;
  fclose(f);
  return ok;
}

bool cost_model_load(CostModel& m, const std::string& path) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  uint32_t hdr[4];
  bool ok = fread(hdr, sizeof hdr, 1, f) == 1 && hdr[0] == kMagic;
  const uint32_t in = ok ? hdr[2] : 0;
  ok = ok && hdr[1] == kVersion && in == (uint32_t)kMlpIn;
  const uint32_t np = kMlpHidden * in + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;
  ok = ok && hdr[3] == np;
  CostModel t;
  std::vector<float> raw(ok ? np : 0);
  ok = ok && fread(&t.y_mean, sizeof(float), 1, f) == 1 && fread(&t.y_std, sizeof(float), 1, f) == 1;
  ok = ok && fread(raw.data(), sizeof(float), np, f) == (size_t)np;
  fclose(f);
  if (!ok) return false;
  // W1[j][0..in) then the rest of the layout unchanged
  for (int j = 0; j < kMlpHidden; j++)
    for (int k = 0; k < kMlpIn; k++) t.params[j * kMlpIn + k] = k < (int)in ? raw[j * in + k] : 0.f;
  std::copy(raw.begin() + kMlpHidden * in, raw.end(), t.params + kMlpHidden * kMlpIn);
  t.ready = true;
  m = t;
  return true;
}

void cost_model_init(CostModel& m, uint64_t seed) {
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  const int I = kMlpIn, H = kMlpHidden;
  int o = 0;
  for (int i = 0; i < H * I; i++) m.params[o++] = nd(rng) * std::sqrt(2.f / I);
  for (int i = 0; i < H; i++) m.params[o++] = 0.f;
  for (int i = 0; i < H * H; i++) m.params[o++] = nd(rng) * std::sqrt(2.f / H);
  for (int i = 0; i < H; i++) m.params[o++] = 0.f;
  for (int i = 0; i < H; i++) m.params[o++] = nd(rng) * std::sqrt(1.f / H);
  m.params[o++] = 0.f;
  m.y_mean = 0.f;
  m.y_std = 1.f;
  m.ready = false;
}

namespace {
struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, n); }
  float* f() { return static_cast<float*>(p); }
};
#define CM_CUDA(x)                                   \
  do {                                               \
    cudaError_t e_ = (x);                            \
    if (e_ != cudaSuccess) {                         \
      err = std::string(#x) + ": " + cudaGetErrorString(e_); \
      return false;                                  \
    }                                                \
  } while (0)
}  // namespace

bool cost_model_train(CostModel& m, const std::vector<float>& X, const std::vector<float>& ms, int steps, float lr,
                      float loss[2], std::string& err) {
  const int B = (int)ms.size();
  if (B == 0 || (int)X.size() != B * kMlpIn) {
    err = "empty or mismatched training set";
    return false;
  }
  // standardised targets: log of the time per state entry (the time of a
  // pass grows with the 4^n entries it sweeps; taking that out keeps the
  // network's job size-independent, so it extrapolates across qubit counts)
  std::vector<float> T(B);
  double mean = 0, var = 0;
  for (int i = 0; i < B; i++) {
    T[i] = (float)(std::log(std::max(ms[i], 1e-6f)) - log_entries(&X[(size_t)i * kMlpIn]));
    mean += T[i];
  }
  mean /= B;
  for (int i = 0; i < B; i++) var += (T[i] - mean) * (T[i] - mean);
  const double sd = std::sqrt(var / B) + 1e-6;
  for (int i = 0; i < B; i++) T[i] = (float)((T[i] - mean) / sd);
  m.y_mean = (float)mean;
  m.y_std = (float)sd;

  cudaStream_t s;
  CM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBuf dp, dX, dT, dg, dm, dv, dl;
  bool ok = true;
  auto fail = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && ok) {
      err = std::string(what) + ": " + cudaGetErrorString(e);
      ok = false;
    }
  };
  fail(dp.alloc(kMlpParams * 4), "alloc");
  fail(dX.alloc((size_t)B * kMlpIn * 4), "alloc");
  fail(dT.alloc((size_t)B * 4), "alloc");
  fail(dg.alloc(kMlpParams * 4), "alloc");
  fail(dm.alloc(kMlpParams * 4), "alloc");
  fail(dv.alloc(kMlpParams * 4), "alloc");
  fail(dl.alloc(4), "alloc");
  if (ok) {
    fail(cudaMemcpyAsync(dp.p, m.params, kMlpParams * 4, cudaMemcpyHostToDevice, s), "copy");
    fail(cudaMemcpyAsync(dX.p, X.data(), (size_t)B * kMlpIn * 4, cudaMemcpyHostToDevice, s), "copy");
    fail(cudaMemcpyAsync(dT.p, T.data(), (size_t)B * 4, cudaMemcpyHostToDevice, s), "copy");
    fail(cudaMemsetAsync(dm.p, 0, kMlpParams * 4, s), "memset");
    fail(cudaMemsetAsync(dv.p, 0, kMlpParams * 4, s), "memset");
  }
  for (int t = 1; ok && t <= steps; t++) {
    fail(mlp_grad(dp.f(), dX.f(), dT.f(), B, dg.f(), dl.f(), s), "mlp_grad");
    if (t == 1) {
      fail(cudaMemcpyAsync(&loss[0], dl.p, 4, cudaMemcpyDeviceToHost, s), "copy");
    }
    fail(mlp_adam(dp.f(), dg.f(), dm.f(), dv.f(), lr, t, s), "mlp_adam");
  }
  if (ok) {
    fail(mlp_grad(dp.f(), dX.f(), dT.f(), B, dg.f(), dl.f(), s), "mlp_grad");
    fail(cudaMemcpyAsync(&loss[1], dl.p, 4, cudaMemcpyDeviceToHost, s), "copy");
    fail(cudaMemcpyAsync(m.params, dp.p, kMlpParams * 4, cudaMemcpyDeviceToHost, s), "copy");
    fail(cudaStreamSynchronize(s), "sync");
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (ok) m.ready = true;
  return ok;
}

bool cost_model_predict(const CostModel& m, const std::vector<float>& X, std::vector<float>& ms, std::string& err) {
  const int B = (int)(X.size() / kMlpIn);
  ms.assign(B, 0.f);
  if (B == 0) return true;
  if (!m.ready) {
    err = "the cost model is not trained or loaded";
    return false;
  }
  cudaStream_t s;
  CM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBuf dp, dX, dy;
  bool ok = true;
  auto fail = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && ok) {
      err = std::string(what) + ": " + cudaGetErrorString(e);
      ok = false;
    }
  };
  fail(dp.alloc(kMlpParams * 4), "alloc");
  fail(dX.alloc((size_t)B * kMlpIn * 4), "alloc");
  fail(dy.alloc((size_t)B * 4), "alloc");
  if (ok) {
    fail(cudaMemcpyAsync(dp.p, m.params, kMlpParams * 4, cudaMemcpyHostToDevice, s), "copy");
    fail(cudaMemcpyAsync(dX.p, X.data(), (size_t)B * kMlpIn * 4, cudaMemcpyHostToDevice, s), "copy");
    fail(mlp_forward(dp.f(), dX.f(), B, dy.f(), s), "mlp_forward");
    fail(cudaMemcpyAsync(ms.data(), dy.p, (size_t)B * 4, cudaMemcpyDeviceToHost, s), "copy");
    fail(cudaStreamSynchronize(s), "sync");
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (!ok) return false;
  for (int i = 0; i < B; i++) ms[i] = (float)std::exp(ms[i] * m.y_std + m.y_mean + log_entries(&X[(size_t)i * kMlpIn]));
  return true;
}

std::vector<PassSpec> plan_learned(const std::vector<Basic>& basics, int n, int maxk, int arith, bool tensor,
                                   const CostModel& m, double* predicted_ms, std::string& err) {
  // candidate plans: the unfused plan, and greedy plans of every width up to
  // maxk under row-density caps.  Each candidate is planned and featurised on
  // its own host thread (features of every pass and of its tensor-core
  // variant where there is one), then one batched GPU inference scores all.
  struct Cand {
    int k, cap;
    std::vector<PassSpec> plan;
    std::vector<float> X;
    std::vector<int> pass_of;
    std::vector<char> is_tc;
  };
  std::vector<Cand> cands;
  cands.push_back({1, kMaxD, {}, {}, {}, {}});
  const int caps[] = {kMaxD, 8, 4, 2};
  for (int k = 2; k <= maxk; k++)
    for (int cap : caps) {
      if (cap >= (1 << k) && cap != kMaxD) continue;  // no effect at this width
      cands.push_back({k, cap, {}, {}, {}, {}});
    }
  // double-float state only: at 17 qubits the model (trained up to 16) picked
  // complex64 tensor passes that ran slower than the FP32 pipe (71.4 s against
  // 62.5 s for the circuit); complex64 tensor passes stay opt-in (option 2)
  // FP64 state: the FP64-width tensor passes (tensor64.cu)
  const bool tc_ok = tensor && (arith == 2 || arith == 0);
  auto work = [&](Cand& c) {
    c.plan = c.k == 1 ? plan_plain(basics) : plan_greedy(basics, c.k, c.cap);
    std::vector<unsigned char> buf(std::max(desc_size(kMaxK), std::max(tc_desc_bytes(kMaxK, 2), tc_desc_bytes(kMaxK, 0))));
    for (size_t i = 0; i < c.plan.size(); i++) {
      const PassSpec& p = c.plan[i];
      if (p.transpose) continue;
      for (int v = 0; v < 2; v++) {
        if (v == 1 && !(tc_ok && tc_eligible(p, n))) break;
        PassFeatures f;
        std::memset(&f, 0, sizeof f);
        if (v == 0) build_desc(p, n, buf.data(), &f, nullptr, nullptr);
        else build_tc_desc(p, n, buf.data(), &f, nullptr, nullptr, false, arith);
        f.arith = arith;
        f.tc = v;
        float x[kMlpIn];
        pass_features(f, x);
        c.X.insert(c.X.end(), x, x + kMlpIn);
        c.pass_of.push_back((int)i);
        c.is_tc.push_back((char)v);
      }
    }
  };
  {
    std::vector<std::thread> threads;
    for (size_t c = 1; c < cands.size(); c++) threads.emplace_back(work, std::ref(cands[c]));
    work(cands[0]);
    for (std::thread& t : threads) t.join();
  }
  std::vector<float> X;
  std::vector<int> owner, pass_of;
  std::vector<char> is_tc;
  for (size_t c = 0; c < cands.size(); c++) {
    X.insert(X.end(), cands[c].X.begin(), cands[c].X.end());
    pass_of.insert(pass_of.end(), cands[c].pass_of.begin(), cands[c].pass_of.end());
    is_tc.insert(is_tc.end(), cands[c].is_tc.begin(), cands[c].is_tc.end());
    owner.insert(owner.end(), cands[c].pass_of.size(), (int)c);
  }
  std::vector<float> ms;
  if (!cost_model_predict(m, X, ms, err)) return {};
  // per pass: the cheaper variant
  std::vector<std::vector<float>> best_ms(cands.size());
  std::vector<std::vector<char>> best_tc(cands.size());
  for (size_t c = 0; c < cands.size(); c++) {
    best_ms[c].assign(cands[c].plan.size(), -1.f);
    best_tc[c].assign(cands[c].plan.size(), 0);
  }
  for (size_t r = 0; r < ms.size(); r++) {
    float& b = best_ms[owner[r]][pass_of[r]];
    if (b < 0 || ms[r] < b) {
      b = ms[r];
      best_tc[owner[r]][pass_of[r]] = is_tc[r];
    }
  }
  std::vector<double> tot(cands.size(), 0.0);
  for (size_t c = 0; c < cands.size(); c++)
    for (float v : best_ms[c])
      if (v > 0) tot[c] += v;
  const size_t best = (size_t)(std::min_element(tot.begin(), tot.end()) - tot.begin());
  if (predicted_ms) *predicted_ms = tot[best];
  std::vector<PassSpec> plan = std::move(cands[best].plan);
  for (size_t i = 0; i < plan.size(); i++) plan[i].tc = tc_ok ? best_tc[best][i] : -1;
  return plan;
}

}  // namespace dmg
