// costmodel.h -- learned pass-time model and the planner that uses it.
#pragma once
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "mlp.h"
#include "plan.h"

namespace dmg {

// Features of one pass for the cost model (kMlpIn floats, roughly in [0,1]).
void pass_features(const PassFeatures& f, float* out);

struct CostModel {
  bool ready = false;
  float params[kMlpParams];
  float y_mean = 0, y_std = 1;  // targets are standardised log(ms)
};

CostModel& global_cost_model();
// ln of the state entries a pass sweeps, from its features
double log_entries(const float* x);
// Held while the process-wide model is trained, loaded, saved or read.
std::mutex& cost_model_mutex();
bool cost_model_save(const CostModel& m, const std::string& path);
bool cost_model_load(CostModel& m, const std::string& path);
// He-initialised weights from a seed.
void cost_model_init(CostModel& m, uint64_t seed);

// GPU training (full batch Adam) on samples X (count x kMlpIn) and ms.
// Returns false with a message on a CUDA error; loss[0], loss[1] = initial, final MSE.
bool cost_model_train(CostModel& m, const std::vector<float>& X, const std::vector<float>& ms, int steps, float lr,
                      float loss[2], std::string& err);
// GPU inference: predicted ms per sample.
bool cost_model_predict(const CostModel& m, const std::vector<float>& X, std::vector<float>& ms, std::string& err);

// The learned planner: scores candidate plans (widths 1..maxk, row-density
// caps, and the unfused plan) with the model, returns the cheapest.
// arith: the arithmetic the chosen plan will run in (kernels.h Arith).
// With `tensor`, every pass that can run on the tensor cores is scored both
// ways and keeps the cheaper (PassSpec::tc).
std::vector<PassSpec> plan_learned(const std::vector<Basic>& basics, int n, int maxk, int arith, bool tensor,
                                   const CostModel& m,
                                   double* predicted_ms, std::string& err);

}  // namespace dmg
