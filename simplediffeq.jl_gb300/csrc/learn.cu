/* Learned schedule (placeholder until the MLP kernels land). */
#include "ode_host.h"

namespace gbode {

struct Model {};

void model_free(Model* m) { delete m; }
bool model_ready(const Model* m, const ode_solve_args* a) { return false; }
float model_dt0_safety(const Model* m) { return 1.0f; }
bool model_seed_dt0(const Model* m) { return false; }
int model_predict_device(ode_handle* h, const ode_solve_args* a, const KParams& kp, float* log_att, float* log_dt,
                         cudaStream_t s, int* launches) {
  return fail(h, ODE_ENOTSUP, "learned schedule not available");
}
int order_by_cost(ode_handle* h, const float* log_att, int64_t n, int* order, cudaStream_t s, int* launches) {
  return fail(h, ODE_ENOTSUP, "learned schedule not available");
}
int seed_dt0(ode_handle* h, const float* log_dt, int64_t n, float safety, double* dt0, cudaStream_t s,
             int* launches) {
  return fail(h, ODE_ENOTSUP, "learned schedule not available");
}

}  // namespace gbode

extern "C" {
void ode_learn_default_opts(ode_learn_opts* o) {
  if (!o) return;
  o->hidden = 64;
  o->epochs = 200;
  o->batch = 1024;
  o->lr = 3e-3f;
  o->seed = 1;
  o->seed_dt0 = 1;
  o->dt0_safety = 1.0f;
}
int ode_learn_fit(ode_handle* h, const ode_solve_args* a, const ode_learn_opts* opts, ode_learn_report* rep) {
  return gbode::fail(h, ODE_ENOTSUP, "learned schedule not available");
}
int ode_learn_predict(ode_handle* h, const ode_solve_args* a, float* log_attempts, float* log_dt_first) {
  return gbode::fail(h, ODE_ENOTSUP, "learned schedule not available");
}
}
