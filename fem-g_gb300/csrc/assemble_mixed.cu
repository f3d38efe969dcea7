// Mixed-precision assembly (placeholder until the tcgen05 contraction lands).
#include "common.cuh"

extern "C" void mixedDestroy(fg_plan *plan) { (void)plan; }

extern "C" int fg_assemble_mixed(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency,
                                 const double *dirichlet, double *csr_values, double *rhs, void *stream, fg_err_report *report) {
  (void)plan; (void)terms; (void)n_terms; (void)frequency; (void)dirichlet; (void)csr_values; (void)rhs; (void)stream; (void)report;
  femg::setLastError("fg_assemble_mixed: not built yet");
  return FG_ERR_UNSUPPORTED;
}

extern "C" int fg_assemble_multi_freq(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, const double *omegas, int32_t n_freq,
                                      int32_t mixed, double *csr_values, void *stream) {
  (void)plan; (void)terms; (void)n_terms; (void)omegas; (void)n_freq; (void)mixed; (void)csr_values; (void)stream;
  femg::setLastError("fg_assemble_multi_freq: not built yet");
  return FG_ERR_UNSUPPORTED;
}

extern "C" int fg_batch_create(fg_plan *const *plans, const fg_term_desc *const *terms, const int32_t *n_terms, int32_t n_problems,
                               int32_t mixed, fg_batch **out) {
  (void)plans; (void)terms; (void)n_terms; (void)n_problems; (void)mixed;
  if (out) *out = nullptr;
  femg::setLastError("fg_batch_create: not built yet");
  return FG_ERR_UNSUPPORTED;
}

extern "C" int fg_batch_run(fg_batch *batch, double *const *csr_values, double *const *rhs, void *stream) {
  (void)batch; (void)csr_values; (void)rhs; (void)stream;
  return FG_ERR_UNSUPPORTED;
}

extern "C" void fg_batch_destroy(fg_batch *batch) { (void)batch; }
