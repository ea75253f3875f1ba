// Batched lambda paths and the serving loop.
#include <cstring>

#include "acdc_internal.cuh"

namespace {
int plain_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems, const double* lambdas,
               const acdc_batch_options* opt, acdc_batch_result* results, double* const* x_out) {
  for (int32_t i = 0; i < count; ++i) {
    acdc_problem* p = problems[i];
    if (!p || p->ctx != ctx) return acdc_set_error(ctx, ACDC_EINVAL, "problem from another context");
    acdc_settings s = p->s;
    s.gap_target = opt->gap_target;
    s.gap_relative = 1;
    s.max_epochs = opt->max_epochs;
    s.refresh_every = opt->refresh_every;
    if (opt->tau_override > 0) s.tau = opt->tau_override;
    int rc = acdc_problem_set_settings(p, &s);
    if (rc) return rc;
    for (int32_t k = 0; k < opt->path_len; ++k) {
      const double lam = lambdas[(size_t)i * opt->path_len + k];
      rc = acdc_problem_set_lambda(p, lam);
      if (rc) return rc;
      acdc_solve_result r;
      rc = acdc_solve(p, &r);
      if (rc) return rc;
      acdc_batch_result& out = results[(size_t)i * opt->path_len + k];
      std::memset(&out, 0, sizeof(out));
      out.eval = r.eval;
      out.lambda = lam;
      out.converged = r.converged;
      out.epochs = r.epochs;
      out.tau = s.tau;
    }
    if (x_out && x_out[i]) {
      rc = acdc_get_x(p, x_out[i]);
      if (rc) return rc;
    }
  }
  return ACDC_OK;
}
}  // namespace

extern "C" int acdc_batch_solve_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems,
                                     const double* lambdas, const acdc_batch_options* opt,
                                     acdc_batch_result* results, double* const* x_out) {
  if (!ctx || count < 0 || (count > 0 && (!problems || !lambdas || !results)) || !opt ||
      opt->path_len < 1 || opt->refresh_every < 1 || opt->max_epochs < 0)
    return acdc_set_error(ctx, ACDC_EINVAL, "invalid batch arguments");
  return plain_path(ctx, count, problems, lambdas, opt, results, x_out);
}

struct acdc_server {
  acdc_ctx* ctx;
};

extern "C" int acdc_server_create(acdc_ctx* ctx, const acdc_server_options* opt, acdc_server** out) {
  (void)opt;
  if (!ctx || !out) return ACDC_EINVAL;
  return acdc_set_error(ctx, ACDC_EUNSUPPORTED, "server not built yet");
}
extern "C" int acdc_server_submit(acdc_server* s, const acdc_request* req, int64_t* ticket) {
  (void)s; (void)req; (void)ticket;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_step(acdc_server* s, int32_t* pending) {
  (void)s; (void)pending;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_poll(acdc_server* s, int64_t ticket, acdc_request_result* res, double* x) {
  (void)s; (void)ticket; (void)res; (void)x;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_release(acdc_server* s, int64_t ticket) {
  (void)s; (void)ticket;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_destroy(acdc_server* s) {
  (void)s;
  return ACDC_EUNSUPPORTED;
}
