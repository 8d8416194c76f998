/* The main.jl run through the C ABI alone (no Python, no Julia): two phases, test
   case 6 of HyperelasticityMPh.jl, path-conservative HLL, frozen ends, nx cells,
   the two-state fill of main.jl:99-106, max_steps steps. Prints the steps taken,
   the time and a checksum of the final state; exit status 0 on success.
   Usage: c_abi_example nx max_steps */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "hyperelastic.h"

static int check(int rc, const hyp_ctx* ctx, const char* what) {
  if (rc != HYP_OK) fprintf(stderr, "%s failed: %d (%s)\n", what, rc, ctx ? hyp_last_error(ctx) : "");
  return rc;
}

int main(int argc, char** argv) {
  const int64_t nx = argc > 1 ? atoll(argv[1]) : 1000;
  const int max_steps = argc > 2 ? atoi(argv[2]) : 100;
  const hyp_barton2009 barton = {8.93, 4.6, 3.9e-4, 300.0, 2.1, 1.0, 3.0, 2.0};  /* EquationsOfState.jl:90 */
  hyp_config cfg = {0};
  cfg.n_cells = nx;
  cfg.model = HYP_MODEL_MULTI;
  cfg.flux = HYP_FLUX_HLL;
  cfg.bc = HYP_BC_FROZEN;
  cfg.precision = HYP_PREC_FP64;
  cfg.x_length = 1.0;
  cfg.cfl = 0.6;
  cfg.eos[0] = barton;
  cfg.eos[1] = barton;
  cfg.eos[1].b0 = 2.1 * sqrt(0.1);
  double Ql[30], Qr[30];
  if (check(hyp_initial_states(&cfg, 6, Ql, Qr), NULL, "hyp_initial_states")) return 1;
  hyp_ctx* ctx = NULL;
  if (check(hyp_create(&cfg, &ctx), NULL, "hyp_create")) return 1;
  int rc = check(hyp_init_riemann(ctx, Ql, Qr), ctx, "hyp_init_riemann");
  int done = 0;
  double t = 0.0;
  if (!rc) rc = check(hyp_step(ctx, max_steps, INFINITY, &done, &t), ctx, "hyp_step");
  double* Q = malloc(sizeof(double) * 30 * (size_t)nx);
  if (!rc && Q) rc = check(hyp_download(ctx, Q, nx, 30), ctx, "hyp_download");
  if (!rc) {
    double sum = 0.0;
    for (int64_t k = 0; k < 30 * nx; ++k) sum += fabs(Q[k]);
    printf("steps %d t %.17g checksum %.17g\n", done, t, sum);
  }
  free(Q);
  hyp_destroy(ctx);
  return rc ? 1 : 0;
}
