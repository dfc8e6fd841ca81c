/* c_driver.c -- the calcFrame loop of common/main.cu:310-635 as a plain C
 * program against the C ABI (include/fivonagi.h), built with gcc: the
 * app's parameters (parameters.h) from fv_default_params, the initial
 * values (init<TTT>), the run to each print time (calcFrame's
 * `while (T < Tprint)`), the state copied back for export (dataExport),
 * then per-step stats through the pipelined calls. Test infrastructure:
 * tests/test_gpu_c_driver.py runs it and compares its output with the
 * Python binding's run of the same steps.
 *
 * usage: c_driver NX NY NPRINT DTPRINT NPIPE OUT.bin
 * writes u1, u2, u3 (float32, NX*NY each) to OUT.bin and prints
 * "T n accepted rejected" on stdout. */
#include <stdio.h>
#include <stdlib.h>

#include "fivonagi.h"

static int check(fv_status s, const char *what) {
  if (s != FV_OK) {
    fprintf(stderr, "%s: status %d: %s\n", what, (int)s, fv_last_error_string());
    return 1;
  }
  return 0;
}

int main(int argc, char **argv) {
  if (argc != 7) {
    fprintf(stderr, "usage: %s NX NY NPRINT DTPRINT NPIPE OUT.bin\n", argv[0]);
    return 2;
  }
  fv_params p;
  if (check(fv_default_params(FV_APP_HIFU_BEAM, &p), "fv_default_params")) return 1;
  p.nx = atoi(argv[1]);
  p.ny = atoi(argv[2]);
  p.xmax = (double)(p.nx - 1) / 16.0;
  p.ymax = (double)(p.ny - 1) / 16.0;
  const int nprint = atoi(argv[3]);
  const double dtprint = atof(argv[4]);
  const int npipe = atoi(argv[5]);
  fv_handle *h = NULL;
  if (check(fv_create(&p, &h), "fv_create")) return 1;
  int rc = check(fv_init_state(h), "fv_init_state");
  fv_run_stats st;
  long long accepted = 0, rejected = 0;
  double tprint = -p.tide + dtprint;
  for (int k = 0; k < nprint && !rc; ++k, tprint += dtprint) {
    rc = check(fv_run_until(h, tprint, &st), "fv_run_until");
    accepted += st.accepted;
    rejected += st.rejected;
  }
  /* then every attempt's stats, the next attempt enqueued before each read */
  if (!rc && npipe > 0) rc = check(fv_steps_async(h, 1), "fv_steps_async");
  for (int k = 0; k < npipe && !rc; ++k) {
    if (k + 1 < npipe) rc = check(fv_steps_async(h, 1), "fv_steps_async");
    if (!rc) rc = check(fv_step_wait(h, &st), "fv_step_wait");
    accepted += st.accepted;
    rejected += st.rejected;
  }
  const size_t n = (size_t)p.nx * (size_t)p.ny;
  float *u = (float *)malloc(3 * n * sizeof(float));
  if (!u) rc = 1;
  if (!rc) rc = check(fv_get_state(h, u, u + n, u + 2 * n, 0), "fv_get_state");
  if (!rc && check(fv_get_stats(h, &st), "fv_get_stats")) rc = 1;
  if (!rc) {
    FILE *f = fopen(argv[6], "wb");
    if (!f || fwrite(u, sizeof(float), 3 * n, f) != 3 * n) rc = 1;
    if (f) fclose(f);
    printf("%.9g %d %lld %lld\n", st.T, st.n, accepted, rejected);
  }
  free(u);
  fv_destroy(h);
  return rc;
}
