/*
 * A plain C99 host of libtensorly_gb300.so: what a cgo, JNI or N-API binding
 * compiles against.  It touches only the calls that need no GPU (version,
 * default options, argument checks) and prints one line per check; the
 * pytest wrapper (tests/test_c_host.py) compiles, links and runs it.
 */
#include <stdio.h>
#include <string.h>

#include "tensorly_gb300.h"

static int failures = 0;

static void expect(int cond, const char* what) {
  printf("%s %s\n", cond ? "ok" : "FAIL", what);
  if (!cond) ++failures;
}

int main(void) {
  expect(tlgb_version() >= 100, "version");

  tlgb_cp_als_options opts;
  memset(&opts, 0xff, sizeof(opts));
  tlgb_cp_als_default_options(&opts);
  expect(opts.n_iter_max == 100 && opts.tol == 1e-8 && opts.precision == TLGB_PREC_NATIVE,
         "cp_als default options (parafac's n_iter_max and tol)");
  expect(opts.callback == NULL && opts.mttkrp_ms == NULL, "cp_als default hooks off");

  tlgb_tucker_options topts;
  tlgb_tucker_default_options(&topts);
  expect(topts.n_iter_max == 100, "tucker default n_iter_max");

  const int64_t shape[3] = {4, 5, 6};
  size_t bytes = 0;
  /* mode out of range: rejected on the host before any CUDA call */
  expect(tlgb_mttkrp_workspace_size(TLGB_F32, 3, shape, 2, 3, &bytes) == TLGB_EINVAL,
         "mttkrp rejects mode 3 of a 3-way tensor");
  expect(strstr(tlgb_last_error(), "mode") != NULL, "error message names the mode");
  /* unknown dtype */
  expect(tlgb_mttkrp_workspace_size(7, 3, shape, 2, 0, &bytes) == TLGB_EINVAL,
         "mttkrp rejects an unknown dtype");
  /* more modes than TLGB_MAX_MODES */
  expect(tlgb_mttkrp_workspace_size(TLGB_F64, TLGB_MAX_MODES + 1, shape, 2, 0, &bytes) ==
             TLGB_EINVAL,
         "mttkrp rejects too many modes");
  /* a proximal operator of unknown kind: rejected before the pointers are used */
  double dummy = 0.0;
  expect(tlgb_proximal(TLGB_F64, &dummy, 1, 99, 0.0, &dummy, NULL, 0, NULL) == TLGB_EINVAL,
         "proximal rejects an unknown kind");
  expect(strstr(tlgb_last_error(), "kind") != NULL, "error message names the kind");
  /* an entry point this library does not implement for the dtype */
  expect(tlgb_proximal(TLGB_BF16, &dummy, 1, TLGB_CONS_NON_NEGATIVE, 0.0, &dummy, NULL, 0, NULL) ==
             TLGB_EINVAL,
         "proximal rejects bf16");

  printf("%d failures\n", failures);
  return failures == 0 ? 0 : 1;
}
