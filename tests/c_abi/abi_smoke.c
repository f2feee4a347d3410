/* A C caller of the library (C99, no C++): the header compiles as C, the entry points link by their plain names,
 * and argument errors come back as status codes with a message, all without a GPU. Built and run by
 * tests/test_host_abi_and_sharding.py. */
#include <stdio.h>
#include <string.h>

#include "spitfire_gb300.h"

static int expect(int got, int want, const char *what)
{
  if (got != want) {
    printf("FAIL %s: status %d, expected %d (%s)\n", what, got, want, sf_last_error());
    return 1;
  }
  return 0;
}

int main(void)
{
  int bad = 0;
  const char *v = sf_version();
  if (!v || !strstr(v, "sm_103a")) {
    printf("FAIL version\n");
    bad++;
  }
  bad += expect(sf_mech_create(NULL, NULL), SF_ERR_INVALID_ARGUMENT, "sf_mech_create(NULL)");
  bad += expect(sf_btddod_solve_batch(0, 0, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL),
                SF_ERR_INVALID_ARGUMENT, "sf_btddod_solve_batch(NULL)");
  bad += expect(sf_newton_lu_batch(-1, 54, NULL, NULL, 0, NULL, NULL, NULL, NULL, NULL), SF_ERR_INVALID_ARGUMENT,
                "sf_newton_lu_batch(n < 0)");
  bad += expect(sf_adjoint_batch(NULL, NULL, 0, NULL, 1, NULL, NULL, NULL, 1, NULL, NULL, NULL, NULL, 0, NULL),
                SF_ERR_INVALID_ARGUMENT, "sf_adjoint_batch(NULL)");
  bad += expect(sf_flamelet_steady_newton_batch(NULL, NULL, NULL, NULL, 1e-6, 10, 1.5, 1e6, -1e-6, 0, NULL, NULL,
                                                NULL, 0, NULL),
                SF_ERR_INVALID_ARGUMENT, "sf_flamelet_steady_newton_batch(NULL)");
  if (sf_adjoint_workspace_size(NULL, NULL, 4, 2) != 0 || sf_flamelet_steady_workspace_size(NULL, NULL) != 0) {
    printf("FAIL workspace sizes of null handles\n");
    bad++;
  }
  if (bad == 0) printf("OK %s\n", v);
  return bad ? 1 : 0;
}
