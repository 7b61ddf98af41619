/* Compiled as C99 against include/fermicc.h and linked with libfermicc.so by
 * tests/test_c_header.py: the header is plain C, and the library's argument
 * checks and status strings work without touching a device.  With a GB300
 * present, fcc_create / fcc_scf_create succeed and the handles are destroyed. */
#include <stdio.h>
#include <string.h>

#include "fermicc.h"
#include "fermicc_testing.h"

static int fails = 0;
#define EXPECT(c)                                                   \
  do {                                                              \
    if (!(c)) { fprintf(stderr, "failed: %s\n", #c); ++fails; }     \
  } while (0)

int main(void) {
  fcc_opts o;
  fcc_default_opts(&o);
  EXPECT(o.max_iter == 50 && o.ndiis == 3 && o.e_conv == 1e-10);
  EXPECT(strcmp(fcc_strerror(FCC_OK), "success") == 0);
  EXPECT(strlen(fcc_strerror(FCC_ERR_NO_DEVICE)) > 0);
  EXPECT(fcc_create(NULL, 5, 19, 84, 0) == FCC_ERR_BAD_ARG);

  fcc_ctx* c = NULL;
  EXPECT(fcc_create(&c, 0, 19, 84, 0) == FCC_ERR_BAD_ARG && c == NULL);
  int rc = fcc_create(&c, 5, 19, 84, 0);
  if (rc == FCC_OK) fcc_destroy(c);
  else EXPECT(rc == FCC_ERR_NO_DEVICE && c == NULL);
  EXPECT(fcc_upload_df(NULL, NULL, NULL, NULL, NULL, NULL, 0.0) == FCC_ERR_BAD_ARG);
  EXPECT(strcmp(fcc_last_error(NULL), "") == 0);

  fcc_scf* s = NULL;
  EXPECT(fcc_scf_create(&s, 24, 0, 0) == FCC_ERR_BAD_ARG && s == NULL);
  rc = fcc_scf_create(&s, 24, 84, 0);
  if (rc == FCC_OK) fcc_scf_destroy(s);
  else EXPECT(rc == FCC_ERR_NO_DEVICE && s == NULL);
  EXPECT(fcc_scf_build_fock(NULL, NULL, NULL, NULL, NULL) == FCC_ERR_BAD_ARG);

  EXPECT(fcc_stat_launches() >= 0);
  if (fails == 0) printf("abi_check ok\n");
  return fails == 0 ? 0 : 1;
}
