/* A C99 caller of the library: compiled against include/sdns_gb300.h and
 * linked with libsdns_gb300.so by tests/test_abi_cpu.py.  It makes only the
 * calls that need no GPU: the ABI version and the argument checks that run
 * before any CUDA call.  Exit status 0 means every check held. */
#include <stdio.h>
#include <string.h>

#include "sdns_gb300.h"

int main(void) {
  if (sdns_abi_version() != SDNS_ABI_VERSION) return 1;
  sdns_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.n[0] = 17; cfg.n[1] = 16; cfg.n[2] = 16;          /* not a power of two */
  cfg.L[0] = cfg.L[1] = cfg.L[2] = 6.283185307179586;
  cfg.nu = 0.000625;
  cfg.precision = SDNS_SINGLE;
  cfg.dealias = SDNS_DEALIAS_23;
  cfg.formulation = SDNS_NS;
  sdns_ctx* ctx = NULL;
  if (sdns_create(&cfg, &ctx) != SDNS_EINVAL || ctx != NULL) return 2;
  if (strstr(sdns_last_error(), "powers of two") == NULL) return 3;
  cfg.n[0] = 16;
  cfg.formulation = 7;                                   /* no such formulation */
  if (sdns_create(&cfg, &ctx) != SDNS_EINVAL) return 4;
  cfg.formulation = SDNS_VV;
  cfg.dealias = SDNS_DEALIAS_32;
  char buf[16];
  /* the allocation-free entry point rejects what it does not implement before any CUDA call */
  if (sdns_compute_rhs_noalloc(&cfg, buf, buf, NULL) != SDNS_EINVAL) return 5;
  if (sdns_lincomb(NULL, buf, NULL, 0, NULL, NULL) != SDNS_EINVAL) return 6;   /* null context */
  printf("c99 caller ok: ABI %d\n", sdns_abi_version());
  return 0;
}
