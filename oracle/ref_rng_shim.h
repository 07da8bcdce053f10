/* Force-included (-include) ahead of the reference engine when it is compiled as
 * the CPU oracle (TEST INFRASTRUCTURE).  Redirects the engine's rand()/srand()
 * to the oracle harness so that the harness can switch between glibc's stream
 * and the counter-based Philox stream that the GPU path and the C oracle share.
 * <stdlib.h> is included first so its own declarations keep their real names. */
#ifndef TIS_REF_RNG_SHIM_H
#define TIS_REF_RNG_SHIM_H
#include <stdlib.h>
#ifdef __cplusplus
extern "C" {
#endif
int tis_shim_rand(void);
void tis_shim_srand(unsigned seed);
#ifdef __cplusplus
}
#endif
#define rand tis_shim_rand
#define srand tis_shim_srand
#endif
