/* A plain C caller of the library, as a cgo or JNI shim would be: the ABI
 * version, the reference CLI's radix resolution, and a context that reports
 * whether a device is present.  Prints one line of results. */
#include <stdio.h>

#include "phj_gpu.h"

int main(void)
{
    uint8_t bits[32];
    uint32_t n = 0;
    const phj_status st = phj_resolve_radix(65536, 2, NULL, 0, bits, &n);
    phj_ctx *ctx = NULL;
    const phj_status cs = phj_ctx_create(0, &ctx);
    printf("abi %u radix %d %u %u %u ctx %d\n", phj_abi_version(), (int)st, n, n > 0 ? bits[0] : 0, n > 1 ? bits[1] : 0, (int)cs);
    if (ctx)
        phj_ctx_destroy(ctx);
    return 0;
}
