/* A plain C99 consumer of the C ABI: what a cgo, JNI or N-API binding
 * compiles against.  Host-only entry points, no GPU needed. */
#include <stdio.h>

#include "fastrecon_gb300.h"

int main(void)
{
    float lut[512];
    int st = fr_kb_lut(4.0f, 1.5f, 512, lut);
    if (st != FR_OK) return 1;
    printf("%s|%s|%.9g|%.9g\n", fr_version(), fr_status_string(FR_OK), lut[0], lut[511]);
    /* null handles are rejected before any CUDA call */
    if (fr_recon_run_host(NULL, NULL, NULL, NULL, 0, NULL, NULL) != FR_ERR_INVALID_ARGUMENT) return 2;
    if (fr_recon_submit_host(NULL, NULL, NULL, NULL, 0, NULL, NULL) != FR_ERR_INVALID_ARGUMENT) return 3;
    if (fr_recon_sync(NULL, NULL) != FR_ERR_INVALID_ARGUMENT) return 4;
    if (fr_grid(NULL, NULL, NULL, 1, NULL, NULL) != FR_ERR_INVALID_ARGUMENT) return 5;
    printf("%s\n", fr_last_error());
    return 0;
}
