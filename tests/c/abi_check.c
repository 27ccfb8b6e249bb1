/* A plain C caller of the C ABI (include/feynsimul.h), as a reference maintainer's FFI
 * would be: validation errors and messages, and an NVRTC compile of the harmonic-oscillator
 * sweep for sm_103a.  Needs no GPU.  Prints "abi ok" and exits 0 on success. */
#include <stdio.h>
#include <string.h>

#include "feynsimul.h"

int main(void)
{
    if (!strstr(fs_version(), "sm_103a")) {
        printf("bad version string: %s\n", fs_version());
        return 1;
    }
    fs_config c;
    memset(&c, 0, sizeof c);
    c.dof = 1;
    c.n_slices = 128;
    c.bisection_level = 3;
    c.beta = 10.0;
    c.n_walkers = 1024;
    c.walkers_per_group = 1;
    c.operator_runs = 100;
    c.metro_steps_per_operator_run = 1;
    c.enable_parallelize_path = 1;
    c.accum = FS_ACCUM_FP64;
    c.fast_math = 1;
    const char *ops[] = {"1.0 * x1 * x1"};
    const char *cors[] = {"x1"};
    static char log[1 << 16];

    /* kernel.py:134-135: N must be a power of 2 */
    c.n_slices = 100;
    int rc = fs_compile_only(&c, "0.5 * 1.0 * x1 * x1", "", ops, 1, cors, 1, NULL, 0, log, sizeof log);
    if (rc != FS_ERR_CONFIG || !strstr(fs_last_error(NULL), "power of 2")) {
        printf("expected the N error, got %d: %s\n", rc, fs_last_error(NULL));
        return 1;
    }
    c.n_slices = 128;
    /* plugin code with the reference's OpenCL spellings */
    rc = fs_compile_only(&c, "0.5 * 1.0 * x1 * x1", "FLOAT_TYPE sqr(FLOAT_TYPE x){return native_exp(0.0) * x*x;}",
                         ops, 1, cors, 1, NULL, 0, log, sizeof log);
    if (rc != FS_OK) {
        printf("compile failed %d: %s\n%s\n", rc, fs_last_error(NULL), log);
        return 1;
    }
    /* a syntax error in plugin code comes back as FS_ERR_COMPILE with the NVRTC log */
    rc = fs_compile_only(&c, "0.5 * x1 *", "", ops, 1, cors, 1, NULL, 0, log, sizeof log);
    if (rc != FS_ERR_COMPILE) {
        printf("expected FS_ERR_COMPILE, got %d\n", rc);
        return 1;
    }
    printf("abi ok\n");
    return 0;
}
