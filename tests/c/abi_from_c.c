/* A C caller of the library's two headers (compiled as C11 by the CPU test
 * test_c_caller_cpu.py): the headers compile as plain C, the library links,
 * and the host-only entry points answer without a GPU. */
#include <stdio.h>
#include <string.h>

#include "accelsearch.h"
#include "bpd_compat.h"

int main(void) {
    accel_config cfg;
    accel_config_init(&cfg);
    printf("version %s\n", accel_version());
    printf("config %d %d %d %d %d\n", cfg.zmax, cfg.numharm, cfg.fftlen, cfg.whiten_initbuf,
           cfg.whiten_maxbuf);
    printf("first_bin %lld\n", accel_first_bin(1LL << 22, 64e-6));
    printf("power_cut %.6f\n", accel_power_cut(6.0, 8, 1.0));
    printf("sigma %.6f\n", accel_sigma_of_power(accel_power_cut(6.0, 8, 1.0), 8, 1.0));
    printf("required_z %d\n", calc_required_z(0.75, 200.0));
    printf("total_harmonics %d\n", getTotalHarmonics(4));
    long long g[5];
    printf("step_harmonic %d", accel_step_harmonic(268, 7734, 3, 4, 114, g));
    for (int i = 0; i < 5; i++) printf(" %lld", g[i]);
    printf("\n");
    float dms[2] = {0.0f, 100.0f};
    int delays[2 * 4], mx = -1;
    int rc = accel_dedisperse_delays(4, 1500.0, -75.0, 64e-6, dms, 2, delays, &mx);
    printf("delays %d %d %d %d %d %d\n", rc, delays[4], delays[5], delays[6], delays[7], mx);
    /* an invalid configuration is refused before any device work */
    accel_ctx *ctx = NULL;
    cfg.numharm = 3;
    rc = accel_create(&cfg, &ctx);
    printf("create_bad %d %s %d\n", rc, ctx == NULL ? "null" : "set", strlen(accel_last_error()) > 0);
    return 0;
}
