/* Reference-side driver for the link test of mpi-rockstar_gb300/shim/gpu_shim.c:
 * linked with the reference's own objects (oracle/_ref/obj, compiled from the
 * unmodified reference sources) and librockstar_gb300.so, it sets up the
 * reference's configuration and particle globals and calls the shim the way
 * src/mpi_main.cpp would.  The reference's error handler is replaced so an
 * abort is visible to the test: it prints the code and exits with 42.  On a
 * machine without a GPU the first library call returns RSG_ERR_NO_DEVICE
 * and the shim must turn that into rockstar_abort. */
#include <stdio.h>
#include <stdlib.h>
#include <unistd.h>

#include "config.h"
#include "config_vars.h"
#include "error.h"
#include "particle.h"
#include "rockstar.h"

void rockstar_gpu(void);
void do_halo_finding_gpu(int batched);
void load_particles_internal_gpu(char *filename, struct particle **parts, int64_t *num_parts);

static void on_abort(int code, const char *file, int line) {
    printf("rockstar_abort(%d) raised at %s:%d\n", code, file, line);
    fflush(stdout);
    _exit(42);
}

int main(int argc, char **argv) {
    rockstar_set_error_handler(on_abort);
    do_config(NULL);
    if (argc > 1) {  /* an internal-format file: read through the shim (no device step) */
        struct particle *q = NULL;
        int64_t nq = 0, sum = 0;
        load_particles_internal_gpu(argv[1], &q, &nq);
        for (int64_t i = 0; i < nq; i++) sum += q[i].id;
        printf("internal: %lld particles, id sum %lld, scale %.6f, box %.3f\n", (long long)nq,
               (long long)sum, SCALE_NOW, BOX_SIZE);
        free(q);
    }
    PARTICLE_MASS = 1e9;
    BOX_SIZE = 40;
    setup_config();
    num_p = 4000;
    p = calloc(num_p, sizeof(struct particle));
    unsigned s = 12345u;
    for (int64_t i = 0; i < num_p; i++) {
        p[i].id = i;
        for (int k = 0; k < 6; k++) {
            s = s * 1103515245u + 12345u;
            float u = (float)((s >> 8) & 0xffff) / 65536.0f;
            p[i].pos[k] = (k < 3) ? (i < 2000 ? 20.0f + 0.05f * u : 40.0f * u) : 100.0f * u;
        }
    }
    rockstar_gpu();
    printf("rockstar_gpu: %lld groups\n", (long long)num_all_fofs);
    do_halo_finding_gpu(0);
    printf("do_halo_finding_gpu: %lld halos\n", (long long)num_halos);
    return 0;
}
