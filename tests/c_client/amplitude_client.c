/* A plain C caller of the C-ABI (include/polyq_gb300.h): builds <11|H0 CX01 T1 H1|00> and a
 * few more amplitudes, the way a compiled host (the reference's Rust FFI, a C++ service)
 * binds the library.  Prints "re im" per amplitude; exit status 0 on success. */
#include <stdio.h>
#include <stdint.h>

#include "polyq_gb300.h"

int main(void) {
    const uint8_t op[] = {0, 10, 6, 0, 9, 4};  /* H 0; CX 0 1; T 1; H 1; CZ 1 2; S 2 */
    const int32_t q0[] = {0, 0, 1, 1, 1, 2};
    const int32_t q1[] = {0, 1, 0, 0, 2, 0};
    const uint32_t ph[] = {0, 0, 0, 0, 0, 0};
    pq_circuit_desc c = {3, 6, op, q0, q1, ph};
    pq_sim *sim = NULL;
    if (pq_sim_create(&c, 0, 0, &sim) != PQ_OK) {
        fprintf(stderr, "create: %s\n", pq_last_error());
        return 1;
    }
    uint64_t x[8], y[8];
    double out[16], err[8];
    for (int i = 0; i < 8; i++) {
        x[i] = 0;
        y[i] = (uint64_t)i;
    }
    if (pq_amplitudes(sim, 8, x, y, out, err) != PQ_OK) {
        fprintf(stderr, "amplitudes: %s\n", pq_last_error());
        pq_sim_destroy(sim);
        return 1;
    }
    for (int i = 0; i < 8; i++) printf("%.17g %.17g\n", out[2 * i], out[2 * i + 1]);
    /* misuse is a status, never an abort */
    if (pq_amplitudes(sim, 0, x, y, out, err) != PQ_ERR_INVALID_ARG) return 2;
    pq_sim_destroy(sim);
    return 0;
}
