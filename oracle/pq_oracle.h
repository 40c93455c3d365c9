/*
 * pq_oracle.h -- CPU oracle for the polyq amplitude path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C restatement of the
 * reference crate's algorithm (src/pathsum.rs, src/normal_form.rs,
 * src/engine.rs, src/rank.rs, src/sim.rs, src/dense.rs).  It is used by the
 * test-suite as the checker, by `__graft_entry__.smoke()` and by bench.py's
 * CPU-baseline leg.  The product library (polyq-v1.0_gb300) never links,
 * loads or calls it.
 *
 * Conventions shared with the product C-ABI:
 *   gate codes   0 H, 1 X, 2 Y, 3 Z, 4 S, 5 SDG, 6 T, 7 TDG, 8 P(phase),
 *                9 CZ(q0,q1), 10 CX(control q0, target q1), 11 SWAP, 12 GPHASE(phase)
 *   phases       uint32 k meaning the angle 2*pi*k/2^32 (src/phase.rs:22-24)
 *   bitstrings   packed little-endian uint64 words, qubit q = bit q
 *   complex out  interleaved (re, im) doubles
 */
#ifndef PQ_ORACLE_H
#define PQ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pqo_sim pqo_sim;

/* strategy: 0 = Auto, 1 = Cached, 2 = Pairs(pairs)   (src/sim.rs:41-48) */
pqo_sim *pqo_sim_new(int nq, int ngates, const uint8_t *op, const int32_t *q0, const int32_t *q1,
                     const uint32_t *phase, int strategy, int pairs);
void pqo_sim_free(pqo_sim *s);

/* EngineStats of branch 0 + pairs: free_vars planes lines radical terms branch_dim pairs num_branches */
void pqo_stats(const pqo_sim *s, int64_t out[8]);

/* <y|C|x> for n boundaries, evaluated on `nthreads` host threads (<=0: all cores). */
void pqo_amplitudes(pqo_sim *s, int n, const uint64_t *xs, const uint64_t *ys, double *out, int nthreads);

/* Branches enumerated by the last pqo_amplitudes call (2^d of each non-vanishing job). */
double pqo_last_branches(const pqo_sim *s);

/* Marginal probability of measuring (qubits[i] -> outcomes[i]) on input x (src/sim.rs:225-231). */
double pqo_marginal(pqo_sim *s, const uint64_t *x, int nmeas, const int32_t *qubits, const uint8_t *outcomes);

/* Path-sum brute force (src/pathsum.rs:454-489) of <y|C|x>; returns -1 if > 26 free vars. */
int pqo_brute_force(pqo_sim *s, const uint64_t *x, const uint64_t *y, double out[2]);
void pqo_sample_many(pqo_sim *s, const uint64_t *x, int64_t shots, uint64_t seed, uint64_t *out);
void pqo_amplitude_estimate(pqo_sim *s, const uint64_t *x, const uint64_t *y, int64_t samples, uint64_t seed,
                            double out[3]);
/* {pair candidates with the io variables fixed, live variables} of the circuit's path sum. */
void pqo_path_info(const pqo_sim *s, int64_t out[2]);
/* approx::estimate_amplitude (approx.rs:96-135): out = (re, im, stderr). */
void pqo_amplitude_estimate_pairs(pqo_sim *s, const uint64_t *x, const uint64_t *y, int pairs, int64_t samples,
                                  uint64_t seed, int exact_dim_limit, double out[3]);

/* Dense statevector (src/dense.rs:12-27); out has 2*2^nq doubles. */
void pqo_dense_statevector(int nq, int ngates, const uint8_t *op, const int32_t *q0, const int32_t *q1,
                           const uint32_t *phase, const uint64_t *x, double *out);

/* Equivalence of two circuits (src/sim.rs:302-314): out = overlap re, im; returns 1 if equivalent. */
int pqo_equivalence(int nq1, int ng1, const uint8_t *op1, const int32_t *a1, const int32_t *b1, const uint32_t *p1,
                    int nq2, int ng2, const uint8_t *op2, const int32_t *a2, const int32_t *b2, const uint32_t *p2,
                    double tol, double out[2]);

/*
 * Canonical dump of branch engine `br`'s normal form and branch data as u64 words,
 * in the layout documented in pq_oracle.c (engine_dump).  Returns the number of words
 * (call with out=NULL to size).
 */
int64_t pqo_engine_dump(const pqo_sim *s, int br, uint64_t *out, int64_t cap);

/*
 * Per-branch Z8 indices of branch engine `br` for boundary (x, y): out[s] = phase8 at the
 * kernel point s (s = sum_j bit_j(s) * kernel_j), for all s < 2^d (d <= 24).
 * Returns d, or -1 if the boundary is contradictory / the subspace is empty.
 */
int pqo_branch_phases(pqo_sim *s, int br, const uint64_t *x, const uint64_t *y, uint8_t *out);

/* Branch dimension d of branch engine `br` (-1 out of range). */
int pqo_branch_dim(const pqo_sim *s, int br);

/*
 * Integers of Engine::prepare for all n boundaries x all branch engines (boundary-major),
 * PQO_PREP_WORDS u64 words per job: vanish flag, constant phase, k0, pivot bits y0, then the
 * Z4 increments Lp_j as bytes (layout in pq_oracle.c, pqo_prepare_info).
 */
#define PQO_PREP_WORDS 12
void pqo_prepare_info(pqo_sim *s, int n, const uint64_t *xs, const uint64_t *ys, uint64_t *out);

/* Pivot-rule-parametrised normal form check on a raw form (src/normal_form.rs:555-606):
 * returns 0 if the basis block-diagonalises the Gram matrix and is invertible. */
int pqo_check_structure(int m, const uint8_t *bmat /* m*m */, const uint8_t *parity, int rule,
                        int32_t out_sizes[3]);

/* Gauss sum of a raw form with shift (src/normal_form.rs:496-501) vs brute force. */
void pqo_gauss_sum(int m, const uint8_t *bmat, const uint8_t *v, const uint8_t *shift, int rule,
                   double out_closed[2], double out_brute[2]);

#ifdef __cplusplus
}
#endif
#endif
