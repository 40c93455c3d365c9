/*
 * pq_oracle.c -- CPU oracle for the polyq amplitude-evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement, in FP64, of the
 * reference crate's algorithm, used as the checker by tests/, by
 * __graft_entry__.smoke() and as bench.py's CPU baseline.  Nothing in the
 * product library (polyq-v1.0_gb300) includes, links or calls this file.
 *
 * What is restated, and where it comes from (paths inside the reference crate):
 *   phase ring, ROOT8 ............ src/phase.rs:22-114
 *   BitVec / BitMat .............. src/bits.rs:16-299 (scalar popcount only)
 *   circuit compiler ............. src/pathsum.rs:100-324 (Compiler::apply/rotate/snapshot/normalize)
 *   boundary, brute force ........ src/pathsum.rs:430-489
 *   substitute, trace closure .... src/pathsum.rs:360-425
 *   sandwich ..................... src/pathsum.rs:304-314
 *   symmetric F2 elimination ..... src/normal_form.rs:61-129 (single_step, hyper_step),
 *                                  :240-336 (Structure::new, First and MinWeight pivot rules)
 *   Z4 diagonal, columns ......... src/normal_form.rs:339-461
 *   phase8, gauss_sum ............ src/normal_form.rs:465-501
 *   Engine::new, Elim, Term ...... src/engine.rs:107-390
 *   prepare/sum_subspace/gray .... src/engine.rs:557-722 (LOW_BITS=14, RECOMPUTE_EVERY=2048)
 *   RankEngine, pair candidates .. src/rank.rs:62-222
 *   Simulator, marginal, equiv ... src/sim.rs:65-314
 *   dense statevector ............ src/dense.rs:12-107
 * Third-party arithmetic restated: num-complex 0.4.6 (Cargo.lock) Complex64 mul/div
 * (schoolbook formulas) and from_polar (r*cos, r*sin).
 *
 * Compiled with -ffp-contract=off so that no multiply-add is fused and the FP64
 * results are the same on x86-64 and aarch64 hosts.
 */
#include "pq_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------ complex */
typedef struct { double re, im; } cx;
static inline cx C(double r, double i) { cx z = {r, i}; return z; }
static inline cx cadd(cx a, cx b) { return C(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return C(a.re - b.re, a.im - b.im); }
static inline cx cmul(cx a, cx b) { return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cscale(cx a, double s) { return C(a.re * s, a.im * s); }
static inline cx cdiv(cx a, cx b) {
    double n = b.re * b.re + b.im * b.im;
    return C((a.re * b.re + a.im * b.im) / n, (a.im * b.re - a.re * b.im) / n);
}

/* ------------------------------------------------------------------ phase ring (src/phase.rs) */
#define PH_PI ((uint32_t)1u << 31)
#define PH_HALF_PI ((uint32_t)1u << 30)
#define PH_QUARTER_PI ((uint32_t)1u << 29)
static const double H_ = 0.70710678118654752440; /* FRAC_1_SQRT_2 */
static cx ROOT8[8];
static void init_root8(void) {
    ROOT8[0] = C(1, 0); ROOT8[1] = C(H_, H_); ROOT8[2] = C(0, 1); ROOT8[3] = C(-H_, H_);
    ROOT8[4] = C(-1, 0); ROOT8[5] = C(-H_, -H_); ROOT8[6] = C(0, -1); ROOT8[7] = C(H_, -H_);
}
static cx phase_to_complex(uint32_t p) { /* phase.rs:60-66 */
    if ((p & ((1u << 29) - 1)) == 0) return ROOT8[p >> 29];
    double th = 2.0 * M_PI * (double)p / 4294967296.0;
    return C(cos(th), sin(th));
}
static int clifford_level(uint32_t p) { /* phase.rs:70-76, -1 = None */
    if ((p & ((1u << 30) - 1)) == 0) return (int)(p >> 30);
    return -1;
}
static uint32_t z4_phase(unsigned k) { return (uint32_t)(k & 3) << 30; }

/* ------------------------------------------------------------------ bit vectors (src/bits.rs) */
typedef struct { int len, nw; uint64_t *w; } bv;
static inline int nwords(int len) { return (len + 63) / 64; }
static void bv_init(bv *v, int len) {
    v->len = len; v->nw = nwords(len);
    v->w = (uint64_t *)calloc((size_t)(v->nw ? v->nw : 1), 8);
}
static void bv_free(bv *v) { free(v->w); v->w = NULL; }
static inline int bv_get(const bv *v, int i) { return (int)((v->w[i >> 6] >> (i & 63)) & 1); }
static inline void bv_set(bv *v, int i, int val) {
    if (val) v->w[i >> 6] |= 1ull << (i & 63); else v->w[i >> 6] &= ~(1ull << (i & 63));
}
static inline void bv_flip(bv *v, int i) { v->w[i >> 6] ^= 1ull << (i & 63); }
static inline void bv_xor(bv *d, const bv *s) { for (int i = 0; i < d->nw; i++) d->w[i] ^= s->w[i]; }
static inline void bv_and(bv *d, const bv *s) { for (int i = 0; i < d->nw; i++) d->w[i] &= s->w[i]; }
static inline void bv_clear(bv *v) { memset(v->w, 0, (size_t)v->nw * 8); }
static inline void bv_copy(bv *d, const bv *s) { memcpy(d->w, s->w, (size_t)d->nw * 8); }
static bv bv_clone(const bv *s) { bv d; bv_init(&d, s->len); bv_copy(&d, s); return d; }
static inline unsigned bv_popc(const bv *v) {
    unsigned c = 0; for (int i = 0; i < v->nw; i++) c += (unsigned)__builtin_popcountll(v->w[i]); return c;
}
static inline unsigned bv_andcount(const bv *a, const bv *b) {
    unsigned c = 0; for (int i = 0; i < a->nw; i++) c += (unsigned)__builtin_popcountll(a->w[i] & b->w[i]); return c;
}
static inline int bv_dot(const bv *a, const bv *b) { return (int)(bv_andcount(a, b) & 1); }
static inline int bv_first_one(const bv *v) {
    for (int i = 0; i < v->nw; i++) if (v->w[i]) return i * 64 + __builtin_ctzll(v->w[i]);
    return -1;
}
static inline int bv_eq(const bv *a, const bv *b) { return memcmp(a->w, b->w, (size_t)a->nw * 8) == 0; }
static inline int bv_is_zero(const bv *v) { for (int i = 0; i < v->nw; i++) if (v->w[i]) return 0; return 1; }
/* iterate set bits: for (int i = bv_next(v, 0); i >= 0; i = bv_next(v, i + 1)) */
static inline int bv_next(const bv *v, int from) {
    if (from >= v->len) return -1;
    int wi = from >> 6;
    uint64_t w = v->w[wi] & (~0ull << (from & 63));
    while (1) {
        if (w) return wi * 64 + __builtin_ctzll(w);
        if (++wi >= v->nw) return -1;
        w = v->w[wi];
    }
}
#define FOR_ONES(i, v) for (int i = bv_next((v), 0); i >= 0; i = bv_next((v), i + 1))

typedef struct { int nrows, ncols; bv *r; } bm;
static void bm_init(bm *m, int nr, int nc) {
    m->nrows = nr; m->ncols = nc; m->r = (bv *)calloc((size_t)(nr ? nr : 1), sizeof(bv));
    for (int i = 0; i < nr; i++) bv_init(&m->r[i], nc);
}
static void bm_free(bm *m) { for (int i = 0; i < m->nrows; i++) bv_free(&m->r[i]); free(m->r); m->r = NULL; }
static bm bm_clone(const bm *s) {
    bm d; d.nrows = s->nrows; d.ncols = s->ncols; d.r = (bv *)calloc((size_t)(s->nrows ? s->nrows : 1), sizeof(bv));
    for (int i = 0; i < s->nrows; i++) d.r[i] = bv_clone(&s->r[i]);
    return d;
}
static inline void bm_flip_sym(bm *m, int i, int j) { bv_flip(&m->r[i], j); bv_flip(&m->r[j], i); }

/* ------------------------------------------------------------------ circuits (src/circuit.rs) */
enum { G_H = 0, G_X, G_Y, G_Z, G_S, G_SDG, G_T, G_TDG, G_P, G_CZ, G_CX, G_SWAP, G_GPHASE };
typedef struct { uint8_t op; int a, b; uint32_t ph; } gate;
typedef struct { int nq, ng; gate *g; } circuit;

static circuit circuit_from(int nq, int ng, const uint8_t *op, const int32_t *q0, const int32_t *q1, const uint32_t *ph) {
    circuit c; c.nq = nq; c.ng = ng; c.g = (gate *)calloc((size_t)(ng ? ng : 1), sizeof(gate));
    for (int i = 0; i < ng; i++) {
        c.g[i].op = op[i]; c.g[i].a = q0[i]; c.g[i].b = q1[i]; c.g[i].ph = ph[i];
    }
    return c;
}
static gate gate_inverse(gate g) { /* circuit.rs:46-56 */
    gate r = g;
    switch (g.op) {
        case G_S: r.op = G_SDG; break;
        case G_SDG: r.op = G_S; break;
        case G_T: r.op = G_TDG; break;
        case G_TDG: r.op = G_T; break;
        case G_P: case G_GPHASE: r.ph = (uint32_t)(0u - g.ph); break;
        default: break;
    }
    return r;
}
static int h_count(const circuit *c) { /* circuit.rs:206-215 */
    int h = 0;
    for (int i = 0; i < c->ng; i++) h += c->g[i].op == G_H ? 1 : (c->g[i].op == G_CX ? 2 : 0);
    return h;
}

/* ------------------------------------------------------------------ path sums (src/pathsum.rs) */
typedef struct {
    int nq, nv, num_h;
    bm b;
    uint8_t *v;
    uint32_t *theta;
    uint32_t global;
    uint8_t *dead;
    int *outputs;
    uint8_t *out_neg;
    int zero;
} pathsum;

typedef struct {
    int n, nvars, num_h, cap;
    int *wire;
    uint8_t *neg;
    bm b;
    uint8_t *v;
    uint32_t *theta;
    uint32_t global;
} compiler;

static void comp_init(compiler *c, int n, int extra) { /* pathsum.rs:100-113 */
    c->n = n; c->nvars = n; c->num_h = 0; c->global = 0;
    c->cap = n + extra;
    if (c->cap < 1) c->cap = 1;
    c->wire = (int *)malloc(sizeof(int) * (size_t)(n ? n : 1));
    c->neg = (uint8_t *)calloc((size_t)(n ? n : 1), 1);
    for (int i = 0; i < n; i++) c->wire[i] = i;
    bm_init(&c->b, c->cap, c->cap);
    c->v = (uint8_t *)calloc((size_t)c->cap, 1);
    c->theta = (uint32_t *)calloc((size_t)c->cap, 4);
}
static void comp_free(compiler *c) { free(c->wire); free(c->neg); bm_free(&c->b); free(c->v); free(c->theta); }
static int comp_new_var(compiler *c) { /* pathsum.rs:120-129 (capacity is a hint) */
    if (c->nvars == c->cap) {
        int nc = c->cap * 2 > 8 ? c->cap * 2 : 8;
        bm nb; bm_init(&nb, nc, nc);
        for (int i = 0; i < c->cap; i++) memcpy(nb.r[i].w, c->b.r[i].w, (size_t)c->b.r[i].nw * 8);
        bm_free(&c->b); c->b = nb;
        c->v = (uint8_t *)realloc(c->v, (size_t)nc); memset(c->v + c->cap, 0, (size_t)(nc - c->cap));
        c->theta = (uint32_t *)realloc(c->theta, (size_t)nc * 4); memset(c->theta + c->cap, 0, (size_t)(nc - c->cap) * 4);
        c->cap = nc;
    }
    c->v[c->nvars] = 0; c->theta[c->nvars] = 0;
    return c->nvars++;
}
static void comp_add_v(compiler *c, int z, unsigned k) { c->v[z] = (uint8_t)((c->v[z] + k) & 3); }
static void comp_rotate(compiler *c, int q, uint32_t th) { /* pathsum.rs:215-224 */
    int z = c->wire[q];
    if (c->neg[q]) { c->theta[z] -= th; c->global += th; }
    else c->theta[z] += th;
}
static void comp_apply(compiler *c, gate g) { /* pathsum.rs:136-213 */
    int q = g.a;
    switch (g.op) {
        case G_H: {
            int z = c->wire[q], zp = comp_new_var(c);
            bm_flip_sym(&c->b, z, zp);
            c->num_h++;
            if (c->neg[q]) { comp_add_v(c, zp, 2); c->neg[q] = 0; }
            c->wire[q] = zp;
        } break;
        case G_X: c->neg[q] = !c->neg[q]; break;
        case G_Z: comp_add_v(c, c->wire[q], 2); if (c->neg[q]) c->global += PH_PI; break;
        case G_S:
            if (c->neg[q]) { comp_add_v(c, c->wire[q], 3); c->global += PH_HALF_PI; }
            else comp_add_v(c, c->wire[q], 1);
            break;
        case G_SDG:
            if (c->neg[q]) { comp_add_v(c, c->wire[q], 1); c->global -= PH_HALF_PI; }
            else comp_add_v(c, c->wire[q], 3);
            break;
        case G_T: comp_rotate(c, q, PH_QUARTER_PI); break;
        case G_TDG: comp_rotate(c, q, (uint32_t)(0u - PH_QUARTER_PI)); break;
        case G_P: comp_rotate(c, q, g.ph); break;
        case G_Y: {
            gate z = {G_Z, q, 0, 0}, x = {G_X, q, 0, 0};
            comp_apply(c, z); comp_apply(c, x); c->global += PH_HALF_PI;
        } break;
        case G_CZ: {
            int a = g.a, b = g.b, za = c->wire[a], zb = c->wire[b];
            bm_flip_sym(&c->b, za, zb);
            if (c->neg[b]) comp_add_v(c, za, 2);
            if (c->neg[a]) comp_add_v(c, zb, 2);
            if (c->neg[a] && c->neg[b]) c->global += PH_PI;
        } break;
        case G_CX: {
            gate h = {G_H, g.b, 0, 0}, cz = {G_CZ, g.a, g.b, 0};
            comp_apply(c, h); comp_apply(c, cz); comp_apply(c, h);
        } break;
        case G_SWAP: {
            int t = c->wire[g.a]; c->wire[g.a] = c->wire[g.b]; c->wire[g.b] = t;
            uint8_t u = c->neg[g.a]; c->neg[g.a] = c->neg[g.b]; c->neg[g.b] = u;
        } break;
        case G_GPHASE: c->global += g.ph; break;
    }
}
static void ps_normalize(pathsum *p) { /* pathsum.rs:317-324 */
    for (int k = 0; k < p->nv; k++) {
        int l = clifford_level(p->theta[k]);
        if (l >= 0) { p->v[k] = (uint8_t)((p->v[k] + l) & 3); p->theta[k] = 0; }
    }
}
static pathsum comp_snapshot(const compiler *c) { /* pathsum.rs:236-261 */
    pathsum p;
    int nv = c->nvars;
    p.nq = c->n; p.nv = nv; p.num_h = c->num_h;
    bm_init(&p.b, nv, nv);
    for (int i = 0; i < nv; i++) {
        const bv *row = &c->b.r[i];
        FOR_ONES(j, row) { if (j < nv) bv_set(&p.b.r[i], j, 1); else break; }
    }
    p.v = (uint8_t *)malloc((size_t)(nv ? nv : 1)); memcpy(p.v, c->v, (size_t)nv);
    p.theta = (uint32_t *)malloc((size_t)(nv ? nv : 1) * 4); memcpy(p.theta, c->theta, (size_t)nv * 4);
    p.global = c->global;
    p.dead = (uint8_t *)calloc((size_t)(nv ? nv : 1), 1);
    p.outputs = (int *)malloc(sizeof(int) * (size_t)(c->n ? c->n : 1)); memcpy(p.outputs, c->wire, sizeof(int) * (size_t)c->n);
    p.out_neg = (uint8_t *)malloc((size_t)(c->n ? c->n : 1)); memcpy(p.out_neg, c->neg, (size_t)c->n);
    p.zero = 0;
    ps_normalize(&p);
    return p;
}
static void ps_free(pathsum *p) { bm_free(&p->b); free(p->v); free(p->theta); free(p->dead); free(p->outputs); free(p->out_neg); }
static pathsum ps_clone(const pathsum *s) {
    pathsum p = *s;
    p.b = bm_clone(&s->b);
    int nv = s->nv ? s->nv : 1, nq = s->nq ? s->nq : 1;
    p.v = (uint8_t *)malloc((size_t)nv); memcpy(p.v, s->v, (size_t)s->nv);
    p.theta = (uint32_t *)malloc((size_t)nv * 4); memcpy(p.theta, s->theta, (size_t)s->nv * 4);
    p.dead = (uint8_t *)malloc((size_t)nv); memcpy(p.dead, s->dead, (size_t)s->nv);
    p.outputs = (int *)malloc(sizeof(int) * (size_t)nq); memcpy(p.outputs, s->outputs, sizeof(int) * (size_t)s->nq);
    p.out_neg = (uint8_t *)malloc((size_t)nq); memcpy(p.out_neg, s->out_neg, (size_t)s->nq);
    return p;
}
static pathsum ps_from_circuit(const circuit *c) { /* pathsum.rs:274-297 (no faults) */
    compiler comp; comp_init(&comp, c->nq, h_count(c));
    for (int i = 0; i < c->ng; i++) comp_apply(&comp, c->g[i]);
    pathsum p = comp_snapshot(&comp);
    comp_free(&comp);
    return p;
}
/* pathsum.rs:304-314: compile C then C^dagger; junction = wires after C. */
static pathsum ps_sandwich(const circuit *c, int *junction, uint8_t *jneg) {
    compiler comp; comp_init(&comp, c->nq, 2 * h_count(c));
    for (int i = 0; i < c->ng; i++) comp_apply(&comp, c->g[i]);
    memcpy(junction, comp.wire, sizeof(int) * (size_t)c->nq);
    memcpy(jneg, comp.neg, (size_t)c->nq);
    for (int i = c->ng - 1; i >= 0; i--) comp_apply(&comp, gate_inverse(c->g[i]));
    pathsum p = comp_snapshot(&comp);
    comp_free(&comp);
    return p;
}
/* pathsum.rs:328-336 */
static int ps_io_vars(const pathsum *p, int *f) {
    int n = 0;
    for (int q = 0; q < p->nq; q++) f[n++] = q;
    for (int q = 0; q < p->nq; q++) {
        int o = p->outputs[q], seen = 0;
        for (int i = 0; i < n; i++) if (f[i] == o) { seen = 1; break; }
        if (!seen) f[n++] = o;
    }
    return n;
}
typedef struct { int var; int val; } asg_t;
static int asg_put(asg_t *a, int *n, int var, int val) { /* pathsum.rs:432-438, sim.rs:79-85 */
    for (int i = 0; i < *n; i++) if (a[i].var == var) return a[i].val == val;
    a[*n].var = var; a[*n].val = val; (*n)++;
    return 1;
}
static inline int bit_of(const uint64_t *w, int q) { return (int)((w[q >> 6] >> (q & 63)) & 1); }
/* pathsum.rs:430-450: returns count, or -1 if contradictory */
static int ps_boundary(const pathsum *p, const uint64_t *x, const uint64_t *y, asg_t *out) {
    int n = 0;
    for (int q = 0; q < p->nq; q++) if (!asg_put(out, &n, q, bit_of(x, q))) return -1;
    for (int q = 0; q < p->nq; q++) if (!asg_put(out, &n, p->outputs[q], bit_of(y, q) ^ p->out_neg[q])) return -1;
    return n;
}
/* pathsum.rs:454-489 */
static int ps_brute_force(const pathsum *p, const asg_t *fixed, int nfix, cx *res) {
    if (p->zero) { *res = C(0, 0); return 0; }
    uint8_t *val = (uint8_t *)calloc((size_t)p->nv + 1, 1), *isf = (uint8_t *)calloc((size_t)p->nv + 1, 1);
    for (int i = 0; i < nfix; i++) { val[fixed[i].var] = (uint8_t)fixed[i].val; isf[fixed[i].var] = 1; }
    int *fr = (int *)malloc(sizeof(int) * ((size_t)p->nv + 1)), nfr = 0;
    int *live = (int *)malloc(sizeof(int) * ((size_t)p->nv + 1)), nl = 0;
    for (int i = 0; i < p->nv; i++) {
        if (!p->dead[i] && !isf[i]) fr[nfr++] = i;
        if (!p->dead[i]) live[nl++] = i;
    }
    if (nfr > 26) { free(val); free(isf); free(fr); free(live); return -1; }
    cx tot = C(0, 0);
    for (uint64_t mask = 0; mask < (1ull << nfr); mask++) {
        for (int bi = 0; bi < nfr; bi++) val[fr[bi]] = (uint8_t)((mask >> bi) & 1);
        uint32_t z4 = 0, th = 0;
        for (int li = 0; li < nl; li++) {
            int j = live[li];
            if (!val[j]) continue;
            z4 += p->v[j]; th += p->theta[j];
            const bv *row = &p->b.r[j];
            for (int k = bv_next(row, j + 1); k >= 0; k = bv_next(row, k + 1)) if (val[k]) z4 += 2;
        }
        tot = cadd(tot, phase_to_complex(z4_phase(z4 & 3) + th));
    }
    *res = cscale(cmul(tot, phase_to_complex(p->global)), pow(2.0, -(double)p->num_h / 2.0));
    free(val); free(isf); free(fr); free(live);
    return 0;
}
/* pathsum.rs:360-394 */
static void ps_substitute(pathsum *p, int a, int b, int c) {
    int bab = bv_get(&p->b.r[a], b);
    uint32_t ta = p->theta[a], tb = p->theta[b];
    uint8_t vb = p->v[b];
    bv nb = bv_clone(&p->b.r[b]);
    bv_set(&nb, a, 0);
    if (!c) {
        p->v[a] = (uint8_t)((p->v[a] + vb + 2 * bab) & 3);
        p->theta[a] = ta + tb;
    } else {
        p->v[a] = (uint8_t)((p->v[a] + 4 - vb) & 3);
        p->theta[a] = ta - tb;
        p->global += z4_phase(vb) + tb;
        FOR_ONES(k, &nb) p->v[k] = (uint8_t)((p->v[k] + 2) & 3);
    }
    FOR_ONES(k, &nb) bm_flip_sym(&p->b, a, k);
    bv nbrs = bv_clone(&p->b.r[b]);
    FOR_ONES(k, &nbrs) bv_set(&p->b.r[k], b, 0);
    bv_clear(&p->b.r[b]);
    p->v[b] = 0; p->theta[b] = 0; p->dead[b] = 1;
    int l = clifford_level(p->theta[a]);
    if (l >= 0) { p->v[a] = (uint8_t)((p->v[a] + l) & 3); p->theta[a] = 0; }
    bv_free(&nb); bv_free(&nbrs);
}
/* pathsum.rs:399-425 */
static void ps_trace_closure(pathsum *p) {
    int nv = p->nv;
    int *rep = (int *)malloc(sizeof(int) * (size_t)(nv + 1));
    uint8_t *par = (uint8_t *)calloc((size_t)nv + 1, 1);
    for (int i = 0; i < nv; i++) rep[i] = i;
    for (int q = 0; q < p->nq; q++) {
        int ra = q, pa = 0, rb = p->outputs[q], pb = 0;
        while (rep[ra] != ra) { pa ^= par[ra]; ra = rep[ra]; }
        while (rep[rb] != rb) { pb ^= par[rb]; rb = rep[rb]; }
        int c = pa ^ pb ^ p->out_neg[q];
        if (ra == rb) { if (c) p->zero = 1; continue; }
        ps_substitute(p, ra, rb, c);
        rep[rb] = ra; par[rb] = (uint8_t)c;
    }
    free(rep); free(par);
}

/* ------------------------------------------------------------------ normal form (src/normal_form.rs) */
typedef struct {
    int m, g, nodd, neven;
    bv *pa, *pb, *odd, *even;
} structure;
typedef struct { bv a, b, o, e; } uvec;
typedef struct { bv wa, wb, o1, o3, we; int sigma; } diag_t;

static void uv_init(uvec *u, const structure *s) {
    bv_init(&u->a, s->g); bv_init(&u->b, s->g); bv_init(&u->o, s->nodd); bv_init(&u->e, s->neven);
}
static void uv_free(uvec *u) { bv_free(&u->a); bv_free(&u->b); bv_free(&u->o); bv_free(&u->e); }
static void uv_xor(uvec *d, const uvec *s) { bv_xor(&d->a, &s->a); bv_xor(&d->b, &s->b); bv_xor(&d->o, &s->o); bv_xor(&d->e, &s->e); }
static void uv_copy(uvec *d, const uvec *s) { bv_copy(&d->a, &s->a); bv_copy(&d->b, &s->b); bv_copy(&d->o, &s->o); bv_copy(&d->e, &s->e); }
static void uv_clear(uvec *u) { bv_clear(&u->a); bv_clear(&u->b); bv_clear(&u->o); bv_clear(&u->e); }

/* normal_form.rs:61-82 */
static void single_step(bv *gram, bv *basis, bv *alive, int a, bv *s_out, bv *pa_out) {
    bv s = bv_clone(&gram[a]);
    bv_and(&s, alive); bv_set(&s, a, 0);
    bv pa = bv_clone(&basis[a]);
    FOR_ONES(bi, &s) { bv_xor(&gram[bi], &s); bv_xor(&basis[bi], &pa); }
    bv_set(alive, a, 0);
    *s_out = s; *pa_out = pa;
}
/* normal_form.rs:87-129 */
static int hyper_step(bv *gram, bv *basis, bv *alive, int a, bv *touched_out, bv *pa_out, bv *pb_out) {
    bv ra = bv_clone(&gram[a]);
    bv_and(&ra, alive);
    int b = bv_first_one(&ra);
    bv sa = ra; bv_set(&sa, b, 0);
    bv sb = bv_clone(&gram[b]); bv_and(&sb, alive); bv_set(&sb, a, 0);
    bv pa = bv_clone(&basis[a]), pb = bv_clone(&basis[b]);
    bv touched = bv_clone(&sa);
    for (int i = 0; i < touched.nw; i++) touched.w[i] |= sb.w[i];
    FOR_ONES(k, &touched) {
        if (bv_get(&sa, k)) { bv_xor(&gram[k], &sb); bv_xor(&basis[k], &pb); }
        if (bv_get(&sb, k)) { bv_xor(&gram[k], &sa); bv_xor(&basis[k], &pa); }
    }
    bv_set(alive, a, 0); bv_set(alive, b, 0);
    bv_free(&sa); bv_free(&sb);
    *touched_out = touched; *pa_out = pa; *pb_out = pb;
    return b;
}

/* Ordered set of (weight, index) as a binary min-heap with lazy deletion: an entry is
 * current iff key[idx] still equals (class, weight).  The minimum current entry is the
 * element BTreeSet::iter().next() returns in normal_form.rs:308/317. */
typedef struct { uint64_t *h; int n, cap; } heap;
static void heap_push(heap *hp, uint64_t x) {
    if (hp->n == hp->cap) { hp->cap = hp->cap ? hp->cap * 2 : 64; hp->h = (uint64_t *)realloc(hp->h, (size_t)hp->cap * 8); }
    int i = hp->n++;
    while (i > 0) { int p = (i - 1) / 2; if (hp->h[p] <= x) break; hp->h[i] = hp->h[p]; i = p; }
    hp->h[i] = x;
}
static void heap_pop(heap *hp) {
    uint64_t x = hp->h[--hp->n];
    int i = 0;
    while (1) {
        int l = 2 * i + 1, r = l + 1, m = i;
        uint64_t mv = x;
        if (l < hp->n && hp->h[l] < mv) { m = l; mv = hp->h[l]; }
        if (r < hp->n && hp->h[r] < mv) { m = r; }
        if (m == i) break;
        hp->h[i] = hp->h[m]; i = m;
    }
    if (hp->n) hp->h[i] = x;
}
typedef struct { uint8_t cls; uint32_t w; } key_t_;
static void reclass(int a, const bv *gram, const bv *alive, key_t_ *key, heap *dset, heap *oset) {
    if (!bv_get(alive, a)) { key[a].cls = 0; key[a].w = 0; return; }
    uint32_t w = bv_andcount(&gram[a], alive);
    if (bv_get(&gram[a], a)) {
        key[a].cls = 1; key[a].w = w; heap_push(dset, ((uint64_t)w << 32) | (uint32_t)a);
    } else if (w > 0) {
        key[a].cls = 2; key[a].w = w; heap_push(oset, ((uint64_t)w << 32) | (uint32_t)a);
    } else { key[a].cls = 0; key[a].w = 0; }
}
static int heap_min_current(heap *hp, const key_t_ *key, uint8_t cls) {
    while (hp->n) {
        uint64_t x = hp->h[0];
        int a = (int)(uint32_t)x;
        uint32_t w = (uint32_t)(x >> 32);
        if (key[a].cls == cls && key[a].w == w) return a;
        heap_pop(hp);
    }
    return -1;
}

#define RULE_FIRST 0
#define RULE_MINWEIGHT 1
typedef struct { bv *v; int n, cap; } bvlist;
static void bl_push(bvlist *l, bv x) {
    if (l->n == l->cap) { l->cap = l->cap ? l->cap * 2 : 16; l->v = (bv *)realloc(l->v, (size_t)l->cap * sizeof(bv)); }
    l->v[l->n++] = x;
}
/* normal_form.rs:240-336 */
static structure structure_new(const bm *b, const bv *parity, int rule) {
    int m = b->nrows;
    bv *gram = (bv *)calloc((size_t)(m ? m : 1), sizeof(bv)), *basis = (bv *)calloc((size_t)(m ? m : 1), sizeof(bv));
    for (int i = 0; i < m; i++) {
        gram[i] = bv_clone(&b->r[i]); bv_set(&gram[i], i, bv_get(parity, i));
        bv_init(&basis[i], m); bv_set(&basis[i], i, 1);
    }
    bv alive; bv_init(&alive, m);
    for (int i = 0; i < m; i++) bv_set(&alive, i, 1);
    bvlist pa = {0}, pb = {0}, odd = {0}, even = {0};
    if (rule == RULE_FIRST) {
        while (1) {
            int a = -1;
            FOR_ONES(i, &alive) if (bv_get(&gram[i], i)) { a = i; break; }
            if (a >= 0) {
                bv s, p; single_step(gram, basis, &alive, a, &s, &p);
                bl_push(&odd, p); bv_free(&s); continue;
            }
            FOR_ONES(i, &alive) if (bv_andcount(&gram[i], &alive) > 0) { a = i; break; }
            if (a < 0) break;
            bv t, x, y; hyper_step(gram, basis, &alive, a, &t, &x, &y);
            bl_push(&pa, x); bl_push(&pb, y); bv_free(&t);
        }
    } else {
        key_t_ *key = (key_t_ *)calloc((size_t)(m ? m : 1), sizeof(key_t_));
        heap dset = {0}, oset = {0};
        for (int a = 0; a < m; a++) reclass(a, gram, &alive, key, &dset, &oset);
        while (1) {
            int a = heap_min_current(&dset, key, 1);
            if (a >= 0) {
                bv s, p; single_step(gram, basis, &alive, a, &s, &p);
                bl_push(&odd, p);
                reclass(a, gram, &alive, key, &dset, &oset);
                FOR_ONES(bi, &s) reclass(bi, gram, &alive, key, &dset, &oset);
                bv_free(&s);
                continue;
            }
            a = heap_min_current(&oset, key, 2);
            if (a >= 0) {
                bv t, x, y;
                int partner = hyper_step(gram, basis, &alive, a, &t, &x, &y);
                bl_push(&pa, x); bl_push(&pb, y);
                reclass(a, gram, &alive, key, &dset, &oset);
                reclass(partner, gram, &alive, key, &dset, &oset);
                FOR_ONES(k, &t) reclass(k, gram, &alive, key, &dset, &oset);
                bv_free(&t);
                continue;
            }
            break;
        }
        free(key); free(dset.h); free(oset.h);
    }
    FOR_ONES(r, &alive) bl_push(&even, bv_clone(&basis[r]));
    for (int i = 0; i < m; i++) { bv_free(&gram[i]); bv_free(&basis[i]); }
    free(gram); free(basis); bv_free(&alive);
    structure s;
    s.m = m; s.g = pa.n; s.nodd = odd.n; s.neven = even.n;
    s.pa = pa.v; s.pb = pb.v; s.odd = odd.v; s.even = even.v;
    return s;
}
static void structure_free(structure *s) {
    for (int i = 0; i < s->g; i++) { bv_free(&s->pa[i]); bv_free(&s->pb[i]); }
    for (int i = 0; i < s->nodd; i++) bv_free(&s->odd[i]);
    for (int i = 0; i < s->neven; i++) bv_free(&s->even[i]);
    free(s->pa); free(s->pb); free(s->odd); free(s->even);
}
/* normal_form.rs:339-348 */
static unsigned z4_value(const bm *b, const bv *v0, const bv *v1, const bv *p) {
    unsigned lin = bv_andcount(p, v0) + 2 * bv_andcount(p, v1);
    unsigned t = 0;
    FOR_ONES(j, p) t += bv_andcount(&b->r[j], p);
    unsigned ep = (t / 2) & 1;
    return (lin + 2 * ep) & 3;
}
/* normal_form.rs:354-391 */
static diag_t structure_diagonal(const structure *s, const bm *b, const uint8_t *v) {
    bv v0, v1; bv_init(&v0, s->m); bv_init(&v1, s->m);
    for (int i = 0; i < s->m; i++) { bv_set(&v0, i, v[i] & 1); bv_set(&v1, i, (v[i] & 2) != 0); }
    diag_t d;
    bv_init(&d.wa, s->g); bv_init(&d.wb, s->g);
    for (int j = 0; j < s->g; j++) {
        bv_set(&d.wa, j, z4_value(b, &v0, &v1, &s->pa[j]) == 2);
        bv_set(&d.wb, j, z4_value(b, &v0, &v1, &s->pb[j]) == 2);
    }
    bv_init(&d.o1, s->nodd); bv_init(&d.o3, s->nodd);
    d.sigma = 0;
    for (int l = 0; l < s->nodd; l++) {
        if (z4_value(b, &v0, &v1, &s->odd[l]) == 1) { bv_set(&d.o1, l, 1); d.sigma++; }
        else { bv_set(&d.o3, l, 1); d.sigma--; }
    }
    bv_init(&d.we, s->neven);
    for (int l = 0; l < s->neven; l++) bv_set(&d.we, l, z4_value(b, &v0, &v1, &s->even[l]) == 2);
    bv_free(&v0); bv_free(&v1);
    return d;
}
static void diag_free(diag_t *d) { bv_free(&d->wa); bv_free(&d->wb); bv_free(&d->o1); bv_free(&d->o3); bv_free(&d->we); }
/* normal_form.rs:437-452: the single column (p_l[j])_l */
static void structure_column_of(const structure *s, int j, uvec *u) {
    uv_init(u, s);
    for (int l = 0; l < s->g; l++) { bv_set(&u->a, l, bv_get(&s->pa[l], j)); bv_set(&u->b, l, bv_get(&s->pb[l], j)); }
    for (int l = 0; l < s->nodd; l++) bv_set(&u->o, l, bv_get(&s->odd[l], j));
    for (int l = 0; l < s->neven; l++) bv_set(&u->e, l, bv_get(&s->even[l], j));
}
/* normal_form.rs:395-406 */
static void structure_transform(const structure *s, const bv *x, uvec *u) {
    uv_init(u, s);
    for (int l = 0; l < s->g; l++) { bv_set(&u->a, l, bv_dot(&s->pa[l], x)); bv_set(&u->b, l, bv_dot(&s->pb[l], x)); }
    for (int l = 0; l < s->nodd; l++) bv_set(&u->o, l, bv_dot(&s->odd[l], x));
    for (int l = 0; l < s->neven; l++) bv_set(&u->e, l, bv_dot(&s->even[l], x));
}
/* normal_form.rs:479-493 */
static unsigned phase8(const diag_t *d, const uvec *u) {
    int pc1 = (int)bv_andcount(&u->o, &d->o1), pc3 = (int)bv_andcount(&u->o, &d->o3);
    int n = d->sigma - 2 * (pc1 - pc3);
    unsigned cnt = 0;
    for (int i = 0; i < d->wa.nw; i++)
        cnt += (unsigned)__builtin_popcountll((d->wa.w[i] ^ u->a.w[i]) & (d->wb.w[i] ^ u->b.w[i]));
    if (cnt & 1) n += 4;
    return (unsigned)(((n % 8) + 8) % 8);
}
static double log2_magnitude(const structure *s) { return (double)s->g + (double)s->neven + (double)s->nodd / 2.0; }

/* ------------------------------------------------------------------ engine (src/engine.rs) */
#define NONE (-1)
#define LOW_BITS 14
#define RECOMPUTE_EVERY 2048
#define PARALLEL_MIN_DIM 16

typedef struct {
    int t, ne, rank;
    int *piv_col; bv *piv_row;
    int ncons; bv *cons;
    int d;
    bv *kernel; int **ksupp; int *ksupp_n;
    uvec *kernel_u;
} elim_t;
typedef struct { cx a[2], up, down; } term_t;

typedef struct {
    int nv, nf, m;
    int *fixed, *fixed_pos, *freev;
    bm b_fixed, b_ff;
    bv parity;
    structure st;
    uvec *ucols; /* nf */
    /* branching */
    int t;
    int *term_vars;
    uvec *mcols;
    elim_t el;
    /* values */
    diag_t dg;
    uint8_t *fixed_v;
    uint32_t *fixed_theta;
    term_t *terms;
    int num_h;
    uint32_t global;
    int zero;
} engine;

/* engine.rs:119-184 */
static void elim_new(elim_t *e, const structure *st, const uvec *mcols, int t) {
    int ne = st->neven;
    e->t = t; e->ne = ne;
    bv *rk = (bv *)calloc((size_t)(ne ? ne : 1), sizeof(bv)), *rr = (bv *)calloc((size_t)(ne ? ne : 1), sizeof(bv));
    for (int r = 0; r < ne; r++) {
        bv_init(&rk[r], t); bv_init(&rr[r], ne); bv_set(&rr[r], r, 1);
        for (int c = 0; c < t; c++) if (bv_get(&mcols[c].e, r)) bv_set(&rk[r], c, 1);
    }
    int *pcols = (int *)malloc(sizeof(int) * (size_t)(t + 1));
    int rank = 0;
    for (int col = 0; col < t; col++) {
        int r = -1;
        for (int i = rank; i < ne; i++) if (bv_get(&rk[i], col)) { r = i; break; }
        if (r < 0) continue;
        bv tk = rk[rank]; rk[rank] = rk[r]; rk[r] = tk;
        bv tr = rr[rank]; rr[rank] = rr[r]; rr[r] = tr;
        for (int r2 = 0; r2 < ne; r2++)
            if (r2 != rank && bv_get(&rk[r2], col)) { bv_xor(&rk[r2], &rk[rank]); bv_xor(&rr[r2], &rr[rank]); }
        pcols[rank++] = col;
    }
    e->rank = rank;
    e->piv_col = pcols;
    e->piv_row = (bv *)calloc((size_t)(rank ? rank : 1), sizeof(bv));
    for (int i = 0; i < rank; i++) e->piv_row[i] = bv_clone(&rr[i]);
    e->ncons = ne - rank;
    e->cons = (bv *)calloc((size_t)(e->ncons ? e->ncons : 1), sizeof(bv));
    for (int i = rank; i < ne; i++) e->cons[i - rank] = bv_clone(&rr[i]);
    uint8_t *isp = (uint8_t *)calloc((size_t)t + 1, 1);
    for (int i = 0; i < rank; i++) isp[pcols[i]] = 1;
    e->d = t - rank;
    e->kernel = (bv *)calloc((size_t)(e->d ? e->d : 1), sizeof(bv));
    e->ksupp = (int **)calloc((size_t)(e->d ? e->d : 1), sizeof(int *));
    e->ksupp_n = (int *)calloc((size_t)(e->d ? e->d : 1), sizeof(int));
    e->kernel_u = (uvec *)calloc((size_t)(e->d ? e->d : 1), sizeof(uvec));
    int kj = 0;
    for (int j = 0; j < t; j++) {
        if (isp[j]) continue;
        bv n; bv_init(&n, t); bv_set(&n, j, 1);
        for (int i = 0; i < rank; i++) if (bv_get(&rk[i], j)) bv_set(&n, pcols[i], 1);
        e->kernel[kj] = n;
        e->ksupp[kj] = (int *)malloc(sizeof(int) * (size_t)(t + 1));
        int c = 0;
        FOR_ONES(k, &n) e->ksupp[kj][c++] = k;
        e->ksupp_n[kj] = c;
        uv_init(&e->kernel_u[kj], st);
        for (int q = 0; q < c; q++) uv_xor(&e->kernel_u[kj], &mcols[e->ksupp[kj][q]]);
        kj++;
    }
    for (int r = 0; r < ne; r++) { bv_free(&rk[r]); bv_free(&rr[r]); }
    free(rk); free(rr); free(isp);
}
static void elim_free(elim_t *e) {
    for (int i = 0; i < e->rank; i++) bv_free(&e->piv_row[i]);
    for (int i = 0; i < e->ncons; i++) bv_free(&e->cons[i]);
    for (int j = 0; j < e->d; j++) { bv_free(&e->kernel[j]); free(e->ksupp[j]); uv_free(&e->kernel_u[j]); }
    free(e->piv_col); free(e->piv_row); free(e->cons); free(e->kernel); free(e->ksupp); free(e->ksupp_n); free(e->kernel_u);
}
/* engine.rs:188-201 */
static int elim_solve(const elim_t *e, const bv *kappa, bv *s) {
    for (int i = 0; i < e->ncons; i++) if (bv_dot(&e->cons[i], kappa)) return 0;
    bv_clear(s);
    for (int i = 0; i < e->rank; i++) if (bv_dot(&e->piv_row[i], kappa)) bv_set(s, e->piv_col[i], 1);
    return 1;
}
/* engine.rs:232-238 */
static term_t term_new(uint32_t theta) {
    cx e = phase_to_complex(theta);
    term_t t;
    t.a[0] = cscale(cadd(C(1, 0), e), 0.5);
    t.a[1] = cscale(csub(C(1, 0), e), 0.5);
    t.up = cdiv(t.a[1], t.a[0]);
    t.down = cdiv(t.a[0], t.a[1]);
    return t;
}
/* engine.rs:289-390 (Engine::new + build_branching + bind_values) */
static engine *engine_new(const pathsum *ps, const int *fixed, int nf) {
    engine *E = (engine *)calloc(1, sizeof(engine));
    int nv = ps->nv;
    E->nv = nv; E->nf = nf;
    E->fixed = (int *)malloc(sizeof(int) * (size_t)(nf + 1)); memcpy(E->fixed, fixed, sizeof(int) * (size_t)nf);
    E->fixed_pos = (int *)malloc(sizeof(int) * (size_t)(nv + 1));
    for (int i = 0; i < nv; i++) E->fixed_pos[i] = NONE;
    for (int i = 0; i < nf; i++) E->fixed_pos[fixed[i]] = i;
    E->freev = (int *)malloc(sizeof(int) * (size_t)(nv + 1));
    int m = 0;
    for (int i = 0; i < nv; i++) if (!ps->dead[i] && E->fixed_pos[i] == NONE) E->freev[m++] = i;
    E->m = m;
    int *fidx = (int *)malloc(sizeof(int) * (size_t)(nv + 1));
    for (int i = 0; i < nv; i++) fidx[i] = NONE;
    for (int i = 0; i < m; i++) fidx[E->freev[i]] = i;
    bm_init(&E->b_ff, m, m);
    for (int i = 0; i < m; i++) FOR_ONES(j, &ps->b.r[E->freev[i]]) if (fidx[j] != NONE) bv_set(&E->b_ff.r[i], fidx[j], 1);
    bv_init(&E->parity, m);
    for (int i = 0; i < m; i++) bv_set(&E->parity, i, ps->v[E->freev[i]] & 1);
    bm_init(&E->b_fixed, nf, nf);
    for (int i = 0; i < nf; i++) FOR_ONES(j, &ps->b.r[fixed[i]]) if (E->fixed_pos[j] != NONE) bv_set(&E->b_fixed.r[i], E->fixed_pos[j], 1);
    E->st = structure_new(&E->b_ff, &E->parity, RULE_MINWEIGHT);
    const structure *st = &E->st;
    /* tcols / ucols: Pᵀ (column of B between free vars and fixed f) */
    E->ucols = (uvec *)calloc((size_t)(nf ? nf : 1), sizeof(uvec));
    uvec *colcache = (uvec *)calloc((size_t)(m ? m : 1), sizeof(uvec));
    uint8_t *have = (uint8_t *)calloc((size_t)m + 1, 1);
    for (int i = 0; i < nf; i++) {
        uv_init(&E->ucols[i], st);
        FOR_ONES(j, &ps->b.r[fixed[i]]) {
            int fj = fidx[j];
            if (fj == NONE) continue;
            if (!have[fj]) { structure_column_of(st, fj, &colcache[fj]); have[fj] = 1; }
            uv_xor(&E->ucols[i], &colcache[fj]);
        }
    }
    /* branching: engine.rs:372-378 */
    E->term_vars = (int *)malloc(sizeof(int) * (size_t)(m + 1));
    int t = 0;
    for (int i = 0; i < m; i++) if (ps->theta[E->freev[i]] != 0) E->term_vars[t++] = i;
    E->t = t;
    E->mcols = (uvec *)calloc((size_t)(t ? t : 1), sizeof(uvec));
    for (int k = 0; k < t; k++) {
        int i = E->term_vars[k];
        if (!have[i]) { structure_column_of(st, i, &colcache[i]); have[i] = 1; }
        uv_init(&E->mcols[k], st); uv_copy(&E->mcols[k], &colcache[i]);
    }
    for (int i = 0; i < m; i++) if (have[i]) uv_free(&colcache[i]);
    free(colcache); free(have); free(fidx);
    elim_new(&E->el, st, E->mcols, t);
    /* bind_values: engine.rs:381-390 */
    uint8_t *vfree = (uint8_t *)malloc((size_t)m + 1);
    for (int i = 0; i < m; i++) vfree[i] = ps->v[E->freev[i]];
    E->dg = structure_diagonal(st, &E->b_ff, vfree);
    free(vfree);
    E->terms = (term_t *)calloc((size_t)(t ? t : 1), sizeof(term_t));
    for (int k = 0; k < t; k++) E->terms[k] = term_new(ps->theta[E->freev[E->term_vars[k]]]);
    E->fixed_v = (uint8_t *)malloc((size_t)nf + 1);
    E->fixed_theta = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nf + 1));
    for (int i = 0; i < nf; i++) { E->fixed_v[i] = ps->v[fixed[i]]; E->fixed_theta[i] = ps->theta[fixed[i]]; }
    E->num_h = ps->num_h; E->global = ps->global; E->zero = ps->zero;
    return E;
}
static void engine_free(engine *E) {
    if (!E) return;
    free(E->fixed); free(E->fixed_pos); free(E->freev);
    bm_free(&E->b_fixed); bm_free(&E->b_ff); bv_free(&E->parity);
    for (int i = 0; i < E->nf; i++) uv_free(&E->ucols[i]);
    free(E->ucols);
    for (int k = 0; k < E->t; k++) uv_free(&E->mcols[k]);
    free(E->mcols); free(E->term_vars);
    elim_free(&E->el);
    diag_free(&E->dg);
    structure_free(&E->st);
    free(E->fixed_v); free(E->fixed_theta); free(E->terms);
    free(E);
}
static double engine_magnitude(const engine *E) { /* engine.rs:563-565 */
    return pow(2.0, log2_magnitude(&E->st) - (double)E->num_h / 2.0);
}
/* Per-evaluation state after prepare (engine.rs:569-610). */
typedef struct {
    int ok;
    uint32_t phase;
    cx c_start;
    uvec u;
    bv s0;
} prep_t;
static void prep_init(prep_t *p, const engine *E) { uv_init(&p->u, &E->st); bv_init(&p->s0, E->t); p->ok = 0; }
static void prep_free(prep_t *p) { uv_free(&p->u); bv_free(&p->s0); }
static int engine_prepare(const engine *E, const uint8_t *values, prep_t *p) {
    p->ok = 0;
    if (E->zero) return 0;
    int nf = E->nf;
    int *ones = (int *)malloc(sizeof(int) * (size_t)(nf + 1)), no = 0;
    for (int i = 0; i < nf; i++) if (values[i]) ones[no++] = i;
    uint32_t z4 = 0, th = E->global;
    for (int ii = 0; ii < no; ii++) {
        int f = ones[ii];
        z4 += E->fixed_v[f]; th += E->fixed_theta[f];
        for (int jj = ii + 1; jj < no; jj++) if (bv_get(&E->b_fixed.r[f], ones[jj])) z4 += 2;
    }
    p->phase = th + z4_phase(z4 & 3);
    uv_clear(&p->u);
    for (int ii = 0; ii < no; ii++) uv_xor(&p->u, &E->ucols[ones[ii]]);
    free(ones);
    bv kappa = bv_clone(&E->dg.we);
    bv_xor(&kappa, &p->u.e);
    int ok = elim_solve(&E->el, &kappa, &p->s0);
    bv_free(&kappa);
    if (!ok) return 0;
    cx c = C(1, 0);
    for (int k = 0; k < E->t; k++) {
        if (bv_get(&p->s0, k)) { uv_xor(&p->u, &E->mcols[k]); c = cmul(c, E->terms[k].a[1]); }
        else c = cmul(c, E->terms[k].a[0]);
    }
    p->c_start = c;
    p->ok = 1;
    return 1;
}
static cx engine_weight(const engine *E, const bv *sv) { /* engine.rs:661-667 */
    cx c = C(1, 0);
    for (int k = 0; k < E->t; k++) c = cmul(c, E->terms[k].a[bv_get(sv, k)]);
    return c;
}
/* engine.rs:674-687 + 696-722: the chunk `hi` of the subspace walk. */
static cx engine_chunk(const engine *E, const prep_t *p, uint64_t hi) {
    const elim_t *e = &E->el;
    int d = e->d, dl = d < LOW_BITS ? d : LOW_BITS;
    uvec u; uv_init(&u, &E->st); uv_copy(&u, &p->u);
    bv sv = bv_clone(&p->s0);
    cx c = p->c_start;
    if (hi != 0) {
        for (int j = 0; j < d - dl; j++)
            if ((hi >> j) & 1) { uv_xor(&u, &e->kernel_u[dl + j]); bv_xor(&sv, &e->kernel[dl + j]); }
        c = engine_weight(E, &sv);
    }
    cx acc = C(0, 0);
    uint64_t steps = 1ull << dl;
    for (uint64_t i = 0; i < steps; i++) {
        unsigned k8 = phase8(&E->dg, &u);
        acc = cadd(acc, cmul(c, ROOT8[k8]));
        if (i + 1 < steps) {
            int j = __builtin_ctzll(i + 1);
            uv_xor(&u, &e->kernel_u[j]);
            if ((i + 1) % RECOMPUTE_EVERY == 0) {
                bv_xor(&sv, &e->kernel[j]);
                c = engine_weight(E, &sv);
            } else {
                for (int q = 0; q < e->ksupp_n[j]; q++) {
                    int k = e->ksupp[j][q];
                    c = cmul(c, bv_get(&sv, k) ? E->terms[k].down : E->terms[k].up);
                    bv_flip(&sv, k);
                }
            }
        }
    }
    uv_free(&u); bv_free(&sv);
    return acc;
}
static int engine_nchunks_log2(const engine *E) { int d = E->el.d; return d - (d < LOW_BITS ? d : LOW_BITS); }

/* ------------------------------------------------------------------ rank engine (src/rank.rs) */
#define MAX_PAIRS 14
#define MASK30 ((1u << 30) - 1)
typedef struct { int a, b; } pair_t;
static int cmp_u64(const void *x, const void *y) {
    uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return a < b ? -1 : (a > b ? 1 : 0);
}
/* rank.rs:62-84: returns number of pairs; *nt = number of T-class pairs. */
static int pair_candidates(const pathsum *ps, const int *fixed, int nf, pair_t *out, int *nt) {
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(ps->nv + 1));
    int nk = 0;
    for (int k = 0; k < ps->nv; k++) {
        if (ps->dead[k] || ps->theta[k] == 0) continue;
        int isf = 0;
        for (int i = 0; i < nf; i++) if (fixed[i] == k) { isf = 1; break; }
        if (isf) continue;
        uint32_t r = ps->theta[k] & MASK30;
        uint32_t o = (uint32_t)(((uint64_t)MASK30 + 1 - r) & MASK30);
        uint32_t canon = r < o ? r : o;
        keys[nk++] = ((uint64_t)canon << 32) | (uint32_t)k; /* groups ordered by canon, vars by k */
    }
    qsort(keys, (size_t)nk, 8, cmp_u64);
    pair_t *tp = (pair_t *)malloc(sizeof(pair_t) * (size_t)(nk + 1)), *gp = (pair_t *)malloc(sizeof(pair_t) * (size_t)(nk + 1));
    int ntp = 0, ngp = 0;
    for (int i = 0; i < nk;) {
        uint32_t canon = (uint32_t)(keys[i] >> 32);
        int j = i;
        while (j < nk && (uint32_t)(keys[j] >> 32) == canon) j++;
        for (int q = i; q + 1 < j; q += 2) {
            pair_t pr = {(int)(uint32_t)keys[q], (int)(uint32_t)keys[q + 1]};
            if (canon == (1u << 29)) tp[ntp++] = pr; else gp[ngp++] = pr;
        }
        i = j;
    }
    memcpy(out, tp, sizeof(pair_t) * (size_t)ntp);
    memcpy(out + ntp, gp, sizeof(pair_t) * (size_t)ngp);
    *nt = ntp;
    free(keys); free(tp); free(gp);
    return ntp + ngp;
}
/* rank.rs:205-222 */
static int best_pairs(const engine *base, int available, int tclass) {
    double m = (double)base->m;
    double words = (double)(base->m / 64 + 1);
    double ldl = 2.0 * m * m * m / 64.0 + 50.0 * m + 2000.0;
    double step = 20.0 + 4.0 * words + (double)base->t / 2.0;
    int best = 0; double bestc = INFINITY;
    int lim = available < MAX_PAIRS ? available : MAX_PAIRS;
    for (int p = 0; p <= lim; p++) {
        int removed = 2 * (p < tclass ? p : tclass) + (p > tclass ? p - tclass : 0);
        int d = base->el.d > removed ? base->el.d - removed : 0;
        double cost = pow(2.0, (double)p) * ((p == 0 ? 0.0 : ldl) + pow(2.0, (double)d) * step);
        if (cost < bestc) { best = p; bestc = cost; }
    }
    return best;
}
typedef struct { int nbr, pairs; engine **br; } rank_engine;
/* rank.rs:88-103 */
static rank_engine rank_new(const pathsum *ps, const int *fixed, int nf, int pairs) {
    pair_t *c = (pair_t *)malloc(sizeof(pair_t) * (size_t)(ps->nv + 1));
    int nt, nc = pair_candidates(ps, fixed, nf, c, &nt);
    int p = pairs < nc ? pairs : nc;
    if (p > MAX_PAIRS) p = MAX_PAIRS;
    rank_engine r; r.pairs = p; r.nbr = 1 << p;
    r.br = (engine **)calloc((size_t)r.nbr, sizeof(engine *));
    for (int pat = 0; pat < r.nbr; pat++) {
        pathsum b = ps_clone(ps);
        for (int i = 0; i < p; i++) ps_substitute(&b, c[i].a, c[i].b, (pat >> i) & 1);
        r.br[pat] = engine_new(&b, fixed, nf);
        ps_free(&b);
    }
    free(c);
    return r;
}
/* rank.rs:115-123 */
static rank_engine rank_auto(const pathsum *ps, const int *fixed, int nf) {
    engine *base = engine_new(ps, fixed, nf);
    pair_t *c = (pair_t *)malloc(sizeof(pair_t) * (size_t)(ps->nv + 1));
    int nt, nc = pair_candidates(ps, fixed, nf, c, &nt);
    free(c);
    int p = best_pairs(base, nc, nt);
    if (p == 0) {
        rank_engine r; r.pairs = 0; r.nbr = 1; r.br = (engine **)calloc(1, sizeof(engine *)); r.br[0] = base;
        return r;
    }
    engine_free(base);
    return rank_new(ps, fixed, nf, p);
}
static rank_engine build_engine(const pathsum *ps, const int *fixed, int nf, int strategy, int pairs) { /* sim.rs:65-71 */
    if (strategy == 0) return rank_auto(ps, fixed, nf);
    if (strategy == 1) return rank_new(ps, fixed, nf, 0);
    return rank_new(ps, fixed, nf, pairs);
}
static void rank_free(rank_engine *r) { for (int i = 0; i < r->nbr; i++) engine_free(r->br[i]); free(r->br); }

/* ------------------------------------------------------------------ parallel evaluation */
/* One (job, chunk) work item list evaluated by a pool of threads; per-item results are
 * summed per job in chunk order afterwards (engine.rs:688-692 sums chunks; here the order
 * is fixed so results are reproducible). */
typedef struct {
    const engine *E;
    prep_t prep;
    int nchunk_log2;
    cx *chunk_out;
} job_t;
typedef struct {
    job_t *jobs;
    int njobs;
    int64_t *item_start; /* prefix sums of chunk counts */
    int64_t nitems;
    atomic_llong next;
} pool_t;
static void *pool_worker(void *arg) {
    pool_t *P = (pool_t *)arg;
    while (1) {
        int64_t it = atomic_fetch_add(&P->next, 1);
        if (it >= P->nitems) break;
        int lo = 0, hi = P->njobs - 1;
        while (lo < hi) { int mid = (lo + hi + 1) / 2; if (P->item_start[mid] <= it) lo = mid; else hi = mid - 1; }
        job_t *J = &P->jobs[lo];
        uint64_t ch = (uint64_t)(it - P->item_start[lo]);
        J->chunk_out[ch] = engine_chunk(J->E, &J->prep, ch);
    }
    return NULL;
}
static void run_pool(job_t *jobs, int njobs, int nthreads) {
    pool_t P; P.jobs = jobs; P.njobs = njobs;
    P.item_start = (int64_t *)malloc(sizeof(int64_t) * (size_t)(njobs + 1));
    int64_t acc = 0;
    for (int i = 0; i < njobs; i++) { P.item_start[i] = acc; if (jobs[i].prep.ok) acc += 1ll << jobs[i].nchunk_log2; }
    P.item_start[njobs] = acc;
    P.nitems = acc;
    atomic_init(&P.next, 0);
    /* jobs whose prepare failed contribute zero items: item_start makes them empty ranges */
    if (nthreads <= 1 || acc <= 1) {
        pool_worker(&P);
    } else {
        pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, pool_worker, &P);
        for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
        free(th);
    }
    free(P.item_start);
}

/* ------------------------------------------------------------------ simulator (src/sim.rs) */
struct pqo_sim {
    circuit c;
    pathsum ps;
    rank_engine eng;
    int strategy, pairs;
    int have_sw;
    double last_branches; /* branches enumerated by the last pqo_amplitudes call */
    pathsum sw;
    int *junction;
    uint8_t *jneg;
};
static int once_init = 0;
pqo_sim *pqo_sim_new(int nq, int ngates, const uint8_t *op, const int32_t *q0, const int32_t *q1,
                     const uint32_t *phase, int strategy, int pairs) {
    if (!once_init) { init_root8(); once_init = 1; }
    pqo_sim *s = (pqo_sim *)calloc(1, sizeof(pqo_sim));
    s->c = circuit_from(nq, ngates, op, q0, q1, phase);
    s->ps = ps_from_circuit(&s->c);
    s->strategy = strategy; s->pairs = pairs;
    int *f = (int *)malloc(sizeof(int) * (size_t)(2 * nq + 1));
    int nf = ps_io_vars(&s->ps, f);
    s->eng = build_engine(&s->ps, f, nf, strategy, pairs);
    free(f);
    return s;
}
void pqo_sim_free(pqo_sim *s) {
    if (!s) return;
    free(s->c.g); ps_free(&s->ps); rank_free(&s->eng);
    if (s->have_sw) { ps_free(&s->sw); free(s->junction); free(s->jneg); }
    free(s);
}
void pqo_stats(const pqo_sim *s, int64_t out[8]) {
    const engine *E = s->eng.br[0];
    out[0] = E->m; out[1] = E->st.g; out[2] = E->st.nodd; out[3] = E->st.neven;
    out[4] = E->t; out[5] = E->el.d; out[6] = s->eng.pairs; out[7] = s->eng.nbr;
}
/* values aligned with E->fixed from an assignment list (engine.rs:521-533) */
static void values_from_asg(const engine *E, const asg_t *a, int na, uint8_t *vals) {
    memset(vals, 0, (size_t)E->nf + 1);
    for (int i = 0; i < na; i++) { int p = E->fixed_pos[a[i].var]; if (p != NONE) vals[p] = (uint8_t)a[i].val; }
}
static int default_threads(int n) {
    if (n > 0) return n;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}
/* Evaluate the rank engine `r` on `na` assignments; out[i] = sum over branches. */
/* Returns the number of branches enumerated (2^d of every job whose prepare succeeded). */
static double eval_many(const rank_engine *r, int na, asg_t **asg, int *asg_n, cx *out, int nthreads) {
    int njobs = na * r->nbr;
    double enumerated = 0.0;
    job_t *jobs = (job_t *)calloc((size_t)(njobs ? njobs : 1), sizeof(job_t));
    for (int i = 0; i < na; i++) {
        for (int b = 0; b < r->nbr; b++) {
            job_t *J = &jobs[i * r->nbr + b];
            const engine *E = r->br[b];
            J->E = E;
            prep_init(&J->prep, E);
            J->nchunk_log2 = engine_nchunks_log2(E);
            if (asg_n[i] < 0) continue;
            uint8_t *vals = (uint8_t *)malloc((size_t)E->nf + 1);
            values_from_asg(E, asg[i], asg_n[i], vals);
            engine_prepare(E, vals, &J->prep);
            free(vals);
            if (J->prep.ok) {
                J->chunk_out = (cx *)calloc((size_t)1 << J->nchunk_log2, sizeof(cx));
                enumerated += ldexp(1.0, E->el.d);
            }
        }
    }
    run_pool(jobs, njobs, nthreads);
    for (int i = 0; i < na; i++) {
        cx tot = C(0, 0);
        for (int b = 0; b < r->nbr; b++) {
            job_t *J = &jobs[i * r->nbr + b];
            cx v = C(0, 0);
            if (J->prep.ok) {
                cx sum = C(0, 0);
                for (uint64_t ch = 0; ch < (1ull << J->nchunk_log2); ch++) sum = cadd(sum, J->chunk_out[ch]);
                v = cscale(cmul(phase_to_complex(J->prep.phase), sum), engine_magnitude(J->E));
            }
            tot = cadd(tot, v);
            prep_free(&J->prep);
            free(J->chunk_out);
        }
        out[i] = tot;
    }
    free(jobs);
    return enumerated;
}
void pqo_amplitudes(pqo_sim *s, int n, const uint64_t *xs, const uint64_t *ys, double *out, int nthreads) {
    int nw = (s->ps.nq + 63) / 64;
    if (nw == 0) nw = 1;
    asg_t **asg = (asg_t **)calloc((size_t)(n ? n : 1), sizeof(asg_t *));
    int *an = (int *)calloc((size_t)(n ? n : 1), sizeof(int));
    for (int i = 0; i < n; i++) {
        asg[i] = (asg_t *)malloc(sizeof(asg_t) * (size_t)(2 * s->ps.nq + 1));
        an[i] = ps_boundary(&s->ps, xs + (size_t)i * nw, ys + (size_t)i * nw, asg[i]);
    }
    cx *res = (cx *)calloc((size_t)(n ? n : 1), sizeof(cx));
    s->last_branches = eval_many(&s->eng, n, asg, an, res, default_threads(nthreads));
    for (int i = 0; i < n; i++) { out[2 * i] = res[i].re; out[2 * i + 1] = res[i].im; free(asg[i]); }
    free(asg); free(an); free(res);
}
/* sim.rs:215-231 */
double pqo_marginal(pqo_sim *s, const uint64_t *x, int nmeas, const int32_t *qubits, const uint8_t *outcomes) {
    int nq = s->ps.nq;
    if (!s->have_sw) {
        s->junction = (int *)malloc(sizeof(int) * (size_t)(nq + 1));
        s->jneg = (uint8_t *)malloc((size_t)nq + 1);
        s->sw = ps_sandwich(&s->c, s->junction, s->jneg);
        s->have_sw = 1;
    }
    asg_t *a = (asg_t *)malloc(sizeof(asg_t) * (size_t)(2 * nq + nmeas + 1));
    int na = 0, ok = 1;
    for (int q = 0; q < nq && ok; q++) ok = asg_put(a, &na, q, bit_of(x, q));
    for (int q = 0; q < nq && ok; q++) ok = asg_put(a, &na, s->sw.outputs[q], bit_of(x, q) ^ s->sw.out_neg[q]);
    for (int i = 0; i < nmeas && ok; i++) ok = asg_put(a, &na, s->junction[qubits[i]], outcomes[i] ^ s->jneg[qubits[i]]);
    if (!ok) { free(a); return 0.0; }
    int *f = (int *)malloc(sizeof(int) * (size_t)(2 * nq + nmeas + 1));
    int nf = ps_io_vars(&s->sw, f);
    for (int i = 0; i < nmeas; i++) {
        int j = s->junction[qubits[i]], seen = 0;
        for (int k = 0; k < nf; k++) if (f[k] == j) { seen = 1; break; }
        if (!seen) f[nf++] = j;
    }
    rank_engine r = build_engine(&s->sw, f, nf, s->strategy, s->pairs);
    cx v;
    asg_t *al[1] = {a};
    int an[1] = {na};
    eval_many(&r, 1, al, an, &v, default_threads(0));
    rank_free(&r); free(f); free(a);
    return v.re > 0.0 ? v.re : 0.0;
}
int pqo_brute_force(pqo_sim *s, const uint64_t *x, const uint64_t *y, double out[2]) {
    asg_t *a = (asg_t *)malloc(sizeof(asg_t) * (size_t)(2 * s->ps.nq + 1));
    int na = ps_boundary(&s->ps, x, y, a);
    cx v = C(0, 0);
    int rc = 0;
    if (na >= 0) rc = ps_brute_force(&s->ps, a, na, &v);
    free(a);
    out[0] = v.re; out[1] = v.im;
    return rc;
}

double pqo_last_branches(const pqo_sim *s) { return s->last_branches; }

/* SplitMix64 (src/rng.rs:12-27): new(seed) = seed + golden; next_u64 advances by golden and mixes;
 * next_f64 = (next_u64 >> 11) / 2^53. */
typedef struct { uint64_t s; } srng;
static srng srng_new(uint64_t seed) { srng r = {seed + 0x9E3779B97F4A7C15ull}; return r; }
static uint64_t srng_u64(srng *r) {
    r->s += 0x9E3779B97F4A7C15ull;
    uint64_t z = r->s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double srng_f64(srng *r) { return (double)(srng_u64(r) >> 11) / 9007199254740992.0; }

/* Engine::estimate (src/engine.rs:616-659): prepare; the exact sum when 2^d <= samples;
 * otherwise samples in chunks of 1024, chunk ci drawing from Rng::new(seed ^ ci * golden),
 * one fresh word per 64 coordinates; x = weight(sv) * ROOT8[phase8(u)].  Chunk sums are
 * accumulated in chunk order (the reference's rayon reduce groups them differently). */
static void engine_estimate(const engine *E, const uint8_t *values, int64_t samples, uint64_t seed, cx *val, double *se) {
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    *val = C(0, 0);
    *se = 0.0;
    prep_t p;
    prep_init(&p, E);
    if (!engine_prepare(E, values, &p)) { prep_free(&p); return; }
    const elim_t *e = &E->el;
    const int d = e->d;
    const cx norm = cscale(phase_to_complex(p.phase), engine_magnitude(E));
    if (d < 63 && (1ull << d) <= (uint64_t)samples) {
        cx sum = C(0, 0);
        for (uint64_t ch = 0; ch < (1ull << engine_nchunks_log2(E)); ch++) sum = cadd(sum, engine_chunk(E, &p, ch));
        *val = cmul(norm, sum);
        prep_free(&p);
        return;
    }
    const int64_t chunks = (samples + 1023) / 1024;
    cx sum = C(0, 0);
    double sq = 0.0;
    uvec u; uv_init(&u, &E->st);
    bv sv = bv_clone(&p.s0);
    for (int64_t ci = 0; ci < chunks; ci++) {
        srng r = srng_new(seed ^ ((uint64_t)ci * golden));
        const int64_t n_here = samples - ci * 1024 < 1024 ? samples - ci * 1024 : 1024;
        for (int64_t k = 0; k < n_here; k++) {
            uv_copy(&u, &p.u);
            bv_free(&sv);
            sv = bv_clone(&p.s0);
            uint64_t word = 0;
            for (int j = 0; j < d; j++) {
                if (j % 64 == 0) word = srng_u64(&r);
                if ((word >> (j % 64)) & 1) { uv_xor(&u, &e->kernel_u[j]); bv_xor(&sv, &e->kernel[j]); }
            }
            const cx x = cmul(engine_weight(E, &sv), ROOT8[phase8(&E->dg, &u)]);
            sum = cadd(sum, x);
            sq += x.re * x.re + x.im * x.im;
        }
    }
    uv_free(&u); bv_free(&sv); prep_free(&p);
    const double n = (double)samples;
    const cx mean = C(sum.re / n, sum.im / n);
    double var = sq / n - (mean.re * mean.re + mean.im * mean.im);
    if (var < 0.0) var = 0.0;
    const double scale = ldexp(1.0, d);
    *val = cscale(cmul(norm, mean), scale);
    *se = sqrt(norm.re * norm.re + norm.im * norm.im) * scale * sqrt(var / n);
}

/* Simulator::amplitude_estimate (src/sim.rs:184-193) -> RankEngine::estimate (src/rank.rs:149-171):
 * one engine: Engine::estimate; 2^p engines: samples i draw Rng::new(seed ^ i * golden).below(nb)
 * and evaluate that engine exactly; value nb * mean, stderr nb * sqrt(var / n). */
void pqo_amplitude_estimate(pqo_sim *s, const uint64_t *x, const uint64_t *y, int64_t samples, uint64_t seed,
                            double out[3]) {
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    out[0] = out[1] = out[2] = 0.0;
    asg_t *a = (asg_t *)malloc(sizeof(asg_t) * (size_t)(2 * s->ps.nq + 1));
    int na = ps_boundary(&s->ps, x, y, a);
    if (na < 0) { free(a); return; }
    const rank_engine *r = &s->eng;
    if (r->nbr == 1) {
        const engine *E = r->br[0];
        uint8_t *vals = (uint8_t *)malloc((size_t)E->nf + 1);
        values_from_asg(E, a, na, vals);
        cx v; double se;
        engine_estimate(E, vals, samples, seed, &v, &se);
        out[0] = v.re; out[1] = v.im; out[2] = se;
        free(vals); free(a);
        return;
    }
    /* exact value of every branch engine once, then the sampled mean */
    rank_engine one; one.nbr = 1; one.pairs = 0;
    cx *vb = (cx *)malloc(sizeof(cx) * (size_t)r->nbr);
    asg_t *al[1] = {a};
    int an[1] = {na};
    for (int b = 0; b < r->nbr; b++) {
        engine *eb = r->br[b];
        one.br = &eb;
        eval_many(&one, 1, al, an, &vb[b], default_threads(0));
    }
    cx sum = C(0, 0);
    double sq = 0.0;
    for (int64_t i = 0; i < samples; i++) {
        srng ri = srng_new(seed ^ ((uint64_t)i * golden));
        const cx v = vb[srng_u64(&ri) % (uint64_t)r->nbr];
        sum = cadd(sum, v);
        sq += v.re * v.re + v.im * v.im;
    }
    const double n = (double)samples, nb = (double)r->nbr;
    const cx mean = C(sum.re / n, sum.im / n);
    double var = sq / n - (mean.re * mean.re + mean.im * mean.im);
    if (var < 0.0) var = 0.0;
    out[0] = mean.re * nb; out[1] = mean.im * nb; out[2] = nb * sqrt(var / n);
    free(vb); free(a);
}

/* Pair candidates of the circuit's path sum with its io variables fixed (rank.rs:62-84) and
 * its live variables (pathsum.rs live_vars): out = {candidates, live variables}. */
void pqo_path_info(const pqo_sim *s, int64_t out[2]) {
    int *f = (int *)malloc(sizeof(int) * (size_t)(2 * s->ps.nq + 1));
    int nf = ps_io_vars(&s->ps, f);
    pair_t *cands = (pair_t *)malloc(sizeof(pair_t) * (size_t)(s->ps.nv + 1));
    int nt;
    out[0] = pair_candidates(&s->ps, f, nf, cands, &nt);
    int live = 0;
    for (int v = 0; v < s->ps.nv; v++) live += !s->ps.dead[v];
    out[1] = live;
    free(cands); free(f);
}

/* approx::estimate_amplitude (src/approx.rs:96-135): lazy pair sampling.  Sample i seeds
 * Rng::new(seed ^ i * golden), draws one bit per pair for the first min(pairs, candidates, 62)
 * pair candidates, builds that branch engine from a copy of the path sum and evaluates it
 * exactly when its dimension is <= exact_dim_limit, else by Engine::estimate with 2^14 points
 * and the sample's next draw as seed.  out: 2^p mean (re, im), 2^p sqrt(var / n). */
void pqo_amplitude_estimate_pairs(pqo_sim *s, const uint64_t *x, const uint64_t *y, int pairs, int64_t samples,
                                  uint64_t seed, int exact_dim_limit, double out[3]) {
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    out[0] = out[1] = out[2] = 0.0;
    asg_t *a = (asg_t *)malloc(sizeof(asg_t) * (size_t)(2 * s->ps.nq + 1));
    int na = ps_boundary(&s->ps, x, y, a);
    if (na < 0) { free(a); return; }
    int *f = (int *)malloc(sizeof(int) * (size_t)(2 * s->ps.nq + 1));
    int nf = ps_io_vars(&s->ps, f);
    pair_t *cands = (pair_t *)malloc(sizeof(pair_t) * (size_t)(s->ps.nv + 1));
    int nt, nc = pair_candidates(&s->ps, f, nf, cands, &nt);
    int p = pairs < nc ? pairs : nc;
    if (p > 62) p = 62;
    cx sum = C(0, 0);
    double sq = 0.0;
    asg_t *al[1] = {a};
    int an[1] = {na};
    for (int64_t i = 0; i < samples; i++) {
        srng r = srng_new(seed ^ ((uint64_t)i * golden));
        pathsum b = ps_clone(&s->ps);
        for (int j = 0; j < p; j++) ps_substitute(&b, cands[j].a, cands[j].b, (int)(srng_u64(&r) & 1ull));
        engine *E = engine_new(&b, f, nf);
        cx v;
        if (E->el.d <= exact_dim_limit) {
            rank_engine one; one.nbr = 1; one.pairs = 0; one.br = &E;
            eval_many(&one, 1, al, an, &v, 1);
        } else {
            uint8_t *vals = (uint8_t *)malloc((size_t)E->nf + 1);
            values_from_asg(E, a, na, vals);
            double se;
            engine_estimate(E, vals, (int64_t)1 << 14, srng_u64(&r), &v, &se);
            free(vals);
        }
        sum = cadd(sum, v);
        sq += v.re * v.re + v.im * v.im;
        engine_free(E);
        ps_free(&b);
    }
    const double n = (double)samples, scale = ldexp(1.0, p);
    const cx mean = C(sum.re / n, sum.im / n);
    double var = sq / n - (mean.re * mean.re + mean.im * mean.im);
    if (var < 0.0) var = 0.0;
    out[0] = mean.re * scale; out[1] = mean.im * scale; out[2] = scale * sqrt(var / n);
    free(cands); free(f); free(a);
}

/* Simulator::sample / sample_many (src/sim.rs:253-284): one seed per shot from Rng::new(seed);
 * per shot, qubit by qubit, p0 = min(prefix marginal with the new bit 0, p_prev) and the bit is 1
 * iff next_f64() * p_prev >= p0.  The prefix marginal of qubits 0..l is the sandwich engine with
 * those junctions fixed, built once per prefix length as the reference's prefix_engines
 * (src/sim.rs:232-249); all shots' marginals of one prefix length are evaluated in one call
 * (threads over shots and chunks, as the reference's parallel map over shots).
 * out: shots x words bitstrings. */
void pqo_sample_many(pqo_sim *s, const uint64_t *x, int64_t shots, uint64_t seed, uint64_t *out) {
    const int nq = s->ps.nq, nw = nq > 0 ? (nq + 63) / 64 : 1;
    if (!s->have_sw) {
        s->junction = (int *)malloc(sizeof(int) * (size_t)(nq + 1));
        s->jneg = (uint8_t *)malloc((size_t)nq + 1);
        s->sw = ps_sandwich(&s->c, s->junction, s->jneg);
        s->have_sw = 1;
    }
    const size_t ns = (size_t)(shots > 0 ? shots : 0);
    srng r = srng_new(seed);
    srng *rs = (srng *)malloc(sizeof(srng) * (ns + 1));
    for (size_t i = 0; i < ns; i++) rs[i] = srng_new(srng_u64(&r));
    double *p_prev = (double *)malloc(sizeof(double) * (ns + 1));
    for (size_t i = 0; i < ns; i++) p_prev[i] = 1.0;
    for (size_t i = 0; i < ns * (size_t)nw; i++) out[i] = 0;
    const int amax = 2 * nq + nq + 1;
    asg_t *abuf = (asg_t *)malloc(sizeof(asg_t) * (ns + 1) * (size_t)amax);
    asg_t **al = (asg_t **)malloc(sizeof(asg_t *) * (ns + 1));
    int *an = (int *)malloc(sizeof(int) * (ns + 1));
    size_t *slot = (size_t *)malloc(sizeof(size_t) * (ns + 1));
    cx *val = (cx *)malloc(sizeof(cx) * (ns + 1));
    int *f = (int *)malloc(sizeof(int) * (size_t)(amax + 1));
    for (int l = 0; l < nq; l++) {
        int nf = ps_io_vars(&s->sw, f);
        for (int q = 0; q <= l; q++) {
            int j = s->junction[q], seen = 0;
            for (int k = 0; k < nf; k++) if (f[k] == j) { seen = 1; break; }
            if (!seen) f[nf++] = j;
        }
        rank_engine eng = build_engine(&s->sw, f, nf, s->strategy, s->pairs);
        size_t nv = 0;
        for (size_t i = 0; i < ns; i++) {
            const uint64_t *y = out + i * (size_t)nw;  /* decided prefix, bit l still 0 */
            asg_t *a = abuf + i * (size_t)amax;
            int na = 0, ok = 1;
            for (int q = 0; q < nq && ok; q++) ok = asg_put(a, &na, q, bit_of(x, q));
            for (int q = 0; q < nq && ok; q++) ok = asg_put(a, &na, s->sw.outputs[q], bit_of(x, q) ^ s->sw.out_neg[q]);
            for (int q = 0; q <= l && ok; q++) ok = asg_put(a, &na, s->junction[q], bit_of(y, q) ^ s->jneg[q]);
            slot[i] = ok ? nv : (size_t)-1;
            if (ok) { al[nv] = a; an[nv] = na; nv++; }
        }
        if (nv) eval_many(&eng, (int)nv, al, an, val, default_threads(0));
        rank_free(&eng);
        for (size_t i = 0; i < ns; i++) {
            double p0 = slot[i] == (size_t)-1 ? 0.0 : (val[slot[i]].re > 0.0 ? val[slot[i]].re : 0.0);
            if (p0 > p_prev[i]) p0 = p_prev[i];
            if (srng_f64(&rs[i]) * p_prev[i] >= p0) {
                out[i * (size_t)nw + (size_t)(l >> 6)] |= 1ull << (l & 63);
                p_prev[i] = p_prev[i] - p0 > 0.0 ? p_prev[i] - p0 : 0.0;
            } else {
                p_prev[i] = p0;
            }
        }
    }
    free(f); free(val); free(slot); free(an); free(al); free(abuf); free(p_prev); free(rs);
}

/* ------------------------------------------------------------------ dense reference (src/dense.rs) */
static void diag1(cx *sv, uint64_t dim, int q, cx ph) {
    uint64_t m = 1ull << q;
    for (uint64_t i = 0; i < dim; i++) if (i & m) sv[i] = cmul(sv[i], ph);
}
static cx polar1(double th) { return C(cos(th), sin(th)); }
static void dense_apply(cx *sv, int n, gate g) {
    uint64_t dim = 1ull << n;
    cx I = C(0, 1);
    switch (g.op) {
        case G_H: {
            uint64_t m = 1ull << g.a;
            for (uint64_t i = 0; i < dim; i++) if (!(i & m)) {
                cx a = sv[i], b = sv[i | m];
                sv[i] = cscale(cadd(a, b), H_); sv[i | m] = cscale(csub(a, b), H_);
            }
        } break;
        case G_X: {
            uint64_t m = 1ull << g.a;
            for (uint64_t i = 0; i < dim; i++) if (!(i & m)) { cx t = sv[i]; sv[i] = sv[i | m]; sv[i | m] = t; }
        } break;
        case G_Y: {
            uint64_t m = 1ull << g.a;
            for (uint64_t i = 0; i < dim; i++) if (!(i & m)) {
                cx a = sv[i], b = sv[i | m];
                sv[i] = cmul(C(-0.0, -1.0), b); sv[i | m] = cmul(I, a);
            }
        } break;
        case G_Z: diag1(sv, dim, g.a, C(-1, 0)); break;
        case G_S: diag1(sv, dim, g.a, I); break;
        case G_SDG: diag1(sv, dim, g.a, C(-0.0, -1.0)); break;
        case G_T: diag1(sv, dim, g.a, polar1(M_PI / 4)); break;
        case G_TDG: diag1(sv, dim, g.a, polar1(-M_PI / 4)); break;
        case G_P: diag1(sv, dim, g.a, polar1(2.0 * M_PI * (double)g.ph / 4294967296.0)); break;
        case G_CZ: {
            uint64_t ma = 1ull << g.a, mb = 1ull << g.b;
            for (uint64_t i = 0; i < dim; i++) if ((i & ma) && (i & mb)) sv[i] = C(-sv[i].re, -sv[i].im);
        } break;
        case G_CX: {
            uint64_t mc = 1ull << g.a, mt = 1ull << g.b;
            for (uint64_t i = 0; i < dim; i++) if ((i & mc) && !(i & mt)) { cx t = sv[i]; sv[i] = sv[i | mt]; sv[i | mt] = t; }
        } break;
        case G_SWAP: {
            uint64_t ma = 1ull << g.a, mb = 1ull << g.b;
            for (uint64_t i = 0; i < dim; i++) if ((i & ma) && !(i & mb)) {
                uint64_t j = (i ^ ma) | mb; cx t = sv[i]; sv[i] = sv[j]; sv[j] = t;
            }
        } break;
        case G_GPHASE: {
            cx f = polar1(2.0 * M_PI * (double)g.ph / 4294967296.0);
            for (uint64_t i = 0; i < dim; i++) sv[i] = cmul(sv[i], f);
        } break;
    }
}
void pqo_dense_statevector(int nq, int ngates, const uint8_t *op, const int32_t *q0, const int32_t *q1,
                           const uint32_t *phase, const uint64_t *x, double *out) {
    if (!once_init) { init_root8(); once_init = 1; }
    uint64_t dim = 1ull << nq;
    cx *sv = (cx *)out;
    for (uint64_t i = 0; i < dim; i++) sv[i] = C(0, 0);
    uint64_t idx = 0;
    for (int q = 0; q < nq; q++) if (bit_of(x, q)) idx |= 1ull << q;
    sv[idx] = C(1, 0);
    for (int i = 0; i < ngates; i++) {
        gate g = {op[i], q0[i], q1[i], phase[i]};
        dense_apply(sv, nq, g);
    }
}

/* ------------------------------------------------------------------ equivalence (src/sim.rs:302-314) */
int pqo_equivalence(int nq1, int ng1, const uint8_t *op1, const int32_t *a1, const int32_t *b1, const uint32_t *p1,
                    int nq2, int ng2, const uint8_t *op2, const int32_t *a2, const int32_t *b2, const uint32_t *p2,
                    double tol, double out[2]) {
    if (!once_init) { init_root8(); once_init = 1; }
    int n = nq1 > nq2 ? nq1 : nq2;
    circuit m; m.nq = n; m.ng = ng1 + ng2; m.g = (gate *)calloc((size_t)(m.ng ? m.ng : 1), sizeof(gate));
    for (int i = 0; i < ng1; i++) { gate g = {op1[i], a1[i], b1[i], p1[i]}; m.g[i] = g; }
    for (int i = 0; i < ng2; i++) { gate g = {op2[ng2 - 1 - i], a2[ng2 - 1 - i], b2[ng2 - 1 - i], p2[ng2 - 1 - i]}; m.g[ng1 + i] = gate_inverse(g); }
    pathsum ps = ps_from_circuit(&m);
    ps_trace_closure(&ps);
    rank_engine r = build_engine(&ps, NULL, 0, 0, 0);
    asg_t dummy[1];
    asg_t *al[1] = {dummy};
    int an[1] = {0};
    cx tr;
    eval_many(&r, 1, al, an, &tr, 1);
    cx ov = cscale(tr, 1.0 / pow(2.0, (double)n));
    /* sim.rs:311 divides by 2^n; dividing by an exact power of two equals multiplying by its inverse */
    out[0] = ov.re; out[1] = ov.im;
    double norm = hypot(ov.re, ov.im);
    rank_free(&r); ps_free(&ps); free(m.g);
    return norm >= 1.0 - tol;
}

/* ------------------------------------------------------------------ canonical dumps */
/*
 * engine_dump layout (u64 words), identical to the product's debug dump:
 *   header[8]: m, g, nodd, neven, t, d, (int64)sigma, nf
 *   basis: pairs_a[g], pairs_b[g], odd[nodd], even[neven]       each nw(m) words
 *   diag:  wa nw(g), wb nw(g), o1 nw(nodd), o3 nw(nodd), we nw(neven)
 *   kernel_u[d]: a nw(g), b nw(g), o nw(nodd)      (the e part is zero by construction)
 *   kernel[d]:   nw(t)
 *   mcols[t]:    a, b, o, e
 *   ucols[nf]:   a, b, o, e
 *   pivots[rank]: col, row nw(neven)
 *   consistency[neven-rank]: nw(neven)
 */
typedef struct { uint64_t *out; int64_t cap, n; } sink;
static void put1(sink *k, uint64_t x) { if (k->out && k->n < k->cap) k->out[k->n] = x; k->n++; }
static void putbv(sink *k, const bv *v) { for (int i = 0; i < v->nw; i++) put1(k, v->w[i]); }
static void putuv(sink *k, const uvec *u, int with_e) { putbv(k, &u->a); putbv(k, &u->b); putbv(k, &u->o); if (with_e) putbv(k, &u->e); }
int64_t pqo_engine_dump(const pqo_sim *s, int br, uint64_t *out, int64_t cap) {
    if (br < 0 || br >= s->eng.nbr) return -1;
    const engine *E = s->eng.br[br];
    const structure *st = &E->st;
    sink k = {out, cap, 0};
    put1(&k, (uint64_t)E->m); put1(&k, (uint64_t)st->g); put1(&k, (uint64_t)st->nodd); put1(&k, (uint64_t)st->neven);
    put1(&k, (uint64_t)E->t); put1(&k, (uint64_t)E->el.d); put1(&k, (uint64_t)(int64_t)E->dg.sigma); put1(&k, (uint64_t)E->nf);
    for (int i = 0; i < st->g; i++) putbv(&k, &st->pa[i]);
    for (int i = 0; i < st->g; i++) putbv(&k, &st->pb[i]);
    for (int i = 0; i < st->nodd; i++) putbv(&k, &st->odd[i]);
    for (int i = 0; i < st->neven; i++) putbv(&k, &st->even[i]);
    putbv(&k, &E->dg.wa); putbv(&k, &E->dg.wb); putbv(&k, &E->dg.o1); putbv(&k, &E->dg.o3); putbv(&k, &E->dg.we);
    for (int j = 0; j < E->el.d; j++) putuv(&k, &E->el.kernel_u[j], 0);
    for (int j = 0; j < E->el.d; j++) putbv(&k, &E->el.kernel[j]);
    for (int q = 0; q < E->t; q++) putuv(&k, &E->mcols[q], 1);
    for (int f = 0; f < E->nf; f++) putuv(&k, &E->ucols[f], 1);
    for (int i = 0; i < E->el.rank; i++) { put1(&k, (uint64_t)E->el.piv_col[i]); putbv(&k, &E->el.piv_row[i]); }
    for (int i = 0; i < E->el.ncons; i++) putbv(&k, &E->el.cons[i]);
    return k.n;
}
int pqo_branch_phases(pqo_sim *s, int br, const uint64_t *x, const uint64_t *y, uint8_t *out) {
    if (br < 0 || br >= s->eng.nbr) return -1;
    const engine *E = s->eng.br[br];
    if (E->el.d > 24) return -1;
    asg_t *a = (asg_t *)malloc(sizeof(asg_t) * (size_t)(2 * s->ps.nq + 1));
    int na = ps_boundary(&s->ps, x, y, a);
    if (na < 0) { free(a); return -1; }
    uint8_t *vals = (uint8_t *)malloc((size_t)E->nf + 1);
    values_from_asg(E, a, na, vals);
    prep_t p; prep_init(&p, E);
    int ok = engine_prepare(E, vals, &p);
    int d = E->el.d;
    if (ok) {
        /* the kernel points in Gray order (engine.rs:696-722 walks them the same way): point
         * s = i ^ (i >> 1) differs from the previous one in kernel column ctz(i) */
        uvec u; uv_init(&u, &E->st);
        uv_copy(&u, &p.u);
        out[0] = (uint8_t)phase8(&E->dg, &u);
        for (uint64_t i = 1; i < (1ull << d); i++) {
            uv_xor(&u, &E->el.kernel_u[__builtin_ctzll(i)]);
            out[i ^ (i >> 1)] = (uint8_t)phase8(&E->dg, &u);
        }
        uv_free(&u);
    }
    prep_free(&p); free(vals); free(a);
    return ok ? d : -1;
}

/* Branch dimension d of branch engine `br` (-1 out of range). */
int pqo_branch_dim(const pqo_sim *s, int br) {
    if (br < 0 || br >= s->eng.nbr) return -1;
    return s->eng.br[br]->el.d;
}

/*
 * Integers of Engine::prepare (engine.rs:569-610, Elim::solve_into :188-201) for every
 * (boundary, branch engine) job, boundary-major: PQO_PREP_WORDS u64 words per job,
 *   [0] 1 if the job vanishes (contradictory boundary, sim.rs:172-174; zero engine, :570;
 *       inconsistent radical system, :595-597), else 0 -- the other words are 0 then
 *   [1] the constant phase (u32 ring units: global + fixed thetas + Z4 fixed terms, :575-588)
 *   [2] k0 = phase8 of the start shift u (normal_form.rs:479-493)
 *   [3] y0: bit i = the particular solution s0 at pivot column i (pivots in Elim order)
 *   [4..11] Lp_j = (phase8(u ^ kernel_u[j]) - k0) / 2 mod 4 as bytes, j < min(d, 64);
 *       an odd increment is recorded as 0xFF (the closed form has only even ones)
 */
void pqo_prepare_info(pqo_sim *s, int n, const uint64_t *xs, const uint64_t *ys, uint64_t *out) {
    int nw = (s->ps.nq + 63) / 64;
    if (nw == 0) nw = 1;
    const int nb = s->eng.nbr;
    asg_t *a = (asg_t *)malloc(sizeof(asg_t) * (size_t)(2 * s->ps.nq + 1));
    for (int i = 0; i < n; i++) {
        int na = ps_boundary(&s->ps, xs + (size_t)i * nw, ys + (size_t)i * nw, a);
        for (int b = 0; b < nb; b++) {
            uint64_t *rec = out + ((size_t)i * nb + b) * PQO_PREP_WORDS;
            memset(rec, 0, sizeof(uint64_t) * PQO_PREP_WORDS);
            const engine *E = s->eng.br[b];
            int ok = 0;
            prep_t p; prep_init(&p, E);
            if (na >= 0) {
                uint8_t *vals = (uint8_t *)malloc((size_t)E->nf + 1);
                values_from_asg(E, a, na, vals);
                ok = engine_prepare(E, vals, &p);
                free(vals);
            }
            if (!ok) {
                rec[0] = 1;
                prep_free(&p);
                continue;
            }
            const unsigned k0 = phase8(&E->dg, &p.u);
            rec[1] = p.phase;
            rec[2] = k0;
            for (int r = 0; r < E->el.rank && r < 64; r++)
                if (bv_get(&p.s0, E->el.piv_col[r])) rec[3] |= 1ull << r;
            uvec u; uv_init(&u, &E->st);
            for (int j = 0; j < E->el.d && j < 64; j++) {
                uv_copy(&u, &p.u);
                uv_xor(&u, &E->el.kernel_u[j]);
                const unsigned L = (phase8(&E->dg, &u) - k0) & 7u;
                const uint64_t byte = (L & 1u) ? 0xFFull : (uint64_t)(L >> 1);
                rec[4 + (j >> 3)] |= byte << (8 * (j & 7));
            }
            uv_free(&u);
            prep_free(&p);
        }
    }
    free(a);
}

/* ------------------------------------------------------------------ raw-form checks (normal_form.rs tests) */
static void raw_form(int m, const uint8_t *bmat, bm *b) {
    bm_init(b, m, m);
    for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) if (bmat[i * m + j]) bv_set(&b->r[i], j, 1);
}
static int gram_entry(const bm *b, const bv *parity, const bv *p, const bv *q) { /* normal_form.rs:545-552 */
    int acc = 0;
    FOR_ONES(j, p) { acc ^= bv_dot(&b->r[j], q); acc ^= bv_get(parity, j) & bv_get(q, j); }
    return acc;
}
int pqo_check_structure(int m, const uint8_t *bmat, const uint8_t *parity_in, int rule, int32_t out_sizes[3]) {
    bm b; raw_form(m, bmat, &b);
    bv parity; bv_init(&parity, m);
    for (int i = 0; i < m; i++) bv_set(&parity, i, parity_in[i] & 1);
    structure s = structure_new(&b, &parity, rule);
    out_sizes[0] = s.g; out_sizes[1] = s.nodd; out_sizes[2] = s.neven;
    int bad = 0;
    if (2 * s.g + s.nodd + s.neven != m) bad = 1;
    int n = 2 * s.g + s.nodd + s.neven;
    bv **all = (bv **)malloc(sizeof(bv *) * (size_t)(n + 1));
    int *tp = (int *)malloc(sizeof(int) * (size_t)(n + 1)), *ix = (int *)malloc(sizeof(int) * (size_t)(n + 1)), c = 0;
    for (int j = 0; j < s.g; j++) { all[c] = &s.pa[j]; tp[c] = 0; ix[c++] = j; }
    for (int j = 0; j < s.g; j++) { all[c] = &s.pb[j]; tp[c] = 1; ix[c++] = j; }
    for (int j = 0; j < s.nodd; j++) { all[c] = &s.odd[j]; tp[c] = 2; ix[c++] = j; }
    for (int j = 0; j < s.neven; j++) { all[c] = &s.even[j]; tp[c] = 3; ix[c++] = j; }
    for (int p = 0; p < n && !bad; p++)
        for (int q = 0; q < n && !bad; q++) {
            int expect = ((tp[p] == 0 && tp[q] == 1) || (tp[p] == 1 && tp[q] == 0) || (tp[p] == 2 && tp[q] == 2)) ? ix[p] == ix[q] : 0;
            if (gram_entry(&b, &parity, all[p], all[q]) != expect) bad = 2;
        }
    if (!bad) {
        bv *rows = (bv *)malloc(sizeof(bv) * (size_t)(n + 1));
        for (int i = 0; i < n; i++) rows[i] = bv_clone(all[i]);
        int rank = 0;
        for (int col = 0; col < m; col++) {
            int r = -1;
            for (int i = rank; i < n; i++) if (bv_get(&rows[i], col)) { r = i; break; }
            if (r < 0) continue;
            bv t = rows[rank]; rows[rank] = rows[r]; rows[r] = t;
            for (int r2 = 0; r2 < n; r2++) if (r2 != rank && bv_get(&rows[r2], col)) bv_xor(&rows[r2], &rows[rank]);
            rank++;
        }
        if (rank != m) bad = 3;
        for (int i = 0; i < n; i++) bv_free(&rows[i]);
        free(rows);
    }
    free(all); free(tp); free(ix);
    structure_free(&s); bv_free(&parity); bm_free(&b);
    return bad;
}
void pqo_gauss_sum(int m, const uint8_t *bmat, const uint8_t *v, const uint8_t *shift_in, int rule,
                   double out_closed[2], double out_brute[2]) {
    if (!once_init) { init_root8(); once_init = 1; }
    bm b; raw_form(m, bmat, &b);
    bv parity; bv_init(&parity, m);
    bv shift; bv_init(&shift, m);
    for (int i = 0; i < m; i++) { bv_set(&parity, i, v[i] & 1); bv_set(&shift, i, shift_in[i] & 1); }
    structure s = structure_new(&b, &parity, rule);
    diag_t d = structure_diagonal(&s, &b, v);
    uvec u; structure_transform(&s, &shift, &u);
    cx got = C(0, 0);
    if (bv_eq(&u.e, &d.we)) got = cscale(ROOT8[phase8(&d, &u)], pow(2.0, log2_magnitude(&s)));
    out_closed[0] = got.re; out_closed[1] = got.im;
    /* normal_form.rs:522-543 brute force */
    cx tot = C(0, 0);
    for (uint32_t x = 0; x < (1u << m); x++) {
        unsigned q = 0;
        for (int j = 0; j < m; j++) {
            if (!((x >> j) & 1)) continue;
            q += v[j];
            if (bv_get(&shift, j)) q += 2;
            for (int k = j + 1; k < m; k++) if (((x >> k) & 1) && bv_get(&b.r[j], k)) q += 2;
        }
        tot = cadd(tot, ROOT8[2 * (q & 3)]);
    }
    out_brute[0] = tot.re; out_brute[1] = tot.im;
    uv_free(&u); diag_free(&d); structure_free(&s); bv_free(&parity); bv_free(&shift); bm_free(&b);
}
