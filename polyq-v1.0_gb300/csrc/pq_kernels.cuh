// pq_kernels.cuh -- sm_103a kernels of the amplitude path.
//
//   prepare_kernel   one warp per (branch engine, boundary) job: boundary values, fixed
//                    constants, boundary shift u0 = xor of resident boundary columns, radical
//                    consistency + particular solution (pivot bits y0), start shift, Z8 index
//                    k0 and the Z4 linear coefficients Lp_j        (src/engine.rs:569-610)
//   enum_kernel      persistent: each warp pulls work items (a job's contiguous range of
//                    units of 1-8 chunks) from an atomic counter; lane l walks units l, l+32,
//                    ... in Gray order in a rotating frame over the sign-folded weight table:
//                    per step one table load and index xor shared by the unit's chunks, and a
//                    quarter-turn-and-add of each chunk's exact-grid hi and FP32 lo sums; FP64
//                    scaling of each chunk and an FP64 warp-shuffle reduce
//                    (src/engine.rs:669-722, normal_form.rs:479-493)
//   job_reduce       FP64 sum of a job's item partials in item order, times the Z8 root of k0,
//                    e^{i phase} and 2^{(mag2 - h)/2}                  (src/engine.rs:557-565)
//   out_reduce       FP64 sum over the 2^p branch engines of each boundary (src/rank.rs:184-190)
#pragma once
#include <cuda_runtime.h>

#include "pq_core.cuh"

namespace pq {

#define PQ_FULL 0xffffffffu

__constant__ double c_root8[16] = {1.0, 0.0, 0.70710678118654752440, 0.70710678118654752440, 0.0, 1.0,
                                   -0.70710678118654752440, 0.70710678118654752440, -1.0, 0.0,
                                   -0.70710678118654752440, -0.70710678118654752440, 0.0, -1.0,
                                   0.70710678118654752440, -0.70710678118654752440};

struct KArgs {
    const EngineDev *engines;
    const IoMapDev *maps;
    JobDev *jobs;
    int njobs;
    const int *perm;            // job id of the k-th job in item order
    const int *kinv;            // position of job j in item order
    const long long *istart;    // njobs + 1 prefix sums of item counts (item order)
    const int *jdl;             // per job: Gray steps per chunk (log2)
    const unsigned *jcpi;       // per job: chunks per item
    const unsigned long long *jnch;  // per job: chunks
    long long nitems;
    double2 *partials;
    unsigned long long *counter;  // nslices counters (item slices, enum_kernel)
    int nslices;                  // 0 or 1: one counter over all items
    double2 *job_vals;
    double *job_err;
    const int *out_jobs;        // nout + 1: jobs of output o are [out_jobs[o], out_jobs[o+1])
    int nout;
    double *out;                // 2 * nout
    double *err;                // nout or null
    int out_prob;               // write |amp|^2 instead of amp
    const uint64_t *xs;
    const uint64_t *ys;
    int nw;
    int smem_words;             // per-warp words of the prepare kernel
    uint8_t *dbg;               // per-branch Z8 indices (debug mode)
    int *errflag;
    uint8_t *lpx;               // optional: Lp of every coordinate, lpx_stride bytes per job (any d)
    int lpx_stride;
    int use_ctab;               // chunk sums from the engines' chunk-sum tables where they apply
    int fp64_mode;              // the enumeration ran with FP64 weights (error bound of that path)
    const long long *ioff;      // optional, per job: index of its first work item (a launch that
                                // evaluates a range of a job's items; null: all of them)
};

__device__ __forceinline__ int warp_sum_i(int v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(PQ_FULL, v, o);
    return v;
}
__device__ __forceinline__ unsigned warp_sum_u(unsigned v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(PQ_FULL, v, o);
    return v;
}

// ------------------------------------------------------------------------------ prepare
// One (branch engine, boundary) job on one warp: boundary bits x, y -> fixed values, fixed
// constants, boundary shift, radical system, start shift, k0 and Lp (src/engine.rs:569-610).
// u: this warp's scratch of at least W + ceil(nf / 64) words.
__device__ __forceinline__ void prepare_job(const KArgs &a, int jid, const uint64_t *x, const uint64_t *y,
                                            uint64_t *u, int lane) {
    JobDev *J = &a.jobs[jid];
    const EngineDev &E = a.engines[J->engine];
    const IoMapDev &M = a.maps[J->iomap];
    uint64_t *vals = u + E.W;
    // fixed-variable values from the boundary bits
    for (int base = 0; base < E.nf; base += 64) {
        int i0 = base + lane, i1 = base + 32 + lane;
        int b0 = i0 < E.nf ? src_bit(M.src[i0], x, y) : 0;
        int b1 = i1 < E.nf ? src_bit(M.src[i1], x, y) : 0;
        unsigned lo = __ballot_sync(PQ_FULL, b0), hi = __ballot_sync(PQ_FULL, b1);
        if (lane == 0) vals[base >> 6] = (uint64_t)lo | ((uint64_t)hi << 32);
    }
    __syncwarp();
    int bad = 0;
    for (int c = lane; c < M.ncf; c += 32) bad |= bit_at(vals, M.cf_pos[c]) != src_bit(M.cf_src[c], x, y);
    bad = __any_sync(PQ_FULL, bad) || E.zero;
    // constants from fixed-fixed terms (engine.rs:575-588)
    uint32_t z4 = 0, th = 0;
    fixed_constants_partial(E, vals, lane, 32, z4, th);
    z4 = warp_sum_u(z4);
    th = warp_sum_u(th);
    // u0 = xor of boundary columns (engine.rs:589-592)
    boundary_shift_partial(E, vals, u, lane, 32);
    __syncwarp();
    // radical system K s = kappa (engine.rs:593-597, :188-201)
    int badc = 0;
    for (int r = lane; r < E.ncons; r += 32) badc |= kappa_dot(E, E.cons + (size_t)r * E.we, u);
    bad = bad || __any_sync(PQ_FULL, badc);
    uint64_t y0 = 0;
    for (int base = 0; base < E.rank; base += 32) {
        int i = base + lane;
        int bit = i < E.rank ? kappa_dot(E, E.pivrow + (size_t)i * E.we, u) : 0;
        y0 |= (uint64_t)__ballot_sync(PQ_FULL, bit) << base;
    }
    // start shift u = u0 ^ sum of the pivot columns (engine.rs:598-607)
    apply_pivots_partial(E, y0, u, lane, 32);
    __syncwarp();
    int n1 = 0, cnt = 0;
    phase8_partial(E, u, nullptr, lane, 32, n1, cnt);
    n1 = warp_sum_i(n1);
    cnt = warp_sum_i(cnt);
    const uint32_t k0 = phase8_finish(E, n1, cnt);
    int lerr = 0;
    for (int j = lane; j < E.d; j += 32) {
        int a1 = 0, c1 = 0;
        phase8_partial(E, u, E.ku + (size_t)j * E.abo, 0, 1, a1, c1);
        uint32_t L = (phase8_finish(E, a1, c1) - k0) & 7u;
        lerr |= (int)(L & 1u);
        if (j < 64) J->Lp[j] = (uint8_t)(L >> 1);
        if (a.lpx) a.lpx[(size_t)jid * a.lpx_stride + j] = (uint8_t)(L >> 1);
    }
    lerr = __any_sync(PQ_FULL, lerr);
    if (lane == 0) {
        J->vanish = bad ? 1 : 0;
        J->phase = E.global + th + ((z4 & 3u) << 30);
        J->k0 = k0;
        J->y0 = y0;
        J->err = (uint32_t)lerr;
        if (lerr) atomicOr(a.errflag, 1);
    }
    __syncwarp();
}

__global__ void __launch_bounds__(128) prepare_kernel(KArgs a) {
    extern __shared__ uint64_t psm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    uint64_t *u = psm + (size_t)wib * a.smem_words;
    for (int jid = blockIdx.x * wpb + wib; jid < a.njobs; jid += gridDim.x * wpb) {
        const int req = a.jobs[jid].req;
        prepare_job(a, jid, a.xs + (size_t)req * a.nw, a.ys + (size_t)req * a.nw, u, lane);
    }
}

// ------------------------------------------------------------------------------ enumerate

// Parity of the quadratic part sum_{i<j} G_ij x_i x_j restricted to the bits of x (G symmetric,
// zero diagonal): every pair is counted twice by sum_{j in x} popc(G_j & x).
__device__ __forceinline__ uint32_t quad_parity(const uint64_t *G, uint64_t x) {
    uint32_t t = 0;
    for (uint64_t r = x; r; r &= r - 1) t += (uint32_t)popc64(G[ctz64(r)] & x);
    return (t >> 1) & 1u;
}

// a + b = s + e exactly (two-sum, no ordering of |a|, |b| assumed).
__device__ __forceinline__ float two_sum_f(float a, float b, float &e) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

// (ur, ui) += P S in FP32 pairs (value = hi + lo): P = (P.x + P.z) + i (P.y + P.w), S = (hx + lx)
// + i (hy + ly) with hx, hy exact.  The products of the hi parts are exact (FMA residuals), the
// accumulation of their hi words is exact (two-sums); cross terms with a lo part go into the lo
// word in FP32 (lo x lo dropped).
__device__ __forceinline__ void ff_cmul_acc(const float4 &P, float hx, float hy, float lx, float ly, float &urh,
                                            float &url, float &uih, float &uil) {
    float e1, e2;
    {
        const float a = __fmul_rn(P.x, hx), ae = __fmaf_rn(P.x, hx, -a);
        const float b = __fmul_rn(P.y, hy), be = __fmaf_rn(P.y, hy, -b);
        urh = two_sum_f(urh, a, e1);
        urh = two_sum_f(urh, -b, e2);
        float t = __fadd_rn(__fsub_rn(ae, be), __fadd_rn(e1, e2));
        t = __fmaf_rn(P.x, lx, t);
        t = __fmaf_rn(P.z, hx, t);
        t = __fmaf_rn(-P.y, ly, t);
        t = __fmaf_rn(-P.w, hy, t);
        url = __fadd_rn(url, t);
    }
    {
        const float a = __fmul_rn(P.x, hy), ae = __fmaf_rn(P.x, hy, -a);
        const float b = __fmul_rn(P.y, hx), be = __fmaf_rn(P.y, hx, -b);
        uih = two_sum_f(uih, a, e1);
        uih = two_sum_f(uih, b, e2);
        float t = __fadd_rn(__fadd_rn(ae, be), __fadd_rn(e1, e2));
        t = __fmaf_rn(P.x, ly, t);
        t = __fmaf_rn(P.z, hy, t);
        t = __fmaf_rn(P.y, lx, t);
        t = __fmaf_rn(P.w, hx, t);
        uil = __fadd_rn(uil, t);
    }
}

// Gray walk over the 2^dl inner coordinates of K chunks (dl >= 3) in a rotating frame.
//
// The weight table W holds w(y, s_lo) * (-1)^{q(s_lo)}, q = sum_{i<j<DI} G_ij s_i s_j: the
// quadratic phase among the low coordinates is folded into the table.  What remains of the Z4
// index over the walked coordinates is linear: flipping coordinate j up adds L'_j = Lp_j + 2 c_j
// (c_j = parity(G_j & s_hi), constant inside a chunk), flipping it down subtracts L'_j.
//
// With m_k the (folded) index of the k-th branch, the walk keeps A_k = i^{-m_k} sum_{l<=k}
// i^{m_l} w_l, so that A_{k+1} = i^{-Delta_k} A_k + w_{k+1}: each step is a quarter-turn of the
// accumulator by a per-chunk constant plus the table entry, with no per-branch phase arithmetic.
// The parity of Delta on coordinate j is that of Lp_j, the same for every boundary of an engine,
// so it is a compile-time case (PAR, bit j for j < 3): an even step is A <- rho A + w, an odd one
// (re, im) <- rho (im, -re) + w, with rho = +-1 from bit 1 of L'_j (negated on an odd down-flip).
// Either is two FFMA per complex number, exact on the hi parts (multiples of the table grid).
// The K chunks of a unit differ only in coordinates that touch no pivot, so they read the same
// table entry at every step (one load feeds K accumulators); they differ in their c_j.
// Unrolled by 8: coordinates 0 and 1 flip at fixed positions with fixed directions (0+, 1+, 0-,
// 0+, 1-, 0-), coordinate 2 once per group with the group's direction, and the group boundary
// flips coordinate 3 + ctz(g+1) (its parity is warp-uniform: a uniform branch).
//   sidx   (pivot bits << DI) | low DI coordinates: the table index; the table is aligned to
//          its size, so the walk keeps the entry's address and XORs byte strides into it
//   Pc[k]  bit j = c_j of chunk k for the walked coordinates
//   T_j    ((1 << j) | (R_j << DI)) * 16: the change of the entry's address when coordinate j flips
// On return acc[k] = (hi.re, hi.im, lo.re, lo.im) of chunk k's A at the last branch, whose
// folded index is m[k] + L'_{dl-1} (the walk ends on the unit vector of coordinate dl-1).
// Accumulators and table entries travel as pairs of FP32 in one 64-bit register, (re, im): an
// even quarter-turn-and-add is then one fma.rn.f32x2 per pair (same rounding as two fmaf); an
// odd one swaps re and im and is done on the halves.
__device__ __forceinline__ uint64_t pk2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void up2(uint64_t p, float &a, float &b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(p)); }
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// even: A <- rho A + w (rho2 = (rho, rho)); odd: (re, im) <- rho (im, -re) + w
__device__ __forceinline__ void qturn_even(uint64_t &H, uint64_t &L, uint64_t rho2, const ulonglong2 &w) {
    H = ffma2(rho2, H, w.x);
    L = ffma2(rho2, L, w.y);
}
__device__ __forceinline__ void qturn_odd(uint64_t &H, uint64_t &L, float rho, const ulonglong2 &w) {
    float hr, hi, lr, li, wx, wy, wz, ww;
    up2(H, hr, hi);
    up2(L, lr, li);
    up2(w.x, wx, wy);
    up2(w.y, wz, ww);
    H = pk2(fmaf(rho, hi, wx), fmaf(-rho, hr, wy));
    L = pk2(fmaf(rho, li, wz), fmaf(-rho, lr, ww));
}


template <int MODE, int K, int PAR>
__device__ __forceinline__ void gray_chunk_rot(const float4 *__restrict__ W4, uint32_t sidx, const uint32_t (&Pc)[K],
                                               const uint32_t *Tg, const uint8_t *Lp, int dl, float (&acc)[K][4],
                                               uint8_t *dbg, const uint64_t (&sbase)[K], uint32_t k0,
                                               uint32_t (&m)[K], const uint64_t *G, uint32_t lomask) {
    constexpr int O0 = PAR & 1, O1 = (PAR >> 1) & 1, O2 = (PAR >> 2) & 1;
    // the table is aligned to its size: an entry's address is the base OR its byte offset, and
    // a flip XORs the coordinate's byte stride into it
    uint64_t wad = reinterpret_cast<uint64_t>(W4) | ((uint64_t)sidx << 4);
    const uint32_t T0 = Tg[0], T1 = Tg[1], T2 = Tg[2];
    const uint32_t Lp0 = Lp[0], Lp1 = Lp[1], Lp2 = Lp[2];
    uint64_t H[K], L[K];
    const ulonglong2 w0 = __ldg(reinterpret_cast<const ulonglong2 *>(wad));
#pragma unroll
    for (int k = 0; k < K; k++) {
        H[k] = w0.x;
        L[k] = w0.y;
    }
    const uint32_t inner = (1u << dl) - 1u;
    const uint32_t ngroups = 1u << (dl - 3);
    // the next step's entry is loaded one step ahead (the last prefetch of the walk reads an
    // entry of the table that is not used)
    ulonglong2 wn = __ldg(reinterpret_cast<const ulonglong2 *>(wad ^ (uint64_t)T0));
    // MODE 2 records the true Z8 index: folded index + 2 q(s_lo) (the sign held by the table)
#define PQ_REC(k)                                                                                        \
    if (MODE == 2)                                                                                       \
        dbg[sbase[k] | (((uint32_t)wad >> 4) & inner)] =                                               \
            (uint8_t)((k0 + 2u * (m[k] + 2u * quad_parity(G, ((uint32_t)wad >> 4) & lomask))) & 7u);
    // flip by T, then A <- quarter-turn(A) + w for every chunk of the unit, w the entry loaded
    // one step earlier; the entry of the following step (stride TN) is loaded here.  RHO2: the
    // (rho, rho) pair of an even step; RHO: the signed rho of an odd step.
#define PQ_Q(ODD, T, TN, RHO2, RHO, DM)                                            \
    {                                                                              \
        const ulonglong2 w = wn;                                                   \
        wad ^= (uint64_t)(T);                                                      \
        wn = __ldg(reinterpret_cast<const ulonglong2 *>(wad ^ (uint64_t)(TN)));    \
        _Pragma("unroll") for (int k = 0; k < K; k++) {                            \
            if (ODD) qturn_odd(H[k], L[k], (RHO), w);                              \
            else qturn_even(H[k], L[k], (RHO2), w);                                \
            if (MODE == 2) m[k] += (DM);                                           \
            PQ_REC(k)                                                              \
        }                                                                          \
    }
    if (MODE == 2) {
#pragma unroll
        for (int k = 0; k < K; k++) PQ_REC(k)
    }
#define PQ_L0 (Lp0 + ((Pc[k] & 1u) << 1))
#define PQ_L1 (Lp1 + (Pc[k] & 2u))
#define PQ_L2 (Lp2 + ((Pc[k] >> 1) & 2u))
    // rho of coordinates 0..2 per chunk, formed at each use from c_j (bit j of Pc[k]) rather than
    // held in registers: +-1.0f with sign bit (Lp_j >> 1) ^ c_j, negated on an odd down-flip
    const uint32_t u0 = (((Lp0 >> 1) & 1u) << 31) | 0x3F800000u, u0n = u0 ^ (O0 ? 0x80000000u : 0u);
    const uint32_t u1 = (((Lp1 >> 1) & 1u) << 31) | 0x3F800000u, u1n = u1 ^ (O1 ? 0x80000000u : 0u);
#define PQ_R0 __uint_as_float(((Pc[k] & 1u) << 31) ^ u0)
#define PQ_R0N __uint_as_float(((Pc[k] & 1u) << 31) ^ u0n)
#define PQ_R1 __uint_as_float((((Pc[k] >> 1) & 1u) << 31) ^ u1)
#define PQ_R1N __uint_as_float((((Pc[k] >> 1) & 1u) << 31) ^ u1n)
    for (uint32_t g = 0;; ++g) {
        PQ_Q(O0, T0, T1, pk2(PQ_R0, PQ_R0), PQ_R0, PQ_L0);
        PQ_Q(O1, T1, T0, pk2(PQ_R1, PQ_R1), PQ_R1, PQ_L1);
        PQ_Q(O0, T0, T2, pk2(PQ_R0, PQ_R0), PQ_R0N, 0u - PQ_L0);
        {
            const bool up = ((uint32_t)wad ^ T2) & 64u;  // coordinate 2's bit after the flip
            const uint32_t u2 = ((((Lp2 >> 1) ^ (O2 && !up ? 1u : 0u)) & 1u) << 31) | 0x3F800000u;
#define PQ_R2 __uint_as_float((((Pc[k] >> 2) & 1u) << 31) ^ u2)
            PQ_Q(O2, T2, T0, pk2(PQ_R2, PQ_R2), PQ_R2, up ? PQ_L2 : 0u - PQ_L2);
#undef PQ_R2
        }
        PQ_Q(O0, T0, T1, pk2(PQ_R0, PQ_R0), PQ_R0, PQ_L0);
        PQ_Q(O1, T1, T0, pk2(PQ_R1, PQ_R1), PQ_R1N, 0u - PQ_L1);
        const bool last = g + 1 == ngroups;
        const int j = last ? 0 : 3 + ctz32(g + 1);
        const uint32_t Tj = Tg[j];
        PQ_Q(O0, T0, Tj, pk2(PQ_R0, PQ_R0), PQ_R0N, 0u - PQ_L0);
        if (last) break;
        const uint32_t down = ((uint32_t)wad >> (j + 4)) & 1u;  // bit j is set before a down flip
        const uint32_t Lpj = Lp[j];
        // rho = -1 iff bit 1 of L'_j = Lp_j + 2 c_j is set, negated on an odd down-flip: its sign
        // bit is c_j xor a warp-uniform bit, placed at bit 31 of +1.0f
        const uint32_t u31 = ((((Lpj >> 1) ^ (down & Lpj)) & 1u) << 31) | 0x3F800000u;
#define PQ_RHO_J __uint_as_float(((Pc[k] >> j) << 31) ^ u31)
#define PQ_DM_J (down ? 0u - (Lpj + (((Pc[k] >> j) & 1u) << 1)) : Lpj + (((Pc[k] >> j) & 1u) << 1))
        if (Lpj & 1u) {
            PQ_Q(1, Tj, T0, 0ull, PQ_RHO_J, PQ_DM_J);
        } else {
            PQ_Q(0, Tj, T0, pk2(PQ_RHO_J, PQ_RHO_J), 0.f, PQ_DM_J);
        }
#undef PQ_RHO_J
#undef PQ_DM_J
    }
#undef PQ_R0
#undef PQ_R0N
#undef PQ_R1
#undef PQ_R1N
#undef PQ_L0
#undef PQ_L1
#undef PQ_L2
#undef PQ_Q
#undef PQ_REC
#pragma unroll
    for (int k = 0; k < K; k++) {
        up2(H[k], acc[k][0], acc[k][1]);
        up2(L[k], acc[k][2], acc[k][3]);
    }
}

// Dispatch on the parities of Lp_0..2 (an engine constant, warp-uniform).
template <int MODE, int K>
__device__ __forceinline__ void gray_chunk_rot_any(const float4 *__restrict__ W, uint32_t sidx, const uint32_t (&Pc)[K],
                                                   const uint32_t *Tg, const uint8_t *Lp, int dl, float (&acc)[K][4],
                                                   uint8_t *dbg, const uint64_t (&sbase)[K], uint32_t k0,
                                                   uint32_t (&m)[K], const uint64_t *G, uint32_t lomask) {
    const int par = (Lp[0] & 1) | ((Lp[1] & 1) << 1) | ((Lp[2] & 1) << 2);
    switch (par) {
#define PQ_CASE(P) \
    case P: gray_chunk_rot<MODE, K, P>(W, sidx, Pc, Tg, Lp, dl, acc, dbg, sbase, k0, m, G, lomask); break;
        PQ_CASE(0) PQ_CASE(1) PQ_CASE(2) PQ_CASE(3) PQ_CASE(4) PQ_CASE(5) PQ_CASE(6) PQ_CASE(7)
#undef PQ_CASE
    }
}

// ------------------------------------------------------------------------------ bucket walk
// Walks of up to 2^kGroupTableMaxDl steps keep their group tables (two words per group: the
// table of 8-point groups, then that of 16-point groups) after the 32 stride words of a warp's
// staging array.
static constexpr int kGroupTableMaxDl = 10;
static constexpr int kTgWords = 32 + 2 * (1 << (kGroupTableMaxDl - 3)) + 2 * (1 << (kGroupTableMaxDl - 4));
// The K chunks of a unit differ only in pair coordinates, so chunk k's sign for a walked
// coordinate j is a common one times (-1)^{k . g_j}, g_j the bits of coordinate j in the pair
// coordinates' G rows.  Its sum is therefore
//     S_k = i^{m_k(0)} sum_x (-1)^{popc(x & k)} T_x,   T_x = sum_{s: x(s) = x} i^{e(s)} w(s),
// x(s) = XOR of g_j over the set walked coordinates of s, e(s) the Z4 index of chunk 0 relative
// to the walk's start: every branch point s adds its table entry to ONE bucket T_{x(s)}, and a
// Walsh-Hadamard transform over the K buckets gives the K chunk sums -- the arithmetic of one
// chunk for K.  With coordinates 0..2 of even Z4 increment and g_0 = g_1 = gam (the host orders
// them so; del = g_2), the eight points of a group (coordinates 0..2 walked, the others fixed)
// fall in at most four buckets -- x0, x0 ^ gam, x0 ^ gam ^ del, x0 ^ del, two points each -- with
// per-lane signs that repeat every group: they are summed in local pairs and added into their
// buckets once per group (merged where buckets coincide, PAT below: two when del = gam, one when
// both are 0), turned by the group's start index i^{e0}.  Hi parts stay on the exact grid (every partial sum
// is a signed sub-sum of the chunk's terms); lo parts are summed in at most 2^dl / 8 + 6
// roundings per term, inside the walk's 2^dl-term bound.
template <int K>
__device__ __forceinline__ void bucket_add(uint64_t (&T)[K][2], uint32_t x, uint64_t s2, uint64_t h, uint64_t l) {
    switch (x) {
#define PQ_BA(c)                             \
    case c:                                  \
        if (c < K) {                         \
            T[c % K][0] = ffma2(s2, h, T[c % K][0]); \
            T[c % K][1] = ffma2(s2, l, T[c % K][1]); \
        }                                    \
        break;
        PQ_BA(0) PQ_BA(1) PQ_BA(2) PQ_BA(3) PQ_BA(4) PQ_BA(5) PQ_BA(6) PQ_BA(7)
#undef PQ_BA
    }
}

// i * (re, im) = (-im, re) on a pair
__device__ __forceinline__ uint64_t times_i(uint64_t p) {
    float a, b;
    up2(p, a, b);
    return pk2(-b, a);
}

// Walsh-Hadamard transform over the buckets, S_k = sum_x (-1)^{popc(x & k)} T_x, unpacked to
// (hi.re, hi.im, lo.re, lo.im) per chunk
template <int K>
__device__ __forceinline__ void bucket_transform(uint64_t (&T)[K][2], float (&S)[K][4]) {
    const uint64_t one2 = pk2(1.f, 1.f), neg2 = pk2(-1.f, -1.f);
#pragma unroll
    for (int h = 1; h < K; h <<= 1)
#pragma unroll
        for (int x = 0; x < K; x++)
            if (!(x & h)) {
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    const uint64_t a = T[x][c], bb = T[x | h][c];
                    T[x][c] = ffma2(one2, bb, a);
                    T[x | h][c] = ffma2(neg2, bb, a);
                }
            }
#pragma unroll
    for (int k = 0; k < K; k++) {
        up2(T[k][0], S[k][0], S[k][1]);
        up2(T[k][1], S[k][2], S[k][3]);
    }
}

// Bucket walk of one unit: on return S[k] = (hi.re, hi.im, lo.re, lo.im) of chunk k's sum
// without its start factor i^{m_k(0)}.  P1: c_j of chunk 0; grow[i]: pair coordinate i's G row
// over the walked coordinates; wad: the start point's entry address.
// PAT: which of a group's four bucket offsets coincide -- 0: gam = del = 0 (one bucket), 1:
// del = gam != 0 (x0, x0 ^ gam), 2: gam = 0 != del (x0, x0 ^ del), 3: none assumed (four adds,
// correct for every pattern; the one the enumeration instantiates for 8-point groups).
template <int K, int PAT>
__device__ __forceinline__ void bucket_walk(uint64_t wad, uint32_t P1, const uint32_t (&grow)[3],
                                            const uint32_t *Tg, const uint8_t *Lp, int dl, float (&S)[K][4]) {
    constexpr int NP = K == 8 ? 3 : (K == 4 ? 2 : 1);
    auto gbits = [&](int j) -> uint32_t {
        uint32_t g = 0;
#pragma unroll
        for (int i = 0; i < NP; i++) g |= ((grow[i] >> j) & 1u) << i;
        return g;
    };
    const uint32_t gam = gbits(0), del = gbits(2);  // gbits(1) == gam
    const uint32_t T0 = Tg[0], T1 = Tg[1], T2 = Tg[2];
    // sign of group position p (relative coordinates gray(p) = 0,1,3,2,6,7,5,4): parity of b & gray(p)
    const uint32_t b = ((((uint32_t)Lp[0] >> 1) ^ P1) & 1u) | (((((uint32_t)Lp[1] >> 1) ^ (P1 >> 1)) & 1u) << 1) |
                       (((((uint32_t)Lp[2] >> 1) ^ (P1 >> 2)) & 1u) << 2);
    auto sgn = [&](uint32_t gp) -> uint64_t {
        const float f = __uint_as_float(((__popc(b & gp) & 1u) << 31) | 0x3F800000u);
        return pk2(f, f);
    };
    const uint64_t s1p = sgn(1), s2p = sgn(3), s3p = sgn(2), s4p = sgn(6), s5p = sgn(7), s6p = sgn(5), s7p = sgn(4);
    const uint64_t one2 = pk2(1.f, 1.f), zero2 = 0ull;
    uint64_t T[K][2];
#pragma unroll
    for (int k = 0; k < K; k++) T[k][0] = T[k][1] = 0ull;
    // the eight entries of a group are loaded one group ahead: each position's register is
    // refilled with the next group's entry as soon as it has been added
#define PQ_LD(a) __ldg(reinterpret_cast<const ulonglong2 *>(a))
    ulonglong2 q0, q1, q2, q3, q4, q5, q6, q7;
    {
        uint64_t a = wad;
        q0 = PQ_LD(a);
        a ^= T0; q1 = PQ_LD(a);
        a ^= T1; q2 = PQ_LD(a);
        a ^= T0; q3 = PQ_LD(a);
        a ^= T2; q4 = PQ_LD(a);
        a ^= T0; q5 = PQ_LD(a);
        a ^= T1; q6 = PQ_LD(a);
        a ^= T0; q7 = PQ_LD(a);
    }
    // group g starts at S = gray(8 g); the job's group table (stage_job) holds, per group, the
    // XOR of S's coordinate strides, the bucket x(S) and the Z4 sum of Lp over S: the group's
    // entry addresses, bucket and start index i^{e0}, e0 = sum Lp S + 2 parity(P1 & S), follow
    // without any state carried from group to group
    const uint2 *Gt = reinterpret_cast<const uint2 *>(Tg + 32);
    const uint32_t ngroups = 1u << (dl - 3);
    uint2 gcur = Gt[0];
    for (uint32_t g = 0;; ++g) {
        const bool last = g + 1 == ngroups;
        const uint2 gnext = Gt[last ? g : g + 1];
        const uint32_t Sg = (g << 3) ^ (g << 2);
        const uint32_t x0 = gcur.y & (uint32_t)(K - 1);
        const uint32_t e0 = (gcur.y >> 8) + ((__popc(P1 & Sg) & 1u) << 1);
        uint64_t a = wad ^ (uint64_t)gnext.x;  // the next group's first point
        // positions 0, 2 -> x0 (A); 1, 3 -> x0 ^ gam (B); 4, 6 -> x0 ^ gam ^ del (C); 5, 7 -> x0 ^ del (D)
        uint64_t AH = q0.x, AL = q0.y, BH, BL, CH, CL, DH, DL;
        q0 = PQ_LD(a);
        a ^= T0; BH = ffma2(s1p, q1.x, zero2); BL = ffma2(s1p, q1.y, zero2); q1 = PQ_LD(a);
        a ^= T1; AH = ffma2(s2p, q2.x, AH); AL = ffma2(s2p, q2.y, AL); q2 = PQ_LD(a);
        a ^= T0; BH = ffma2(s3p, q3.x, BH); BL = ffma2(s3p, q3.y, BL); q3 = PQ_LD(a);
        a ^= T2; CH = ffma2(s4p, q4.x, zero2); CL = ffma2(s4p, q4.y, zero2); q4 = PQ_LD(a);
        a ^= T0; DH = ffma2(s5p, q5.x, zero2); DL = ffma2(s5p, q5.y, zero2); q5 = PQ_LD(a);
        a ^= T1; CH = ffma2(s6p, q6.x, CH); CL = ffma2(s6p, q6.y, CL); q6 = PQ_LD(a);
        a ^= T0; DH = ffma2(s7p, q7.x, DH); DL = ffma2(s7p, q7.y, DL); q7 = PQ_LD(a);
        // the group's sums (merged where buckets coincide), turned by i^{e0}, into their buckets
        if (PAT == 0 || PAT == 1) {  // C -> x0, D -> x0 ^ gam
            AH = ffma2(one2, CH, AH);
            AL = ffma2(one2, CL, AL);
            BH = ffma2(one2, DH, BH);
            BL = ffma2(one2, DL, BL);
        }
        if (PAT == 0 || PAT == 2) {  // B -> x0, D -> x0 ^ del
            AH = ffma2(one2, BH, AH);
            AL = ffma2(one2, BL, AL);
        }
        if (PAT == 2) {
            CH = ffma2(one2, DH, CH);
            CL = ffma2(one2, DL, CL);
        }
        if (e0 & 1u) {
            AH = times_i(AH);
            AL = times_i(AL);
            if (PAT != 0) {
                if (PAT == 2) {
                    CH = times_i(CH);
                    CL = times_i(CL);
                } else {
                    BH = times_i(BH);
                    BL = times_i(BL);
                }
            }
            if (PAT == 3) {
                CH = times_i(CH);
                CL = times_i(CL);
                DH = times_i(DH);
                DL = times_i(DL);
            }
        }
        const float sg = __uint_as_float(((e0 & 2u) << 30) | 0x3F800000u);
        const uint64_t sg2 = pk2(sg, sg);
        bucket_add<K>(T, x0, sg2, AH, AL);
        if (PAT == 1 || PAT == 3) bucket_add<K>(T, x0 ^ gam, sg2, BH, BL);
        if (PAT == 2) bucket_add<K>(T, x0 ^ del, sg2, CH, CL);
        if (PAT == 3) {
            bucket_add<K>(T, x0 ^ gam ^ del, sg2, CH, CL);
            bucket_add<K>(T, x0 ^ del, sg2, DH, DL);
        }
        if (last) break;
        gcur = gnext;
    }
#undef PQ_LD
    bucket_transform<K>(T, S);
}

// 16-point groups: coordinates 0..3 walked inside a group, g_0 = g_1 = gam and g_2 = g_3 = del,
// all four of even Z4 increment.  The group's 16 points fall in the same four buckets as an
// 8-point group, four points each; its second eight points (coordinates 2 and 3 both flipped
// relative to the first eight) repeat the first eight's buckets and signs times one per-lane
// sign s23 = (-1)^{b_2 ^ b_3}: the locals are multiplied by s23 between the halves and the
// group's sums added with s23 again.  The group table (stage_job, after the 8-point one) holds
// the same three fields for S = gray(16 g).
template <int K, int PAT>
__device__ __forceinline__ void bucket_walk16(uint64_t wad, uint32_t P1, const uint32_t (&grow)[3],
                                              const uint32_t *Tg, const uint8_t *Lp, int dl, float (&S)[K][4]) {
    constexpr int NP = K == 8 ? 3 : (K == 4 ? 2 : 1);
    auto gbits = [&](int j) -> uint32_t {
        uint32_t g = 0;
#pragma unroll
        for (int i = 0; i < NP; i++) g |= ((grow[i] >> j) & 1u) << i;
        return g;
    };
    const uint32_t gam = gbits(0), del = gbits(2);  // gbits(1) == gam, gbits(3) == del
    const uint32_t T0 = Tg[0], T1 = Tg[1], T2 = Tg[2], T23 = Tg[2] ^ Tg[3];
    uint32_t b = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) b |= ((((uint32_t)Lp[j] >> 1) ^ (P1 >> j)) & 1u) << j;
    auto sgn = [&](uint32_t gp) -> uint64_t {
        const float f = __uint_as_float(((__popc(b & gp) & 1u) << 31) | 0x3F800000u);
        return pk2(f, f);
    };
    const uint64_t s1p = sgn(1), s2p = sgn(3), s3p = sgn(2), s4p = sgn(6), s5p = sgn(7), s6p = sgn(5), s7p = sgn(4);
    const uint32_t s23bit = (((b >> 2) ^ (b >> 3)) & 1u) << 31;
    const uint64_t s23p = sgn(12);
    const uint64_t one2 = pk2(1.f, 1.f), zero2 = 0ull;
    uint64_t T[K][2];
#pragma unroll
    for (int k = 0; k < K; k++) T[k][0] = T[k][1] = 0ull;
#define PQ_LD(a) __ldg(reinterpret_cast<const ulonglong2 *>(a))
    ulonglong2 q0, q1, q2, q3, q4, q5, q6, q7;
    {
        uint64_t a = wad;
        q0 = PQ_LD(a);
        a ^= T0; q1 = PQ_LD(a);
        a ^= T1; q2 = PQ_LD(a);
        a ^= T0; q3 = PQ_LD(a);
        a ^= T2; q4 = PQ_LD(a);
        a ^= T0; q5 = PQ_LD(a);
        a ^= T1; q6 = PQ_LD(a);
        a ^= T0; q7 = PQ_LD(a);
    }
    const uint2 *Gt = reinterpret_cast<const uint2 *>(Tg + 32) + (1 << (kGroupTableMaxDl - 3));
    const uint32_t ngroups = 1u << (dl - 4);
    uint2 gcur = Gt[0];
    uint64_t AH, AL, BH, BL, CH, CL, DH, DL;
    // one half of a group: its eight entries (in q0..q7) into the locals, each register
    // refilled from the half that follows (first point at address nxt)
#define PQ_HALF(FIRST, nxt)                                                                              \
    {                                                                                                    \
        uint64_t a = (nxt);                                                                              \
        if (FIRST) { AH = q0.x; AL = q0.y; } else { AH = ffma2(one2, q0.x, AH); AL = ffma2(one2, q0.y, AL); } \
        q0 = PQ_LD(a);                                                                                   \
        a ^= T0; BH = ffma2(s1p, q1.x, FIRST ? zero2 : BH); BL = ffma2(s1p, q1.y, FIRST ? zero2 : BL); q1 = PQ_LD(a); \
        a ^= T1; AH = ffma2(s2p, q2.x, AH); AL = ffma2(s2p, q2.y, AL); q2 = PQ_LD(a);                    \
        a ^= T0; BH = ffma2(s3p, q3.x, BH); BL = ffma2(s3p, q3.y, BL); q3 = PQ_LD(a);                    \
        a ^= T2; CH = ffma2(s4p, q4.x, FIRST ? zero2 : CH); CL = ffma2(s4p, q4.y, FIRST ? zero2 : CL); q4 = PQ_LD(a); \
        a ^= T0; DH = ffma2(s5p, q5.x, FIRST ? zero2 : DH); DL = ffma2(s5p, q5.y, FIRST ? zero2 : DL); q5 = PQ_LD(a); \
        a ^= T1; CH = ffma2(s6p, q6.x, CH); CL = ffma2(s6p, q6.y, CL); q6 = PQ_LD(a);                    \
        a ^= T0; DH = ffma2(s7p, q7.x, DH); DL = ffma2(s7p, q7.y, DL); q7 = PQ_LD(a);                    \
    }
    for (uint32_t g = 0;; ++g) {
        const bool last = g + 1 == ngroups;
        const uint2 gnext = Gt[last ? g : g + 1];
        const uint32_t Sg = (g << 4) ^ (g << 3);
        const uint32_t x0 = gcur.y & (uint32_t)(K - 1);
        const uint32_t e0 = (gcur.y >> 8) + ((__popc(P1 & Sg) & 1u) << 1);
        PQ_HALF(true, wad ^ (uint64_t)gcur.x ^ (uint64_t)T23)
        AH = ffma2(s23p, AH, zero2); AL = ffma2(s23p, AL, zero2);
        BH = ffma2(s23p, BH, zero2); BL = ffma2(s23p, BL, zero2);
        CH = ffma2(s23p, CH, zero2); CL = ffma2(s23p, CL, zero2);
        DH = ffma2(s23p, DH, zero2); DL = ffma2(s23p, DL, zero2);
        PQ_HALF(false, wad ^ (uint64_t)gnext.x)
        if (PAT == 0 || PAT == 1) {
            AH = ffma2(one2, CH, AH);
            AL = ffma2(one2, CL, AL);
            BH = ffma2(one2, DH, BH);
            BL = ffma2(one2, DL, BL);
        }
        if (PAT == 0 || PAT == 2) {
            AH = ffma2(one2, BH, AH);
            AL = ffma2(one2, BL, AL);
        }
        if (PAT == 2) {
            CH = ffma2(one2, DH, CH);
            CL = ffma2(one2, DL, CL);
        }
        if (e0 & 1u) {
            AH = times_i(AH);
            AL = times_i(AL);
            if (PAT != 0) {
                if (PAT == 2) {
                    CH = times_i(CH);
                    CL = times_i(CL);
                } else {
                    BH = times_i(BH);
                    BL = times_i(BL);
                }
            }
            if (PAT == 3) {
                CH = times_i(CH);
                CL = times_i(CL);
                DH = times_i(DH);
                DL = times_i(DL);
            }
        }
        const float sg = __uint_as_float((((e0 & 2u) << 30) ^ s23bit) | 0x3F800000u);
        const uint64_t sg2 = pk2(sg, sg);
        bucket_add<K>(T, x0, sg2, AH, AL);
        if (PAT == 1 || PAT == 3) bucket_add<K>(T, x0 ^ gam, sg2, BH, BL);
        if (PAT == 2) bucket_add<K>(T, x0 ^ del, sg2, CH, CL);
        if (PAT == 3) {
            bucket_add<K>(T, x0 ^ gam ^ del, sg2, CH, CL);
            bucket_add<K>(T, x0 ^ del, sg2, DH, DL);
        }
        if (last) break;
        gcur = gnext;
    }
#undef PQ_HALF
#undef PQ_LD
    bucket_transform<K>(T, S);
}

// One unit of K chunks (K = 2^np: the chunk at s1 and those that differ from it in the first np
// pair coordinates) on the FP32 joint-table path: folded start indices, c_j of the walked
// coordinates, the rotating-frame walk, each chunk's sum rotated to its last index, the chunks
// combined with their pair-coordinate weights, and the unit's sum scaled by the weight of its
// other high coordinates and added into (accx, accy).
template <int MODE, int K>
__device__ __forceinline__ void walk_unit(const EngineDev &E, const JobDev &J, const uint64_t *G, const uint64_t *R,
                                          const uint8_t *Lp, const uint32_t *Tg, int dl, uint64_t s1, uint64_t lomask,
                                          uint8_t *dbg, double &accx, double &accy) {
    const uint64_t himask = ~lomask;
    const uint32_t wmask = (1u << dl) - 1u;
    uint32_t m1;
    uint64_t yy;
    chunk_start(Lp, G, R, J.y0, s1, m1, yy);
    m1 -= 2u * quad_parity(G, s1 & lomask);  // the table holds the low-coordinate quadratic part
    uint32_t P1 = 0;
    for (int j = 0; j < dl; j++) P1 |= (uint32_t)(popc64(G[j] & s1 & himask) & 1) << j;
    const uint32_t sidx = (uint32_t)((joint_pivots(E, yy) << E.DI) | (s1 & lomask));
    // chunk k = s1 + the pair coordinates of the bits of k: its index grows by their linear terms
    // at s1 plus 2 G between each two of them; its c_j by their G rows
    uint32_t dlin[3] = {0u, 0u, 0u}, grow[3] = {0u, 0u, 0u};
#pragma unroll
    for (int i = 0; i < 3; i++)
        if ((1 << i) < K) {
            const int p = E.pairc[i];
            dlin[i] = (uint32_t)Lp[p] + 2u * (uint32_t)(popc64(G[p] & s1) & 1);
            grow[i] = (uint32_t)G[p] & wmask;
        }
    // index and high-coordinate bits of chunk k, recomputed where needed to keep registers free
    auto chunk_m = [&](int k) -> uint32_t {
        uint32_t mk = m1;
#pragma unroll
        for (int i = 0; i < 3; i++)
            if ((1 << i) < K && ((k >> i) & 1)) {
                mk += dlin[i];
#pragma unroll
                for (int i2 = 0; i2 < i; i2++)
                    if ((k >> i2) & 1) mk += 2u * (uint32_t)((G[E.pairc[i]] >> E.pairc[i2]) & 1ull);
            }
        return mk;
    };
    auto chunk_s = [&](int k) -> uint64_t {
        uint64_t sk = s1;
#pragma unroll
        for (int i = 0; i < 3; i++)
            if ((1 << i) < K && ((k >> i) & 1)) sk |= 1ull << E.pairc[i];
        return sk;
    };
    float acc[K][4];
    uint32_t qk[K];  // quarter turns from each chunk's walk result to its sum
    // bucket walk: units of 4 or 8 chunks whose first three walked coordinates have even Z4
    // increments and whose first two have equal bits in the pair coordinates' G rows
    bool bucket = false;
    if (MODE == 0 && (K == 4 || K == 8) && dl >= 3 && dl <= kGroupTableMaxDl && !((Lp[0] | Lp[1] | Lp[2]) & 1)) {
        constexpr int NPK = K == 8 ? 3 : 2;
        bool same = true;
#pragma unroll
        for (int i = 0; i < NPK; i++) {
            const uint32_t gi = grow[i] & 3u;
            same = same && (gi == 0u || gi == 3u);
        }
        bucket = same;
    }
    if (bucket) {
        const uint64_t wad = reinterpret_cast<uint64_t>(E.wtab) | ((uint64_t)sidx << 4);
        constexpr int NPB = K == 8 ? 3 : 2;
        uint32_t g0 = 0, g2 = 0;
        bool pair23 = dl >= 4 && !(Lp[3] & 1);  // coordinates 2 and 3 agree: 16-point groups
#pragma unroll
        for (int i = 0; i < NPB; i++) {
            g0 |= (grow[i] & 1u) << i;
            g2 |= ((grow[i] >> 2) & 1u) << i;
            const uint32_t h = (grow[i] >> 2) & 3u;
            pair23 = pair23 && (h == 0u || h == 3u);
        }
        const int pat = (g0 == 0u && g2 == 0u) ? 0 : (g2 == g0 ? 1 : (g0 == 0u ? 2 : 3));
        if (pair23) {
            if (pat == 0) bucket_walk16<K, 0>(wad, P1, grow, Tg, Lp, dl, acc);
            else if (pat == 1) bucket_walk16<K, 1>(wad, P1, grow, Tg, Lp, dl, acc);
            else if (pat == 2) bucket_walk16<K, 2>(wad, P1, grow, Tg, Lp, dl, acc);
            else bucket_walk16<K, 3>(wad, P1, grow, Tg, Lp, dl, acc);
        } else {
            // 8-point groups (engines without two equally coupled pairs): one variant for all
            // bucket patterns keeps the kernel's hot code small
            bucket_walk<K, 3>(wad, P1, grow, Tg, Lp, dl, acc);
        }
#pragma unroll
        for (int k = 0; k < K; k++) qk[k] = chunk_m(k) & 3u;
    } else {
    uint32_t Pc[K], mm[K];
    uint64_t sb[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        uint32_t pk = P1;
#pragma unroll
        for (int i = 0; i < 3; i++)
            if ((1 << i) < K && ((k >> i) & 1)) pk ^= grow[i];
        Pc[k] = pk;
        if (MODE == 2) {
            mm[k] = chunk_m(k);
            sb[k] = chunk_s(k);
        } else {
            mm[k] = 0u;
            sb[k] = 0ull;
        }
    }
    gray_chunk_rot_any<MODE, K>(E.wtab, sidx, Pc, Tg, Lp, dl, acc, dbg, sb, J.k0, mm, G, (uint32_t)lomask);
    const int jl = dl - 1;
#pragma unroll
    for (int k = 0; k < K; k++) qk[k] = (chunk_m(k) + (uint32_t)Lp[jl] + (((Pc[k] >> jl) & 1u) << 1)) & 3u;
    }
    // The unit's chunks differ only in pair coordinates: their high-coordinate weights are
    // chi_rest(s1) P(pattern), so the unit sum is chi_rest(s1) sum_k P(k | pat) S_k.  The inner
    // sum runs in FP32 pairs (exact products by FMA, two-sums), the outer product in FP64 once
    // per unit.
    constexpr int npk = K == 8 ? 3 : (K == 4 ? 2 : (K == 2 ? 1 : 0));
    uint32_t pat = 0;  // bits of s1 at the pair coordinates the unit does not vary
    for (int i = npk; i < E.npairc; i++) pat |= (uint32_t)((s1 >> E.pairc[i]) & 1ull) << i;
    float urh = 0.f, url = 0.f, uih = 0.f, uil = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) {
        // the chunk's sum: an exact quarter turn of the FP32 pairs (walk: i^{m_end} A, m_end =
        // m + L'_{dl-1}; bucket walk: i^{m_k(0)} S)
        const uint32_t q = qk[k];
        float hx = acc[k][0], hy = acc[k][1], lx = acc[k][2], ly = acc[k][3];
        if (q & 1u) {
            const float t = hx; hx = -hy; hy = t;
            const float t2 = lx; lx = -ly; ly = t2;
        }
        if (q & 2u) { hx = -hx; hy = -hy; lx = -lx; ly = -ly; }
        const float4 P = E.pf[(uint32_t)k | pat];
        ff_cmul_acc(P, hx, hy, lx, ly, urh, url, uih, uil);
    }
    const double ux = (double)urh + (double)url, uy = (double)uih + (double)uil;
    // the unit's chunks share their pivots outside a partial table (the walked and the pair
    // coordinates do not touch them): one FP64 factor with the other high coordinates' weight
    const double2 chi = E.thp ? cmul_d(chunk_rest_weight(E, s1), high_pivot_weight(E, yy)) : chunk_rest_weight(E, s1);
    accx += ux * chi.x - uy * chi.y;
    accy += ux * chi.y + uy * chi.x;
}

// Stage job jb's walk data (quadratic form rows, pivot masks, Z4 increments and their negatives,
// table byte strides) into one warp's shared arrays.
__device__ __forceinline__ void stage_job(const KArgs &a, int jb, uint64_t *G, uint64_t *R, uint8_t *Lp, uint8_t *Lm,
                                          uint32_t *Tg, int lane) {
    const JobDev &J = a.jobs[jb];
    const EngineDev &E = a.engines[J.engine];
    __syncwarp();
    const int dlj = a.jdl[jb] & 255;
    for (int j = lane; j < E.d; j += 32) {
        G[j] = E.G[j];
        R[j] = E.R[j];
        Lp[j] = J.Lp[j];
        Lm[j] = (uint8_t)((4u - J.Lp[j]) & 3u);
        if (j < dlj) Tg[j] = ((1u << j) | ((uint32_t)E.Rc[j] << E.DI)) << 4;
    }
    __syncwarp();
    // the bucket walk's group table, after the 32 stride words: for group g its start point
    // S = gray(8 g) (bits 2 .. dl - 1): the XOR of S's strides, the parities of S with the pair
    // coordinates' G rows (bucket) and, from bit 8, the sum of Lp over S mod 4
    const int npj = (a.jdl[jb] >> 8) & 3;
    // (8-point groups, S = gray(8 g), then 16-point groups, S = gray(16 g))
    if (E.joint && npj >= 2 && dlj >= 3 && dlj <= kGroupTableMaxDl) {
        uint2 *Gt = reinterpret_cast<uint2 *>(Tg + 32);
        const int n8 = 1 << (dlj - 3), n16 = dlj >= 4 ? 1 << (dlj - 4) : 0;
        for (int e = lane; e < n8 + n16; e += 32) {
            const uint32_t g = (uint32_t)(e < n8 ? e : e - n8);
            const uint32_t S = e < n8 ? (g << 3) ^ (g << 2) : (g << 4) ^ (g << 3);
            uint32_t off = 0, u = 0, x = 0;
            for (int j = 2; j < dlj; j++)
                if ((S >> j) & 1u) {
                    off ^= Tg[j];
                    u += Lp[j];
                }
            for (int i = 0; i < npj; i++) x |= (uint32_t)(popc64(G[E.pairc[i]] & (uint64_t)S) & 1) << i;
            Gt[e < n8 ? g : (1u << (kGroupTableMaxDl - 3)) + g] = make_uint2(off, x | ((u & 3u) << 8));
        }
        __syncwarp();
    }
}

// Sum of work item iin of job `job` (its staged data in G, R, Lp, Lm, Tg): every lane walks its
// units, then an FP64 warp-shuffle reduce in a fixed order; lane 0's value is the item's partial.
template <int MODE, int MINB>
__device__ __forceinline__ double2 item_partial(const KArgs &a, int job, long long iin, const uint64_t *G,
                                                const uint64_t *R, const uint8_t *Lp, const uint8_t *Lm,
                                                const uint32_t *Tg, int lane) {
    const JobDev &J = a.jobs[job];
    const EngineDev &E = a.engines[J.engine];
    double accx = 0.0, accy = 0.0;
    if (!J.vanish) {
        const int dl = a.jdl[job] & 255;
        const int np = (a.jdl[job] >> 8) & 3;  // pair coordinates used by this job's units
        const int nk = 1 << np;
        const unsigned cpi = a.jcpi[job];
        const unsigned long long nun = a.jnch[job];
        const unsigned long long c0 = (unsigned long long)iin * cpi;
        unsigned long long cend = c0 + cpi;
        if (cend > nun) cend = nun;
        const uint64_t lomask = (E.DI >= 64) ? ~0ull : ((1ull << E.DI) - 1ull);
        const uint32_t steps = 1u << dl;
        if (MODE != 2 && a.use_ctab && E.ctab && dl == E.DI && np == 0 && (cpi & (cpi - 1)) == 0) {
            // Chunk-sum tables: lane l sums the item's chunks base .. base + q - 1 (base =
            // c0 + l q, q = cpi / 32 a power of two) in Gray order, one FP64 table lookup per
            // chunk.  A step flips one high coordinate j: the folded index gains
            // +-Lp_j + 2 parity(G_j & s), the pivot bits R_j, the low-coordinate signs b the
            // row G_j; chunks past the item's end are walked but not added.
            const unsigned long long q = (unsigned long long)(cpi >> 5) ? (unsigned long long)(cpi >> 5) : 1ull;
            const unsigned long long base = c0 + (unsigned long long)lane * q;
            if (base < cend) {
                uint64_t s = (uint64_t)base << dl;
                uint32_t m;
                uint64_t yy;
                chunk_start(Lp, G, R, J.y0, s, m, yy);
                uint32_t b = 0;
                for (int j = 0; j < dl; j++)
                    b |= (((uint32_t)(Lp[j] >> 1) ^ (uint32_t)popc64(G[j] & s)) & 1u) << j;
                const uint32_t lm32 = (uint32_t)lomask;
                // the run varies the coordinates dl .. dl + log2(q) - 1; when they all lie in
                // the first byte slice of the high weight, the other slices are one factor
                const bool one_slice = (dl + ctz64(q)) <= E.DI + 8;
                double rx = 0.0, ry = 0.0;
                for (unsigned long long i = 0;; ++i) {
                    const unsigned long long ch = base + (i ^ (i >> 1));
                    if (ch < cend) {
                        double2 v = rot4d(E.ctab[(joint_pivots(E, yy) << E.DI) | b], m & 3u);
                        if (E.thp) v = cmul_d(v, high_pivot_weight(E, yy));
                        const double2 chi = one_slice ? (E.nsl_th > 0 ? E.th[(int)((s >> E.DI) & 255ull)]
                                                                      : make_double2(1.0, 0.0))
                                                      : chunk_high_weight(E, s);
                        rx += v.x * chi.x - v.y * chi.y;
                        ry += v.x * chi.y + v.y * chi.x;
                    }
                    if (i + 1 == q) break;
                    const int j = dl + ctz64(i + 1);
                    m += (((s >> j) & 1ull) ? Lm[j] : Lp[j]) + 2u * (uint32_t)(popc64(G[j] & s) & 1);
                    yy ^= R[j];
                    b ^= (uint32_t)G[j] & lm32;
                    s ^= 1ull << j;
                }
                double2 rest = make_double2(1.0, 0.0);
                if (one_slice)
                    for (int sl = 1; sl < E.nsl_th; sl++)
                        rest = cmul_d(rest, E.th[sl * 256 + (int)((s >> (E.DI + 8 * sl)) & 255ull)]);
                accx += rx * rest.x - ry * rest.y;
                accy += rx * rest.y + ry * rest.x;
            }
        } else
        for (unsigned long long un = c0 + lane; un < cend; un += 32) {
            // unit -> its first chunk (zeros inserted at the pair coordinates' chunk bits)
            unsigned long long ch = un;
            for (int i = 0; i < np; i++) ch = insert_zero(ch, E.pairc[i] - dl);
            const uint64_t s1 = (uint64_t)ch << dl;
            if (MODE != 2 && a.use_ctab && E.ctab && dl == E.DI) {
                // chunk-sum tables on a plan laid out for the walk (units of several
                // chunks): each chunk from its own start
                for (int kc = 0; kc < nk; kc++) {
                    uint64_t s = s1;
                    for (int i = 0; i < np; i++)
                        if ((kc >> i) & 1) s |= 1ull << E.pairc[i];
                    uint32_t m;
                    uint64_t yy;
                    chunk_start(Lp, G, R, J.y0, s, m, yy);
                    uint32_t b = 0;
                    for (int j = 0; j < dl; j++)
                        b |= (((uint32_t)(Lp[j] >> 1) ^ (uint32_t)popc64(G[j] & s)) & 1u) << j;
                    double2 v = rot4d(E.ctab[(joint_pivots(E, yy) << E.DI) | b], m & 3u);
                    if (E.thp) v = cmul_d(v, high_pivot_weight(E, yy));
                    const double2 chi = chunk_high_weight(E, s);
                    accx += v.x * chi.x - v.y * chi.y;
                    accy += v.x * chi.y + v.y * chi.x;
                }
                continue;
            }
            if (MODE != 1 && E.joint && dl >= 3) {
                if (np == 3) {
                    if (MINB == 2) {  // eight accumulators per lane: only with the 128-register budget
                        walk_unit<MODE, (MINB == 2 ? 8 : 4)>(E, J, G, R, Lp, Tg, dl, s1, lomask, a.dbg, accx, accy);
                    } else {
                        walk_unit<MODE, 4>(E, J, G, R, Lp, Tg, dl, s1, lomask, a.dbg, accx, accy);
                        walk_unit<MODE, 4>(E, J, G, R, Lp, Tg, dl, s1 | (1ull << E.pairc[2]), lomask, a.dbg, accx,
                                           accy);
                    }
                } else if (np == 2) walk_unit<MODE, 4>(E, J, G, R, Lp, Tg, dl, s1, lomask, a.dbg, accx, accy);
                else if (np == 1) walk_unit<MODE, 2>(E, J, G, R, Lp, Tg, dl, s1, lomask, a.dbg, accx, accy);
                else walk_unit<MODE, 1>(E, J, G, R, Lp, Tg, dl, s1, lomask, a.dbg, accx, accy);
                continue;
            }
            const uint64_t himask = ~lomask;
            for (int kc = 0; kc < nk; kc++) {
                uint64_t s = s1;
                for (int i = 0; i < np; i++)
                    if ((kc >> i) & 1) s |= 1ull << E.pairc[i];
                uint32_t m;
                uint64_t yy;
                chunk_start(Lp, G, R, J.y0, s, m, yy);
                uint64_t ss = s;
                double vx, vy;  // the chunk's sum before the weight of the coordinates >= DI
                double2 tph = make_double2(1.0, 0.0);  // weight of pivots outside a partial table
                if (MODE == 1 || !E.joint) {
                    // FP64 weights and accumulation (verification mode, and engines with more
                    // pivots than the joint table holds)
                    double sx = 0.0, sy = 0.0;
                    for (uint32_t i = 1;; ++i) {
                        if (MODE == 2) a.dbg[ss] = (uint8_t)((J.k0 + 2u * m) & 7u);
                        double2 w = E.tlo64[ss & lomask];
                        for (int sl = 0; sl < E.nsl_tp; sl++)
                            w = cmul_d(w, E.tp64[sl * 256 + (int)((yy >> (8 * sl)) & 255ull)]);
                        w = rot4d(w, m & 3u);
                        sx += w.x;
                        sy += w.y;
                        if (i == steps) break;
                        const int j = ctz32(i);
                        m += (((ss >> j) & 1ull) ? Lm[j] : Lp[j]) + 2u * (uint32_t)(popc64(G[j] & ss) & 1);
                        ss ^= 1ull << j;
                        yy ^= R[j];
                    }
                    vx = sx;
                    vy = sy;
                } else {
                    // FP32, chunks of fewer than 8 steps: per-branch folded index over the
                    // sign-folded table, plain sums
                    m -= 2u * quad_parity(G, s & lomask);
                    float hx = 0.f, hy = 0.f, lx = 0.f, ly = 0.f;
                    const float4 *__restrict__ W = E.wtab;
                    const int DI = E.DI;
                    // pivots outside the table: constant over the chunk (its walked coordinates
                    // touch only pivots in pmask)
                    tph = high_pivot_weight(E, yy);
                    for (uint32_t i = 1;; ++i) {
                        if (MODE == 2)
                            a.dbg[ss] = (uint8_t)((J.k0 + 2u * (m + 2u * quad_parity(G, ss & lomask))) & 7u);
                        const float4 w = rot4q(__ldg(&W[(joint_pivots(E, yy) << DI) | (ss & lomask)]), m & 3u);
                        hx += w.x;
                        hy += w.y;
                        lx += w.z;
                        ly += w.w;
                        if (i == steps) break;
                        const int j = ctz32(i);
                        m += (((ss >> j) & 1ull) ? Lm[j] : Lp[j]) + 2u * (uint32_t)(popc64(G[j] & ss & himask) & 1);
                        ss ^= 1ull << j;
                        yy ^= R[j];
                    }
                    vx = (double)hx + (double)lx;
                    vy = (double)hy + (double)ly;
                }
                const double2 chi = cmul_d(chunk_high_weight(E, s), tph);
                accx += vx * chi.x - vy * chi.y;
                accy += vx * chi.y + vy * chi.x;
            }
        }
    }
    for (int o = 16; o; o >>= 1) {
        accx += __shfl_xor_sync(PQ_FULL, accx, o);
        accy += __shfl_xor_sync(PQ_FULL, accy, o);
    }
    return make_double2(accx, accy);
}

// MODE 0: FP32 weights (exact-grid hi + lo) in the rotating-frame walk.  MODE 1: FP64 weights
// and accumulation.  In both, jobs with chunk-sum tables take their chunk sums from them when
// the launch asks for tables (use_ctab).
// MODE 2: record the Z8 index of every branch into dbg (single-job debug launches).
// MINB: resident blocks of 256 threads per SM the register allocation is sized for (2: 128,
// 3: 80, 4: 64 registers per thread) -- chosen per launch by measurement.
template <int MODE, int MINB = 3>
__global__ void __launch_bounds__(256, MINB) enum_kernel(KArgs a) {
    __shared__ uint64_t sG[8][64];
    __shared__ uint64_t sR[8][64];
    __shared__ uint8_t sLp[8][64];
    __shared__ uint8_t sLm[8][64];
    // byte stride of coordinate j in the table, ((1 << j) | (R_j << DI)) * 16, then the bucket
    // walk's group table
    __shared__ __align__(16) uint32_t sTg[8][kTgWords];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t *G = sG[wib];
    uint64_t *R = sR[wib];
    uint8_t *Lp = sLp[wib];
    uint8_t *Lm = sLm[wib];
    uint32_t *Tg = sTg[wib];
    int cur_k = -1;  // position (item order) of the job whose data is staged
    long long kbeg = 0, kend = 0;
    // The items (jobs in engine order) are cut into nslices contiguous slices, one per SM: the
    // warps of an SM take the items of its slice in order -- neighbouring items, mostly one
    // engine's jobs, so they share its table in L1 -- and then those of the following slices.
    // Each slice's counter hands out every item of it once; a warp stops after it has found
    // every slice exhausted.
    const int ns = a.nslices > 1 ? a.nslices : 1;
    unsigned smid;
    asm("mov.u32 %0, %%smid;" : "=r"(smid));
    int sl = (int)(smid % (unsigned)ns), left = ns;
    while (true) {
        const long long sb = a.nitems * sl / ns, se = a.nitems * (sl + 1) / ns;
        unsigned long long it0 = 0;
        if (lane == 0) it0 = atomicAdd(a.counter + sl, 1ull);
        const long long it = sb + (long long)__shfl_sync(PQ_FULL, it0, 0);
        if (it >= se) {
            if (--left == 0) break;
            sl = sl + 1 == ns ? 0 : sl + 1;
            continue;
        }
        if (!(it >= kbeg && it < kend)) {
            int lo = 0, hi = a.njobs - 1;  // last k with istart[k] <= it
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (a.istart[mid] <= it) lo = mid; else hi = mid - 1;
            }
            cur_k = lo;
            kbeg = a.istart[lo];
            kend = a.istart[lo + 1];
            stage_job(a, a.perm[lo], G, R, Lp, Lm, Tg, lane);
        }
        const int job = a.perm[cur_k];
        const double2 p = item_partial<MODE, MINB>(a, job, it - kbeg + (a.ioff ? a.ioff[job] : 0), G, R, Lp, Lm,
                                                   Tg, lane);
        if (lane == 0) a.partials[it] = p;
    }
}

// ------------------------------------------------------------------------------ reductions
__device__ __forceinline__ double2 phase_to_complex_dev(uint32_t p) {
    if ((p & ((1u << 29) - 1u)) == 0) {
        int k = (int)(p >> 29);
        return make_double2(c_root8[2 * k], c_root8[2 * k + 1]);
    }
    double s, c;
    sincospi((double)p * 4.656612873077392578125e-10, &s, &c);  // angle = pi * p / 2^31
    return make_double2(c, s);
}

// Value and error bound of job j from the sum (sx, sy) of its item partials in item order.
__device__ __forceinline__ void job_finish(const KArgs &a, int j, double sx, double sy, double2 &v, double &eb) {
    const JobDev &J = a.jobs[j];
    const EngineDev &E = a.engines[J.engine];
    v = make_double2(0.0, 0.0);
    eb = 0.0;
    if (!J.vanish) {
        const int k = a.kinv[j];
        const double2 r8 = make_double2(c_root8[2 * (J.k0 & 7u)], c_root8[2 * (J.k0 & 7u) + 1]);
        v = cmul_d(cmul_d(make_double2(sx, sy), r8), phase_to_complex_dev(J.phase));
        const double mag = pow2_half(E.mag2 - E.num_h);
        v.x *= mag;
        v.y *= mag;
        // Bound on |computed - exact| relative to sum_s |c(s)| * mag (conservative):
        //  joint table: weights exact to 2^-46 (hi + lo of an FP64 product); hi chunk sums are
        //  exact, the terms below keep an allowance of gamma_n^2 + 2 n u^2 (gamma_n = n u /
        //  (1 - n u), n = 2^dl) for them; FP64 unit scaling and reductions a few 2^-52; the lo
        //  sums add errfac (per engine, from the grid).  FP64 path: (n + 2 nsl_tp + 8 + nsl_th)
        //  2^-52.  Every path adds the FP64 running sums over a lane's chunks and a job's items.
        const double u32 = 5.9604644775390625e-08, u64 = 1.1102230246251565e-16;
        const double n = (double)(1ull << (a.jdl[j] & 255));
        double rel;
        const int dlj = a.jdl[j] & 255;
        const bool ctab = a.use_ctab && E.ctab && dlj == E.DI;
        // FP64 running sums shared by every path: a lane's chunks (at most nk ceil(cpi / 32)),
        // the job's items (recursive summation: n terms, n u relative to sum |c|)
        const unsigned long long cpi = a.jcpi[j];
        const double lane_chunks = (double)(1 << ((a.jdl[j] >> 8) & 3)) * (double)((cpi + 31) / 32);
        const double items = (double)(a.istart[k + 1] - a.istart[k]);
        const double sums = (lane_chunks + items) * 2.0 * u64;
        if (ctab) {
            // FP64 throughout, in units of 2u: the table entry (complex products of at most
            // DI + 13 factors, sqrt(5) u each, then a DI-stage transform), each chunk's
            // high-coordinate factor (nsl_th products of 8-factor slice products) and its
            // product with the entry, the 5-level warp reduction, the final scalings
            rel = (2.0 * (double)E.DI + 16.0 + 10.0 * (double)E.nsl_th + 5.0 + 64.0) * 2.0 * u64;
            if (E.thp) rel += (2.0 * E.nsl_tp + 2.0) * 2.0 * u64;  // the chunk's other-pivot factor
        } else if (E.joint && !a.fp64_mode) {
            // + 1e-12: the FP32-pair combination of a unit's chunks (at most 8 terms, each with
            // error a few 2^-48 of its magnitude)
            const double g = n * u32 / (1.0 - n * u32);
            rel = g * g + 2.0 * n * u32 * u32 + 1.5e-14 + 64.0 * u64 + 1e-12;
            // a partial table's pivot factor: nsl_tp FP64 complex products per unit
            if (E.thp) rel += (2.0 * E.nsl_tp + 2.0) * 2.0 * u64;
        } else {
            rel = (n + 2.0 * E.nsl_tp + 8.0 + (double)E.nsl_th) * 2.0 * u64;
        }
        rel += sums;
        eb = rel * E.sum_abs_bound * mag;
        // lo-part sums of the walk, and the FP32 rounding of their products with the pair
        // weights when a unit's chunks are combined (at most 16 u |P| |lo sum| per chunk: 4 / n
        // of the sums' own bound)
        if (E.joint && !ctab && !a.fp64_mode) eb += E.errfac * (1.0 + 4.0 / n) * mag;
    }
}

__global__ void job_reduce_kernel(KArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.njobs) return;
    double sx = 0.0, sy = 0.0;
    if (!a.jobs[j].vanish) {
        const int k = a.kinv[j];
        for (long long i = a.istart[k]; i < a.istart[k + 1]; i++) {
            sx += a.partials[i].x;
            sy += a.partials[i].y;
        }
    }
    double2 v;
    double eb;
    job_finish(a, j, sx, sy, v, eb);
    a.job_vals[j] = v;
    a.job_err[j] = eb;
}

// Output o from its jobs' values and bounds (vals[i], errs[i] of job out_jobs[o] + i), summed
// in job order.
__device__ __forceinline__ void out_finish(const KArgs &a, int o, const double2 *vals, const double *errs) {
    double sx = 0.0, sy = 0.0, eb = 0.0;
    const int nj = a.out_jobs[o + 1] - a.out_jobs[o];
    for (int i = 0; i < nj; i++) {
        sx += vals[i].x;
        sy += vals[i].y;
        eb += errs[i];
    }
    // a failed device self-check (prepare saw an odd Z8 increment, which the closed form rules
    // out) makes every result of the launch NaN, so callers that do not wait on the host still
    // see it in the results
    if (a.errflag && *(volatile const int *)a.errflag) sx = sy = eb = __longlong_as_double(0x7ff8000000000000ll);
    const double mod = sqrt(sx * sx + sy * sy);
    eb += 4.0 * 1.1102230246251565e-16 * mod;  // FP64 output rounding
    if (a.out_prob) {
        a.out[o] = sx * sx + sy * sy;
        if (a.err) a.err[o] = eb * (2.0 * mod + eb);
    } else {
        a.out[2 * o] = sx;
        a.out[2 * o + 1] = sy;
        if (a.err) a.err[o] = eb;
    }
}

__global__ void out_reduce_kernel(KArgs a) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= a.nout) return;
    out_finish(a, o, a.job_vals + a.out_jobs[o], a.job_err + a.out_jobs[o]);
}

// ------------------------------------------------------------------------------ fused small launch
// The whole evaluation of a small launch (every output's branch engines of at most
// kSmallMaxJobs jobs and few work items) in one kernel: a block per output, its warps take the
// output's jobs in turn -- prepare, then the job's work items one after another with the
// enumeration's own per-item code, summed in item order as job_reduce sums them -- and the
// block sums the job values in job order as out_reduce does.  The arithmetic and its order are
// those of the four-kernel sequence, so the results are the same numbers.  The output's
// boundary is copied into shared memory first (it may live in mapped host memory).
static const int kSmallMaxJobs = 64;

// Shared-memory working set of the fused evaluation of one output (per block).
struct SmallShared {
    uint64_t G[8][64];
    uint64_t R[8][64];
    uint8_t Lp[8][64];
    uint8_t Lm[8][64];
    alignas(16) uint32_t Tg[8][kTgWords];
    double2 val[kSmallMaxJobs];
    double err[kSmallMaxJobs];
};

// Output o of a fused launch on one block, its boundary already in shared memory (bx, by): the
// warps take the output's jobs in turn, then thread 0 sums them.  Every thread of the block
// calls it; it ends with the output written.
template <int MINB>
__device__ __forceinline__ void small_output(const KArgs &a, int o, const uint64_t *bx, const uint64_t *by,
                                             uint64_t *u, SmallShared &sh, int lane, int wib, int wpb) {
    const int j0 = a.out_jobs[o], nj = a.out_jobs[o + 1] - j0;
    for (int i = wib; i < nj; i += wpb) {
        const int j = j0 + i;
        prepare_job(a, j, bx, by, u, lane);
        double sx = 0.0, sy = 0.0;
        if (!a.jobs[j].vanish) {
            stage_job(a, j, sh.G[wib], sh.R[wib], sh.Lp[wib], sh.Lm[wib], sh.Tg[wib], lane);
            const int k = a.kinv[j];
            const long long nit = a.istart[k + 1] - a.istart[k], i0 = a.ioff ? a.ioff[j] : 0;
            for (long long iin = 0; iin < nit; iin++) {
                const double2 p = item_partial<0, MINB>(a, j, i0 + iin, sh.G[wib], sh.R[wib], sh.Lp[wib], sh.Lm[wib],
                                                        sh.Tg[wib], lane);
                sx += __shfl_sync(PQ_FULL, p.x, 0);
                sy += __shfl_sync(PQ_FULL, p.y, 0);
            }
        }
        if (lane == 0) {
            double2 v;
            double eb;
            job_finish(a, j, sx, sy, v, eb);
            sh.val[i] = v;
            sh.err[i] = eb;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) out_finish(a, o, sh.val, sh.err);
}

template <int MINB>
__global__ void __launch_bounds__(256, MINB) small_kernel(KArgs a) {
    __shared__ SmallShared sh;
    extern __shared__ uint64_t fsm[];  // 2 nw words of boundary, then smem_words per warp
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    uint64_t *bx = fsm, *by = fsm + a.nw;
    uint64_t *u = fsm + 2 * a.nw + (size_t)wib * a.smem_words;
    for (int o = blockIdx.x; o < a.nout; o += gridDim.x) {
        __syncthreads();  // the previous output's values are consumed
        for (int w = threadIdx.x; w < a.nw; w += blockDim.x) {
            bx[w] = a.xs[(size_t)o * a.nw + w];
            by[w] = a.ys[(size_t)o * a.nw + w];
        }
        __syncthreads();
        small_output<MINB>(a, o, bx, by, u, sh, lane, wib, wpb);
    }
}

// ------------------------------------------------------------------------------ resident mode
// A one-block kernel that stays on its SM and serves one-boundary evaluations requested through
// mapped pinned host memory: the host writes the boundary, then a new request number; thread 0
// sees it (polling), the block evaluates it with the fused path's code (its instructions and
// the engine's data stay in that SM's caches between requests) and writes the result and a copy
// of the boundary it read, then the request number as done (a release store: the host that
// sees the number sees the rest).  No acquire fence is taken on the request side -- one would
// drop the SM's L1 contents on every request, about a third of the request's device time on a
// d = 7 engine -- so a boundary read ahead of its request number is possible in principle; the
// host compares the copy with what it sent and asks again when they differ.  Every wait is
// bounded: the kernel returns when no request has come for idle_ns nanoseconds, when the host
// sets `stop`, or after max_polls polls, and the host launches it again on its next request.
struct ResidentBox {
    unsigned int req_seq;    // written by the host: number of the latest request
    unsigned int done_seq;   // written by the kernel: number of the latest request served
    int stop;                // written by the host: return now
    int exited;              // written by the kernel on return
    double out[2];           // result of the latest request
    double err;
    int errflag;
    int pad;
    uint64_t words[1];       // nw words of x, nw words of y (the request), then the same 2 nw
                             // words as the kernel read them (allocated to size)
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <int MINB>
__global__ void __launch_bounds__(256, MINB) resident_kernel(KArgs a, ResidentBox *box, unsigned int served,
                                                             unsigned long long idle_ns, unsigned long long max_polls) {
    __shared__ SmallShared sh;
    __shared__ unsigned int s_req;
    __shared__ int s_quit;
    extern __shared__ uint64_t fsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    uint64_t *bx = fsm, *by = fsm + a.nw;
    uint64_t *u = fsm + 2 * a.nw + (size_t)wib * a.smem_words;
    volatile ResidentBox *vb = box;
    unsigned long long polls = 0, t_last = global_ns();
    while (true) {
        if (threadIdx.x == 0) {
            int quit = 0;
            unsigned int r = served;
            while (true) {
                r = vb->req_seq;
                if (r != served) break;
                if (vb->stop) { quit = 1; break; }
                if (++polls >= max_polls || global_ns() - t_last > idle_ns) { quit = 1; break; }
            }
            s_req = r;
            s_quit = quit;
        }
        __syncthreads();
        if (s_quit) break;
        const unsigned int r = s_req;
        for (int w = threadIdx.x; w < a.nw; w += blockDim.x) {
            bx[w] = vb->words[w];
            by[w] = vb->words[a.nw + w];
        }
        if (threadIdx.x == 0) *(volatile int *)a.errflag = 0;  // device memory; copied out below
        __syncthreads();
        small_output<MINB>(a, 0, bx, by, u, sh, lane, wib, wpb);
        if (threadIdx.x == 0) {
            vb->errflag = *(volatile int *)a.errflag;
            for (int w = 0; w < a.nw; w++) {
                vb->words[2 * a.nw + w] = bx[w];
                vb->words[3 * a.nw + w] = by[w];
            }
            // result, flag and boundary copy (this thread's writes) before the request number
            asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(&box->done_seq), "r"(r) : "memory");
            t_last = global_ns();
        }
        served = r;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence_system();
        vb->exited = 1;
    }
}

// ------------------------------------------------------------------------------ Monte Carlo
// Engine::estimate (src/engine.rs:616-659): the mean of c(s) i^{m(s)} over `samples` points s of
// the branch subspace.  Sample k belongs to chunk ci = k / 1024, whose generator is
// Rng::new(seed ^ ci * golden) (src/rng.rs:12-27); its point is the (k mod 1024)-th next_u64 of
// that stream (one word: d <= 64), masked to d bits.  SplitMix64's state after n draws is
// init + n * golden, so every sample's word is computed directly.  FP64 throughout; one
// (sum.re, sum.im, sum |x|^2) partial per block, summed on the host in block order.
__device__ __forceinline__ uint64_t splitmix_at(uint64_t state) {
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) mc_kernel(const EngineDev *__restrict__ Ep, const JobDev *__restrict__ Jp,
                                                 uint64_t seed, long long samples, double *partials) {
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    const EngineDev &E = *Ep;
    const JobDev &J = *Jp;
    __shared__ uint64_t sG[64], sR[64];
    __shared__ uint8_t sLp[64];
    __shared__ double red[3][256];
    for (int j = threadIdx.x; j < E.d; j += blockDim.x) {
        sG[j] = E.G[j];
        sR[j] = E.R[j];
        sLp[j] = J.Lp[j];
    }
    __syncthreads();
    const uint64_t dmask = E.d >= 64 ? ~0ull : ((1ull << E.d) - 1ull);
    const uint64_t lomask = E.DI >= 64 ? ~0ull : ((1ull << E.DI) - 1ull);
    double sx = 0.0, sy = 0.0, sq = 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < samples;
         k += (long long)gridDim.x * blockDim.x) {
        const uint64_t ci = (uint64_t)(k >> 10), kk = (uint64_t)(k & 1023);
        const uint64_t s = to_device_order(E, splitmix_at((seed ^ (ci * golden)) + golden + (kk + 1ull) * golden) & dmask);
        uint32_t m;
        uint64_t yy;
        chunk_start(sLp, sG, sR, J.y0, s, m, yy);
        double2 w = E.tlo64[s & lomask];
        for (int sl = 0; sl < E.nsl_tp; sl++) w = cmul_d(w, E.tp64[sl * 256 + (int)((yy >> (8 * sl)) & 255ull)]);
        w = cmul_d(w, chunk_high_weight(E, s));
        w = rot4d(w, m & 3u);
        sx += w.x;
        sy += w.y;
        sq += w.x * w.x + w.y * w.y;
    }
    red[0][threadIdx.x] = sx;
    red[1][threadIdx.x] = sy;
    red[2][threadIdx.x] = sq;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int q = 0; q < 3; q++) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) partials[3 * blockIdx.x + q] = red[q][0];
}

// Engine::estimate for branch dimensions above 64 (up to 64 * MC_WORDS): the same per-chunk
// streams, each point drawn as ceil(d / 64) consecutive words of its chunk's stream (the
// reference takes a fresh word every 64 coordinates).  Z4 index from the multi-word quadratic
// form (m = sum of Lp_j + 2 q(s), q from popcounts of G rows), pivot bits from R, weight from the
// FP64 byte-slice tables.
constexpr int MC_WORDS = 8;

__device__ __forceinline__ uint32_t bits8_at(const uint64_t *s, int b) {
    const int w = b >> 6, o = b & 63;
    uint64_t v = s[w] >> o;
    if (o > 56 && w + 1 < MC_WORDS) v |= s[w + 1] << (64 - o);
    return (uint32_t)(v & 255ull);
}

__global__ void __launch_bounds__(256) mc_big_kernel(const EngineDev *__restrict__ Ep, const JobDev *__restrict__ Jp,
                                                     const uint8_t *__restrict__ lp, uint64_t seed, long long samples,
                                                     double *partials) {
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    const EngineDev &E = *Ep;
    const JobDev &J = *Jp;
    __shared__ double red[3][256];
    const int d = E.d, nwd = (d + 63) >> 6;
    const uint64_t lomask = E.DI >= 64 ? ~0ull : ((1ull << E.DI) - 1ull);
    double sx = 0.0, sy = 0.0, sq = 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < samples;
         k += (long long)gridDim.x * blockDim.x) {
        const uint64_t ci = (uint64_t)(k >> 10), kk = (uint64_t)(k & 1023);
        const uint64_t st0 = (seed ^ (ci * golden)) + golden;
        uint64_t s[MC_WORDS];
#pragma unroll
        for (int w = 0; w < MC_WORDS; w++) {
            s[w] = 0ull;
            if (w < nwd) {
                uint64_t v = splitmix_at(st0 + (kk * (uint64_t)nwd + (uint64_t)w + 1ull) * golden);
                if (w == nwd - 1 && (d & 63)) v &= (1ull << (d & 63)) - 1ull;
                s[w] = v;
            }
        }
        s[0] = to_device_order(E, s[0]);  // the reordered low coordinates all lie in word 0
        uint32_t m = 0, t = 0;
        uint64_t yy = J.y0;
        for (int w = 0; w < nwd; w++)
            for (uint64_t r = s[w]; r; r &= r - 1) {
                const int j = (w << 6) + ctz64(r);
                m += lp[j];
                const uint64_t *g = E.Gw + (size_t)j * E.dw;
                for (int w2 = 0; w2 < nwd; w2++) t += (uint32_t)popc64(g[w2] & s[w2]);
                yy ^= E.R[j];
            }
        m += ((t >> 1) & 1u) << 1;
        double2 wt = E.tlo64[s[0] & lomask];
        for (int sl = 0; sl < E.nsl_tp; sl++) wt = cmul_d(wt, E.tp64[sl * 256 + (int)((yy >> (8 * sl)) & 255ull)]);
        for (int sl = 0; sl < E.nsl_th; sl++) wt = cmul_d(wt, E.th[sl * 256 + (int)bits8_at(s, E.DI + 8 * sl)]);
        wt = rot4d(wt, m & 3u);
        sx += wt.x;
        sy += wt.y;
        sq += wt.x * wt.x + wt.y * wt.y;
    }
    red[0][threadIdx.x] = sx;
    red[1][threadIdx.x] = sy;
    red[2][threadIdx.x] = sq;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int q = 0; q < 3; q++) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) partials[3 * blockIdx.x + q] = red[q][0];
}

}  // namespace pq
