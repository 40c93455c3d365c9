// pq_core.cuh -- data layout in HBM and the per-branch arithmetic of the enumeration.
//
// Everything here is plain-old-data plus __host__ __device__ helpers: the kernels in
// pq_device.cu call them per lane, with (start, stride) = (lane, 32).
//
// Arithmetic of one branch engine (reference: src/engine.rs:557-722, normal_form.rs:479-493):
//   amplitude = e^{i phase} * 2^{(mag2 - num_h)/2} * sum_{s in F2^d} c(s) * w8^{k8(s)}
//   * k8(s) is the Z8 Gauss-sum index of kernel point s.  Its second differences along
//     kernel columns are 4*G_ij (boundary independent), so
//         k8(s) = k0 + 2 * ( sum_j s_j Lp_j + 2 * sum_{i<j} G_ij s_i s_j )   (mod 8)
//     with k0 = phase8(u_start) and 2*Lp_j = phase8(u_start ^ kernel_u_j) - k0.  The parity
//     of k8 is the parity of #odd lines for every branch, so the walk tracks the Z4 index
//     m = (k8 - k0)/2: a Gray step on coordinate j adds +-Lp_j + 2*parity(G_j & s).
//   * c(s) = prod_k a_k[sv_k] over the t terms.  The free column of kernel vector j carries
//     bit s_j; pivot column i carries bit y_i = y0_i ^ parity(R . s) (R_j = pivot mask of
//     kernel vector j).  Hence c(s) = W[y, s & lomask] * CHI(s >> DI): W is the FP64 product of
//     the first DI coordinates' weights and the pivot weights, stored as an FP32 hi/lo pair;
//     CHI is the FP64 product over byte slices of the coordinates >= DI (once per chunk).
//     hi lies on an exact power-of-two grid, so its chunk sums are exact in FP32 in any
//     order and under quarter turns; lo = W - hi is summed in plain FP32, so the per-branch
//     rounding left is that of the small lo parts.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PQ_HD __host__ __device__ __forceinline__
#else
#define PQ_HD inline
#endif

namespace pq {

#if !defined(__CUDACC__)
struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
struct double2 { double x, y; };
#endif

static const int kMaxD = 62;        // kernel coordinates fit a u64 with room for shifts
static const int kMaxPivots = 64;   // pivot coordinates y fit a u64

// One branch engine resident in HBM (built once per circuit and strategy branch).
struct EngineDev {
    int nf, t, d, rank, ncons;
    int wg, wo, we, wf, W, abo;     // word counts; W = 2wg+wo+we, abo = 2wg+wo
    int sigma, mag2, num_h;
    uint32_t global;
    int zero;
    int DI, nsl_tp, nsl_th;
    int joint;               // 1: weights from the joint hi/lo table; 0: FP64 product path
    int plo;                 // pivots indexed by the joint table (all of them, or those the
    uint64_t pmask;          // walked coordinates touch: bits pmask of the pivot bits y)
    uint8_t cperm[64];       // reference coordinate of device coordinate j (j < min(d, 64))
    int npairc;              // pair coordinates: the lowest (<= 3) coordinates >= DI with R = 0
    int pairc[3];            // (flipping one keeps every table index): chunks that differ only
                             // in them are walked together
    double sum_abs_bound;
    double grid;             // hi parts of wtab are integer multiples of this power of two
    double errfac;           // bound on a job's FP32 lo-sum error (before the 2^{(mag2-h)/2} scale)
    const uint64_t *o1, *o3, *wa, *wb, *wem;  // diagonal masks
    const uint64_t *ucols;   // nf x W   boundary columns  [a|b|o|e]
    const uint64_t *mcols;   // t  x W   term columns      [a|b|o|e]
    const uint64_t *ku;      // d  x abo kernel columns    [a|b|o]
    const uint64_t *bfixed;  // nf x wf  adjacency among fixed variables
    const uint8_t *fixed_v;
    const uint32_t *fixed_th;
    const uint64_t *pivrow;  // rank x we  RREF row operations of the pivots
    const uint64_t *cons;    // ncons x we consistency rows
    const int32_t *pivcol;   // rank
    const uint64_t *G;       // d   quadratic form of the Z8 phase over kernel coordinates
    const uint64_t *Gw;      // d x dw  the same for any d (Monte-Carlo sampling above 64)
    int dw;
    const uint64_t *R;       // d   pivot masks
    const uint64_t *Rc;      // d   pivot masks of the walked coordinates in the joint table's
                             //     pivot index (R compressed to the bits of pmask)
    const float2 *tlo;       // 2^DI
    const float2 *tp;        // nsl_tp x 256
    const double2 *th;       // nsl_th x 256
    const double2 *thp;      // nsl_tp x 256: weights of the pivots outside pmask (null: none), a
                             // per-unit FP64 factor of an engine whose table covers only some pivots
    const double2 *thr;      // nsl_th x 256: th with the pair coordinates' factors left out
    const float4 *pf;        // 2^npairc: the pair coordinates' weight for each pattern of their
                             // bits, as FP32 pairs (re hi, im hi, re lo, im lo), hi + lo = FP64
    const double2 *tlo64;    // 2^DI   (FP64 path)
    const double2 *tp64;     // nsl_tp x 256
    const float4 *wtab;      // 2^(DI + plo): (hi.re, hi.im, lo.re, lo.im) of tlo[s] * TP(y) over
                             // the pivots in pmask
    const double2 *ctab;     // 2^(rank + DI) chunk sums (null: none), index (y << DI) | b
};

// Boundary -> fixed-variable values.  src = q | vec << 24 | flip << 25 (vec 0: x, 1: y).
struct IoMapDev {
    int nf, ncf;
    const int32_t *src;     // nf
    const int32_t *cf_pos;  // ncf: fixed position that must equal ...
    const int32_t *cf_src;  // ... this boundary bit
};

// One (engine, boundary) evaluation.  Static fields are set on the host; the rest is
// written by the prepare kernel.
struct JobDev {
    int engine, iomap, req, out;
    int vanish;
    uint32_t phase;  // e^{i 2 pi phase / 2^32} (fixed-variable constants + global phase)
    uint32_t k0;     // Z8 index at s = 0
    uint32_t err;
    uint64_t y0;     // pivot bits at s = 0
    uint8_t Lp[64];  // Z4 linear coefficients (index units of pi/2)
};

// A contiguous range of chunks of one job, processed by one warp.
struct ItemDev {
    int job;
    int dl;          // Gray steps per chunk = 2^dl
    uint32_t nch;    // chunks in this item
    uint32_t pad;
    uint64_t ch0;    // first chunk index; chunk c covers s = (c << dl) + [0, 2^dl)
};

// ---------------------------------------------------------------- helpers
PQ_HD int popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}
PQ_HD int ctz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __ffs((int)x) - 1;
#else
    return __builtin_ctz(x);
#endif
}
PQ_HD int ctz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}
PQ_HD int src_bit(int32_t src, const uint64_t *x, const uint64_t *y) {
    int q = src & 0xFFFFFF;
    const uint64_t *v = ((src >> 24) & 1) ? y : x;
    return (int)((v[q >> 6] >> (q & 63)) & 1ull) ^ ((src >> 25) & 1);
}
PQ_HD int bit_at(const uint64_t *v, int i) { return (int)((v[i >> 6] >> (i & 63)) & 1ull); }

// Multiply the hi and lo parts of a weight by i^q (q in 0..3) exactly.
PQ_HD float4 rot4q(float4 w, uint32_t q) {
    const bool sw = q & 1;
    float a = sw ? w.y : w.x, b = sw ? w.x : w.y;
    float c = sw ? w.w : w.z, d = sw ? w.z : w.w;
    const bool na = (q == 1 || q == 2), nb = (q >= 2);
    float4 r;
    r.x = na ? -a : a;
    r.y = nb ? -b : b;
    r.z = na ? -c : c;
    r.w = nb ? -d : d;
    return r;
}

// Multiply by i^q (q in 0..3) exactly.
PQ_HD double2 rot4d(double2 w, uint32_t q) {
    double a = (q & 1) ? w.y : w.x;
    double b = (q & 1) ? w.x : w.y;
    double2 r;
    r.x = (q == 1 || q == 2) ? -a : a;
    r.y = (q >= 2) ? -b : b;
    return r;
}
PQ_HD double2 cmul_d(double2 a, double2 b) {
    double2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
PQ_HD float2 cmul_f(float2 a, float2 b) {
    float2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// Z8 Gauss-sum index for coordinates u (+ optional kernel column k), over word range
// [w0, ...) with stride ws: returns the partial (n1 = popc(o&o1)-popc(o&o3), cnt = plane count).
PQ_HD void phase8_partial(const EngineDev &E, const uint64_t *u, const uint64_t *k, int w0, int ws, int &n1,
                          int &cnt) {
    const int ob = 2 * E.wg;
    for (int w = w0; w < E.wo; w += ws) {
        uint64_t uo = u[ob + w] ^ (k ? k[ob + w] : 0ull);
        n1 += popc64(uo & E.o1[w]) - popc64(uo & E.o3[w]);
    }
    for (int w = w0; w < E.wg; w += ws) {
        uint64_t ua = u[w] ^ (k ? k[w] : 0ull);
        uint64_t ub = u[E.wg + w] ^ (k ? k[E.wg + w] : 0ull);
        cnt += popc64((E.wa[w] ^ ua) & (E.wb[w] ^ ub));
    }
}
PQ_HD uint32_t phase8_finish(const EngineDev &E, int n1, int cnt) {
    int n = E.sigma - 2 * n1 + ((cnt & 1) ? 4 : 0);
    return (uint32_t)(((n % 8) + 8) % 8);
}

// Fixed-variable constants (src/engine.rs:575-588) over fixed positions [i0, nf) step is:
// z4 sum and theta sum (both to be summed over the partial ranges).
PQ_HD void fixed_constants_partial(const EngineDev &E, const uint64_t *vals, int i0, int is, uint32_t &z4,
                                   uint32_t &th) {
    for (int i = i0; i < E.nf; i += is) {
        if (!bit_at(vals, i)) continue;
        z4 += E.fixed_v[i];
        th += E.fixed_th[i];
        int cnt = 0;
        int wi = i >> 6;
        for (int w = wi; w < E.wf; w++) {
            uint64_t m = E.bfixed[(size_t)i * E.wf + w] & vals[w];
            if (w == wi) m &= ((i & 63) == 63) ? 0ull : (~0ull << ((i & 63) + 1));
            cnt += popc64(m);
        }
        z4 += 2u * (uint32_t)cnt;
    }
}

// u0 = xor of the boundary columns of the fixed variables set to 1, words [w0, W) step ws.
PQ_HD void boundary_shift_partial(const EngineDev &E, const uint64_t *vals, uint64_t *u, int w0, int ws) {
    const int nvw = (E.nf + 63) >> 6;
    for (int w = w0; w < E.W; w += ws) {
        uint64_t acc = 0;
        for (int vw = 0; vw < nvw; vw++)  // only the fixed variables set to 1
            for (uint64_t r = vals[vw]; r; r &= r - 1)
                acc ^= E.ucols[(size_t)((vw << 6) + ctz64(r)) * E.W + w];
        u[w] = acc;
    }
}

// parity of <row, kappa> where kappa = we ^ u.e
PQ_HD int kappa_dot(const EngineDev &E, const uint64_t *row, const uint64_t *u) {
    const int eb = 2 * E.wg + E.wo;
    int p = 0;
    for (int w = 0; w < E.we; w++) p ^= popc64(row[w] & (E.wem[w] ^ u[eb + w])) & 1;
    return p;
}

// u ^= mcols[pivcol[i]] for pivots i set in y0, words [w0, W) step ws
PQ_HD void apply_pivots_partial(const EngineDev &E, uint64_t y0, uint64_t *u, int w0, int ws) {
    for (int w = w0; w < E.W; w += ws) {
        uint64_t acc = u[w];
        for (uint64_t r = y0; r; r &= r - 1) acc ^= E.mcols[(size_t)E.pivcol[ctz64(r)] * E.W + w];
        u[w] = acc;
    }
}

// Magnitude 2^{e/2} for an integer e (exact power of two times sqrt(2) when e is odd).
PQ_HD double pow2_half(int e) {
    int h = (e >= 0) ? e / 2 : -((-e + 1) / 2);  // floor(e/2)
    double r = 1.0;
    if (h > 0) for (int i = 0; i < h; i++) r *= 2.0;
    else for (int i = 0; i < -h; i++) r *= 0.5;
    if (e - 2 * h) r *= 1.41421356237309504880;
    return r;
}

// Work shape of one job: chunks of 2^dl Gray steps (dl = min(d - 5, DI)), grouped into units --
// one chunk, or, when the engine has pair coordinates and the joint table applies, the 2^np
// chunks that differ in its first np pair coordinates (np <= log2(unit_max)): they read the
// same table entry at every step -- and cpi units per work item (at most 2^16 items per job,
// so partial buffers stay bounded).  jdl packs dl (bits 0-7) and np (bits 8-9).
PQ_HD void job_shape(const EngineDev &E, int cpl, int unit_max, int &jdl, unsigned long long &nunits, unsigned &cpi) {
    const int d = E.d;
    const int dl = d <= 5 ? 0 : (d - 5 < E.DI ? d - 5 : E.DI);
    unsigned long long n = 1ull << (d - dl);
    int np = 0;
    if (E.joint && dl >= 3)
        while (np < E.npairc && (2 << np) <= unit_max && n >= 2) {
            n >>= 1;
            np++;
        }
    unsigned long long per = 32ull * (unsigned long long)cpl;
    while ((n + per - 1) / per > (1ull << 16)) per *= 2;
    jdl = dl | (np << 8);
    nunits = n;
    cpi = (unsigned)(n < per ? n : per);
}

// Index with a zero bit inserted at position b.
PQ_HD unsigned long long insert_zero(unsigned long long x, int b) {
    return ((x >> b) << (b + 1)) | (x & ((1ull << b) - 1ull));
}

// A point of the branch subspace in the reference's coordinates, in the device's order (the
// coordinates are reordered when the engine is packed; only within the first 64, which holds the
// reordering of every engine).
PQ_HD uint64_t to_device_order(const EngineDev &E, uint64_t s_ref) {
    const int n = E.d < 64 ? E.d : 64;
    const uint64_t mask = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
    uint64_t s = s_ref & ~mask;
    for (int j = 0; j < n; j++) s |= ((s_ref >> E.cperm[j]) & 1ull) << j;
    return s;
}

// The joint table's pivot index of pivot bits y: y itself, or its bits at pmask packed down.
PQ_HD uint64_t joint_pivots(const EngineDev &E, uint64_t y) {
    if (!E.thp) return y;
    uint64_t r = 0;
    int k = 0;
    for (uint64_t m = E.pmask; m; m &= m - 1, k++) r |= ((y >> ctz64(m)) & 1ull) << k;
    return r;
}

// FP64 weight of the pivots outside the joint table's index at pivot bits y ((1, 0) if none).
PQ_HD double2 high_pivot_weight(const EngineDev &E, uint64_t y) {
    double2 c;
    c.x = 1.0;
    c.y = 0.0;
    if (!E.thp) return c;
    for (int sl = 0; sl < E.nsl_tp; sl++) c = cmul_d(c, E.thp[sl * 256 + (int)((y >> (8 * sl)) & 255ull)]);
    return c;
}

// Chunk start: Z4 index m and pivot bits y at kernel point s (bits in ascending order).
PQ_HD void chunk_start(const uint8_t *Lp, const uint64_t *G, const uint64_t *R, uint64_t y0, uint64_t s,
                       uint32_t &m, uint64_t &y) {
    uint32_t mm = 0;
    uint64_t yy = y0, pre = 0;
    for (uint64_t x = s; x; x &= x - 1) {
        int j = ctz64(x);
        mm += Lp[j] + 2u * (uint32_t)(popc64(G[j] & pre) & 1);
        pre |= 1ull << j;
        yy ^= R[j];
    }
    m = mm;
    y = yy;
}

// FP64 weight of the coordinates above DI.
PQ_HD double2 chunk_high_weight(const EngineDev &E, uint64_t s) {
    double2 c;
    c.x = 1.0;
    c.y = 0.0;
    for (int sl = 0; sl < E.nsl_th; sl++) c = cmul_d(c, E.th[sl * 256 + (int)((s >> (E.DI + 8 * sl)) & 255ull)]);
    return c;
}

// FP64 weight of the coordinates above DI other than the pair coordinates.
PQ_HD double2 chunk_rest_weight(const EngineDev &E, uint64_t s) {
    double2 c;
    c.x = 1.0;
    c.y = 0.0;
    if (E.nsl_th == 0) return c;
    c = E.thr[(int)((s >> E.DI) & 255ull)];
    for (int sl = 1; sl < E.nsl_th; sl++) c = cmul_d(c, E.thr[sl * 256 + (int)((s >> (E.DI + 8 * sl)) & 255ull)]);
    return c;
}

}  // namespace pq
