// pq_host.hpp -- host-side producer for the GB300 amplitude path.
//
// The host compiles a circuit into a path sum, factorises the free Z4 form once by
// symmetric F2 elimination, and derives everything the device kernels need per
// branch engine: packed u64 bitsets (diagonal masks, boundary columns, branch
// columns, kernel columns, the RREF of the radical constraint) plus the two
// GB300-specific tables of this design:
//   * G[j]  -- the Z8 phase of a kernel point is quadratic in the kernel coordinates
//              with every second difference in {0,4}; G[j] holds row j of that
//              (symmetric, zero-diagonal) F2 form, so a Gray step updates the Z8 index
//              with one AND + POPC instead of re-popcounting the odd/plane blocks;
//   * weight tables -- FP64-built, FP32-rounded products of the alpha/beta term
//              weights over byte slices of the kernel and pivot coordinates.
// Reference counterparts: src/pathsum.rs (compiler), src/normal_form.rs (elimination,
// diagonal, columns), src/engine.rs (Engine::new, Elim, Term), src/rank.rs (pairs).
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace pq {

// ---------------------------------------------------------------- bit sets
struct Bits {
    int len = 0;
    std::vector<uint64_t> w;
    Bits() = default;
    explicit Bits(int n) : len(n), w((size_t)((n + 63) / 64), 0ull) {}
    int nw() const { return (int)w.size(); }
    bool get(int i) const { return (w[(size_t)i >> 6] >> (i & 63)) & 1ull; }
    void set(int i, bool v) {
        uint64_t m = 1ull << (i & 63);
        if (v) w[(size_t)i >> 6] |= m; else w[(size_t)i >> 6] &= ~m;
    }
    void flip(int i) { w[(size_t)i >> 6] ^= 1ull << (i & 63); }
    void xor_with(const Bits& o) { for (size_t i = 0; i < w.size(); i++) w[i] ^= o.w[i]; }
    void and_with(const Bits& o) { for (size_t i = 0; i < w.size(); i++) w[i] &= o.w[i]; }
    void clear() { for (auto& x : w) x = 0; }
    unsigned popc() const { unsigned c = 0; for (auto x : w) c += (unsigned)__builtin_popcountll(x); return c; }
    unsigned and_count(const Bits& o) const {
        unsigned c = 0;
        for (size_t i = 0; i < w.size(); i++) c += (unsigned)__builtin_popcountll(w[i] & o.w[i]);
        return c;
    }
    bool dot(const Bits& o) const { return and_count(o) & 1u; }
    int first_one() const {
        for (size_t i = 0; i < w.size(); i++) if (w[i]) return (int)(i * 64) + __builtin_ctzll(w[i]);
        return -1;
    }
    bool operator==(const Bits& o) const { return w == o.w; }
    template <class F> void for_each_one(F&& f) const {
        for (size_t i = 0; i < w.size(); i++) {
            uint64_t x = w[i];
            while (x) { int b = __builtin_ctzll(x); f((int)(i * 64) + b); x &= x - 1; }
        }
    }
    std::vector<int> ones() const { std::vector<int> r; for_each_one([&](int i) { r.push_back(i); }); return r; }
};

// ---------------------------------------------------------------- circuits
enum GateCode : uint8_t { H = 0, X, Y, Z, S, SDG, T, TDG, P, CZ, CX, SWAP, GPHASE, NUM_GATES };
struct Gate { uint8_t op; int a, b; uint32_t ph; };
struct Circuit {
    int nq = 0;
    std::vector<Gate> gates;
    int h_count() const;
    Circuit inverse() const;
};
// Returns an empty string if the description is well formed, else the reason.
std::string validate_circuit(int nq, int ng, const uint8_t* op, const int32_t* q0, const int32_t* q1);

// ---------------------------------------------------------------- path sums
struct PathSum {
    int nq = 0, nv = 0, num_h = 0;
    std::vector<Bits> b;          // nv rows of nv bits, symmetric zero diagonal
    std::vector<uint8_t> v;       // Z4 linear part
    std::vector<uint32_t> theta;  // non-Clifford rotations (ring phase units)
    uint32_t global = 0;
    std::vector<uint8_t> dead;
    std::vector<int> outputs;
    std::vector<uint8_t> out_neg;
    bool zero = false;

    static PathSum compile(const Circuit& c);
    // C then C^dagger; junction[q]/jneg[q] = wire q's variable after C (src/pathsum.rs:304-314)
    static PathSum sandwich(const Circuit& c, std::vector<int>& junction, std::vector<uint8_t>& jneg);
    std::vector<int> io_vars() const;
    void substitute(int a, int b, bool c);
    void trace_closure();
};

// ---------------------------------------------------------------- normal form
struct Structure {
    int m = 0;
    std::vector<Bits> pa, pb, odd, even;  // basis vectors over the m free variables
    // words [first, second) outside which each basis vector is zero (same order as above)
    std::vector<std::pair<int, int>> spa, spb, sodd, seven;
    int g() const { return (int)pa.size(); }
};
Structure eliminate(const std::vector<Bits>& b, const Bits& parity);  // MinWeight rule

struct Diag {
    Bits wa, wb, o1, o3, we;
    int sigma = 0;
};

// Coordinates in the normal-form basis, one packed row: [a | b | o | e] words.
struct Layout {
    int g = 0, nodd = 0, neven = 0;
    int wg = 0, wo = 0, we = 0;
    int full() const { return 2 * wg + wo + we; }  // a|b|o|e
    int abo() const { return 2 * wg + wo; }        // a|b|o (kernel columns have e = 0)
    int off_a() const { return 0; }
    int off_b() const { return wg; }
    int off_o() const { return 2 * wg; }
    int off_e() const { return 2 * wg + wo; }
};

struct Cplx { double re, im; };

// One cached branch engine, fully prepared for upload (src/engine.rs:289-390).
struct HostEngine {
    // sizes
    int nv = 0, nf = 0, m = 0, t = 0, d = 0, rank = 0, ncons = 0;
    Layout L;
    int sigma = 0;
    int mag2 = 0;  // 2*log2|G| = 2g + 2#even + #odd
    int num_h = 0;
    uint32_t global = 0;
    bool zero = false;
    // host data (also used for canonical dumps)
    std::vector<int> fixed, freev, term_vars;
    Structure st;
    Diag dg;
    std::vector<uint64_t> ucols;   // nf * full
    std::vector<uint64_t> mcols;   // t * full
    std::vector<uint64_t> ku;      // d * abo
    std::vector<Bits> kernel;      // d rows of t bits
    std::vector<int> piv_col;      // rank
    std::vector<Bits> piv_row;     // rank rows of #even bits
    std::vector<Bits> cons;        // ncons rows of #even bits
    std::vector<uint64_t> bfixed;  // nf * wf
    int wf = 0;
    std::vector<uint8_t> fixed_v;
    std::vector<uint32_t> fixed_th;
    std::vector<Cplx> alpha, beta;  // per term, FP64 (src/engine.rs:232-238)
    // device plan
    std::vector<uint64_t> G;        // d rows, quadratic part of the Z8 phase over kernel coordinates
    std::vector<uint64_t> Gw;       // the same, d rows of dw words (any d)
    std::vector<uint8_t> lp0;       // d: parity of each coordinate's Z4 increment (any boundary)
    int dw = 1;
    std::vector<uint64_t> R;        // d pivot masks (bit i: kernel_j hits pivot column i)
    std::vector<int> free_col;      // d: term index of kernel vector j's free column
    double sum_abs_bound = 0.0;     // upper bound of sum_s |c(s)| (for the per-result error bound)
    int dev_DI = -1;                // walked (low) coordinates chosen by device_order (-1: not set)

    // Z8 index of the Gauss sum for coordinates u (src/normal_form.rs:479-493)
    int phase8(const uint64_t* u_abo) const;
};

// Engine build (src/engine.rs:289-390); `fixed` = fixed variables in evaluation order.
std::unique_ptr<HostEngine> build_engine(const PathSum& ps, const std::vector<int>& fixed);

// Strategy layer (src/rank.rs:62-222, src/sim.rs:65-71)
enum Strategy { STRAT_AUTO = 0, STRAT_CACHED = 1, STRAT_PAIRS = 2 };
struct RankSet {
    int pairs = 0;
    std::vector<std::unique_ptr<HostEngine>> branches;
};
RankSet build_rank(const PathSum& ps, const std::vector<int>& fixed, int strategy, int pairs);
int best_pairs(const HostEngine& base, int available, int tclass);
// Substitution pairs (src/rank.rs:62-84): T-class pairs first; ntclass = their count.
std::vector<std::pair<int, int>> pair_candidates(const PathSum& ps, const std::vector<int>& fixed, int& ntclass);
// The branch engine of one pattern of the first p pairs (bit i: the value substituted for pair
// i), built from a copy of ps (src/approx.rs:112-117).
std::unique_ptr<HostEngine> pattern_engine(const PathSum& ps, const std::vector<int>& fixed,
                                           const std::vector<std::pair<int, int>>& cands, int p, uint64_t pattern);

// Weight tables of one branch engine (FP64; the device also keeps FP32 roundings):
//   tlo[s]  = prod_{j < DI} a_{free(j)}[s_j]                 s < 2^DI, DI = min(d, di_max)
//   tp[b]   = prod_{k < 8} a_{piv(8 sl + k)}[b_k]              per slice sl of the pivot bits
//   th[b]   = prod_{k < 8} a_{free(DI + 8 sl + k)}[b_k]        per slice sl of the coordinates >= DI
//   w[(y << DI) | s] = tlo[s] * prod_i a_{piv(i)}[y_i]         joint table when #pivots <= kJointMaxPivots
//                       (FP64 products; the device stores them as FP32 hi + lo pairs)
static const int kJointMaxPivots = 10;
static const int kJointMaxBits = 13;  // DI + #pivots of the joint table
//   An engine with more than kJointMaxPivots pivots gets a joint table over only the pivots its
//   DI low coordinates touch (pmask, plo of them; device_order picks low coordinates that touch
//   few): w[(ylo << DI) | s] over those pivots, and thp[b] = the other pivots' weights per byte
//   slice of y, a per-chunk FP64 factor (the walked coordinates do not change those pivots).
struct EngineTables {
    int DI = 0, nsl_tp = 0, nsl_th = 0;
    bool joint = false;
    bool partial = false;       // the joint table covers the pivots in pmask only
    int plo = 0;
    uint64_t pmask = 0;
    std::vector<Cplx> tlo, tp, th, w, thp;
    std::vector<uint64_t> Rc;   // d: R_j compressed to the bits of pmask (j < DI), else R_j
};
EngineTables build_tables(const HostEngine& e, int di_max);

// One engine packed into a single blob: EngineDev pointers hold byte offsets into the
// blob until rebased onto the blob's device (or host) address.
}  // namespace pq
#include "pq_core.cuh"
namespace pq {
struct PackedEngine {
    std::vector<uint8_t> blob;
    EngineDev off;              // pointers are offsets into blob, except wtab (null: placed apart)
    std::vector<float> wtab;    // the joint weight table (4 floats per entry), uploaded apart
};
PackedEngine pack_engine(const HostEngine& e, const EngineTables& t);
// Copy of e with its coordinates reordered for the device (see pq_host.cpp) and its low
// (walked) coordinate count set in dev_DI; perm[j] is the reference coordinate of device
// coordinate j.
HostEngine device_order(const HostEngine& e, int di_max, std::vector<int>& perm);
EngineDev rebase_engine(const EngineDev& off, const uint8_t* base);

// Boundary map: `puts` lists (variable, boundary source) in the order the reference's
// `put` sees them (src/pathsum.rs:430-450, src/sim.rs:105-124).  The first occurrence of a
// variable fixes its position; a repeated variable becomes a consistency check.
struct IoMapHost {
    std::vector<int> fixed;      // variables in position order
    std::vector<int32_t> src;    // per position
    std::vector<int32_t> cf_pos, cf_src;
};
inline int32_t io_src(int q, int vec, int flip) { return (int32_t)(q | (vec << 24) | (flip << 25)); }
IoMapHost build_iomap(const std::vector<std::pair<int, int32_t>>& puts);

// Canonical dump of an engine, word-for-word the oracle's layout.
std::vector<uint64_t> engine_dump(const HostEngine& e);

}  // namespace pq
