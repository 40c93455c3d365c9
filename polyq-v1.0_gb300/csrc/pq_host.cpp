// pq_host.cpp -- circuit compiler, symmetric F2 elimination and branch-engine build.
// See pq_host.hpp for the role of each structure; every function names the reference
// function whose semantics it keeps.
#include "pq_host.hpp"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <cmath>
#include <map>
#include <set>
#include <stdexcept>
#include <thread>

namespace pq {

static inline int words_of(int n) { return (n + 63) / 64; }

// ---------------------------------------------------------------- phase ring (src/phase.rs)
static const double kRootHalf = 0.70710678118654752440;
static Cplx root8(int k) {
    static const Cplx R[8] = {{1, 0}, {kRootHalf, kRootHalf}, {0, 1}, {-kRootHalf, kRootHalf},
                              {-1, 0}, {-kRootHalf, -kRootHalf}, {0, -1}, {kRootHalf, -kRootHalf}};
    return R[k & 7];
}
static Cplx phase_complex(uint32_t p) {  // src/phase.rs:60-66
    if ((p & ((1u << 29) - 1)) == 0) return root8((int)(p >> 29));
    double th = 2.0 * M_PI * (double)p / 4294967296.0;
    return {std::cos(th), std::sin(th)};
}
static int clifford_level(uint32_t p) { return (p & ((1u << 30) - 1)) == 0 ? (int)(p >> 30) : -1; }
static inline uint32_t z4_phase(unsigned k) { return (uint32_t)(k & 3u) << 30; }

// ---------------------------------------------------------------- circuits (src/circuit.rs)
int Circuit::h_count() const {
    int h = 0;
    for (const auto& g : gates) h += g.op == H ? 1 : (g.op == CX ? 2 : 0);
    return h;
}
Circuit Circuit::inverse() const {  // src/circuit.rs:46-56, :189-191
    Circuit r;
    r.nq = nq;
    for (auto it = gates.rbegin(); it != gates.rend(); ++it) {
        Gate g = *it;
        switch (g.op) {
            case S: g.op = SDG; break;
            case SDG: g.op = S; break;
            case T: g.op = TDG; break;
            case TDG: g.op = T; break;
            case P: case GPHASE: g.ph = 0u - g.ph; break;
            default: break;
        }
        r.gates.push_back(g);
    }
    return r;
}
std::string validate_circuit(int nq, int ng, const uint8_t* op, const int32_t* q0, const int32_t* q1) {
    if (nq < 0 || ng < 0) return "negative size";
    if (ng > 0 && (!op || !q0 || !q1)) return "null gate array";
    for (int i = 0; i < ng; i++) {
        if (op[i] >= NUM_GATES) return "unknown gate code at index " + std::to_string(i);
        if (op[i] == GPHASE) continue;
        if (q0[i] < 0 || q0[i] >= nq) return "qubit out of range at gate " + std::to_string(i);
        if (op[i] == CZ || op[i] == CX || op[i] == SWAP) {
            if (q1[i] < 0 || q1[i] >= nq) return "qubit out of range at gate " + std::to_string(i);
            if (q1[i] == q0[i]) return "two-qubit gate on one wire at gate " + std::to_string(i);
        }
    }
    return "";
}

// ---------------------------------------------------------------- compiler (src/pathsum.rs:100-324)
namespace {
struct Compiler {
    int n, nvars, num_h = 0, cap;
    std::vector<int> wire;
    std::vector<uint8_t> neg;
    std::vector<Bits> adj;
    std::vector<uint8_t> v;
    std::vector<uint32_t> theta;
    uint32_t global = 0;

    Compiler(int nq, int extra) : n(nq), nvars(nq), cap(std::max(1, nq + extra)), wire(nq), neg(nq, 0) {
        for (int i = 0; i < nq; i++) wire[i] = i;
        adj.assign((size_t)cap, Bits(cap));
        v.assign((size_t)cap, 0);
        theta.assign((size_t)cap, 0);
    }
    int new_var() {
        if (nvars == cap) {  // capacity is only a hint (pathsum.rs:120-129)
            int nc = std::max(cap * 2, 8);
            std::vector<Bits> na((size_t)nc, Bits(nc));
            for (int i = 0; i < cap; i++) std::copy(adj[i].w.begin(), adj[i].w.end(), na[i].w.begin());
            adj.swap(na);
            v.resize((size_t)nc, 0);
            theta.resize((size_t)nc, 0);
            cap = nc;
        }
        v[nvars] = 0;
        theta[nvars] = 0;
        return nvars++;
    }
    void flip_sym(int i, int j) { adj[i].flip(j); adj[j].flip(i); }
    void add_v(int z, unsigned k) { v[z] = (uint8_t)((v[z] + k) & 3u); }
    void rotate(int q, uint32_t th) {  // pathsum.rs:215-224
        int z = wire[q];
        if (neg[q]) { theta[z] -= th; global += th; }
        else theta[z] += th;
    }
    void apply(const Gate& g) {  // pathsum.rs:136-213
        int q = g.a;
        switch (g.op) {
            case H: {
                int z = wire[q], zp = new_var();
                flip_sym(z, zp);
                num_h++;
                if (neg[q]) { add_v(zp, 2); neg[q] = 0; }
                wire[q] = zp;
            } break;
            case X: neg[q] ^= 1; break;
            case Z: add_v(wire[q], 2); if (neg[q]) global += 1u << 31; break;
            case S:
                if (neg[q]) { add_v(wire[q], 3); global += 1u << 30; } else add_v(wire[q], 1);
                break;
            case SDG:
                if (neg[q]) { add_v(wire[q], 1); global -= 1u << 30; } else add_v(wire[q], 3);
                break;
            case T: rotate(q, 1u << 29); break;
            case TDG: rotate(q, 0u - (1u << 29)); break;
            case P: rotate(q, g.ph); break;
            case Y: apply(Gate{Z, q, 0, 0}); apply(Gate{X, q, 0, 0}); global += 1u << 30; break;
            case CZ: {
                int a = g.a, b = g.b, za = wire[a], zb = wire[b];
                flip_sym(za, zb);
                if (neg[b]) add_v(za, 2);
                if (neg[a]) add_v(zb, 2);
                if (neg[a] && neg[b]) global += 1u << 31;
            } break;
            case CX:
                apply(Gate{H, g.b, 0, 0});
                apply(Gate{CZ, g.a, g.b, 0});
                apply(Gate{H, g.b, 0, 0});
                break;
            case SWAP: std::swap(wire[g.a], wire[g.b]); std::swap(neg[g.a], neg[g.b]); break;
            case GPHASE: global += g.ph; break;
        }
    }
    PathSum snapshot() const {  // pathsum.rs:236-261
        PathSum p;
        int nv = nvars;
        p.nq = n; p.nv = nv; p.num_h = num_h;
        p.b.assign((size_t)nv, Bits(nv));
        for (int i = 0; i < nv; i++) {
            for (int wi = 0; wi < p.b[i].nw(); wi++) p.b[i].w[wi] = adj[i].w[wi];
            if (nv & 63) p.b[i].w.back() &= (1ull << (nv & 63)) - 1;  // columns >= nv are never set
        }
        p.v.assign(v.begin(), v.begin() + nv);
        p.theta.assign(theta.begin(), theta.begin() + nv);
        p.global = global;
        p.dead.assign((size_t)nv, 0);
        p.outputs = wire;
        p.out_neg = neg;
        for (int k = 0; k < nv; k++) {  // normalize: pathsum.rs:317-324
            int l = clifford_level(p.theta[k]);
            if (l >= 0) { p.v[k] = (uint8_t)((p.v[k] + l) & 3); p.theta[k] = 0; }
        }
        return p;
    }
};
}  // namespace

PathSum PathSum::compile(const Circuit& c) {
    Compiler comp(c.nq, c.h_count());
    for (const auto& g : c.gates) comp.apply(g);
    return comp.snapshot();
}
PathSum PathSum::sandwich(const Circuit& c, std::vector<int>& junction, std::vector<uint8_t>& jneg) {
    Compiler comp(c.nq, 2 * c.h_count());
    for (const auto& g : c.gates) comp.apply(g);
    junction = comp.wire;
    jneg = comp.neg;
    Circuit inv = c.inverse();
    for (const auto& g : inv.gates) comp.apply(g);
    return comp.snapshot();
}
std::vector<int> PathSum::io_vars() const {  // pathsum.rs:328-336
    std::vector<int> f;
    for (int q = 0; q < nq; q++) f.push_back(q);
    for (int q = 0; q < nq; q++)
        if (std::find(f.begin(), f.end(), outputs[q]) == f.end()) f.push_back(outputs[q]);
    return f;
}
void PathSum::substitute(int a, int bb, bool c) {  // pathsum.rs:360-394
    bool bab = b[a].get(bb);
    uint32_t ta = theta[a], tb = theta[bb];
    uint8_t vb = v[bb];
    Bits nb = b[bb];
    nb.set(a, false);
    if (!c) {
        v[a] = (uint8_t)((v[a] + vb + 2 * (int)bab) & 3);
        theta[a] = ta + tb;
    } else {
        v[a] = (uint8_t)((v[a] + 4 - vb) & 3);
        theta[a] = ta - tb;
        global += z4_phase(vb) + tb;
        nb.for_each_one([&](int k) { v[k] = (uint8_t)((v[k] + 2) & 3); });
    }
    nb.for_each_one([&](int k) { b[a].flip(k); b[k].flip(a); });
    b[bb].for_each_one([&](int k) { b[k].set(bb, false); });
    b[bb].clear();
    v[bb] = 0;
    theta[bb] = 0;
    dead[bb] = 1;
    int l = clifford_level(theta[a]);
    if (l >= 0) { v[a] = (uint8_t)((v[a] + l) & 3); theta[a] = 0; }
}
void PathSum::trace_closure() {  // pathsum.rs:399-425
    std::vector<int> rep((size_t)nv);
    std::vector<uint8_t> par((size_t)nv, 0);
    for (int i = 0; i < nv; i++) rep[i] = i;
    for (int q = 0; q < nq; q++) {
        int ra = q, pa = 0, rb = outputs[q], pb = 0;
        while (rep[ra] != ra) { pa ^= par[ra]; ra = rep[ra]; }
        while (rep[rb] != rb) { pb ^= par[rb]; rb = rep[rb]; }
        int c = pa ^ pb ^ out_neg[q];
        if (ra == rb) { if (c) zero = true; continue; }
        substitute(ra, rb, c);
        rep[rb] = ra;
        par[rb] = (uint8_t)c;
    }
}

// ---------------------------------------------------------------- elimination (src/normal_form.rs:58-336)
// Symmetric LDL^T over F2 with the MinWeight pivot rule: the lightest alive row with a
// diagonal bit is a 1x1 pivot; otherwise the lightest row with an off-diagonal bit is a
// 2x2 pivot with its lowest alive neighbour.  Ties break on the row index.
// Rows are kept with the span of words that may hold set bits, so that the row operations
// of a step cost the span of the vectors involved, not the full width m/64 (the quadratic
// forms of circuits are local: a variable meets few others, and those were created near it).
// The pivot queues hold each variable once under its current key and yield the minimum
// (weight, index), the MinWeight rule's choice.
namespace {
struct SpanRows {
    int W = 0;
    std::vector<uint64_t> w;
    std::vector<int> lo, hi;  // [lo, hi) words that may be nonzero
    SpanRows(int m, int words) : W(words), w((size_t)m * words, 0ull), lo((size_t)m, 0), hi((size_t)m, 0) {}
    uint64_t* row(int i) { return &w[(size_t)i * W]; }
    const uint64_t* row(int i) const { return &w[(size_t)i * W]; }
    void set(int i, int bit) {
        row(i)[bit >> 6] |= 1ull << (bit & 63);
        widen(i, bit >> 6, (bit >> 6) + 1);
    }
    void widen(int i, int a, int b) {
        if (lo[i] == hi[i]) { lo[i] = a; hi[i] = b; return; }
        lo[i] = std::min(lo[i], a);
        hi[i] = std::max(hi[i], b);
    }
    void xor_in(int i, const uint64_t* v, int a, int b) {
        if (a >= b) return;
        uint64_t* r = row(i);
        for (int k = a; k < b; k++) r[k] ^= v[k];
        widen(i, a, b);
    }
    Bits bits(int i, int len) const {
        Bits o(len);
        std::copy(row(i) + lo[i], row(i) + hi[i], o.w.begin() + lo[i]);
        return o;
    }
};
// Pivot queue of one class: the variables keyed by (weight, index), minimum first.  Weights
// below 64 live in per-weight bitsets (with a count and a lowest-word hint), the rest in an
// ordered set; the minimum is the lowest index of the lightest non-empty weight.
struct PivotQueue {
    static const int kB = 64;
    int W;
    std::vector<uint64_t> bits;  // kB x W
    int cnt[kB];
    int hint[kB];                // no bit below this word
    std::set<std::pair<uint32_t, int>> big;
    explicit PivotQueue(int words) : W(words), bits((size_t)kB * words, 0ull) {
        for (int w = 0; w < kB; w++) { cnt[w] = 0; hint[w] = words; }
    }
    void add(uint32_t w, int a) {
        if (w >= (uint32_t)kB) { big.insert({w, a}); return; }
        bits[(size_t)w * W + (a >> 6)] |= 1ull << (a & 63);
        cnt[w]++;
        hint[w] = std::min(hint[w], a >> 6);
    }
    void del(uint32_t w, int a) {
        if (w >= (uint32_t)kB) { big.erase({w, a}); return; }
        bits[(size_t)w * W + (a >> 6)] &= ~(1ull << (a & 63));
        cnt[w]--;
    }
    int min() {
        for (int w = 0; w < kB; w++) {
            if (!cnt[w]) continue;
            const uint64_t* b = &bits[(size_t)w * W];
            for (int q = hint[w]; q < W; q++)
                if (b[q]) { hint[w] = q; return q * 64 + __builtin_ctzll(b[q]); }
        }
        return big.empty() ? -1 : big.begin()->second;
    }
};
// A scratch vector with its word span; cleared over that span.
struct SpanVec {
    std::vector<uint64_t> w;
    int lo = 0, hi = 0;
    explicit SpanVec(int words) : w((size_t)words, 0ull) {}
    void clear() {
        for (int k = lo; k < hi; k++) w[k] = 0;
        lo = hi = 0;
    }
    void trim() {
        while (lo < hi && w[lo] == 0) lo++;
        while (hi > lo && w[hi - 1] == 0) hi--;
    }
    bool get(int i) const { return (w[(size_t)i >> 6] >> (i & 63)) & 1ull; }
    void unset(int i) { w[(size_t)i >> 6] &= ~(1ull << (i & 63)); }
    template <class F> void for_each_one(F&& f) const {
        for (int k = lo; k < hi; k++) {
            uint64_t x = w[k];
            while (x) { f(k * 64 + __builtin_ctzll(x)); x &= x - 1; }
        }
    }
};
}  // namespace

Structure eliminate(const std::vector<Bits>& bmat, const Bits& parity) {
    const int m = (int)bmat.size();
    const int W = std::max(1, (m + 63) / 64);
    SpanRows gram(m, W), basis(m, W);
    for (int i = 0; i < m; i++) {
        bmat[i].for_each_one([&](int j) { gram.set(i, j); });
        if (parity.get(i)) gram.set(i, i);
        basis.set(i, i);
    }
    std::vector<uint64_t> alive((size_t)W, 0ull);
    for (int i = 0; i < m; i++) alive[(size_t)i >> 6] |= 1ull << (i & 63);
    auto is_alive = [&](int i) { return (alive[(size_t)i >> 6] >> (i & 63)) & 1ull; };
    Structure st;
    st.m = m;
    // key[a] = (class, weight): class 1 = diagonal set, 2 = off-diagonal only, 0 = neither
    std::vector<std::pair<uint8_t, uint32_t>> key((size_t)m, {0, 0});
    PivotQueue dq(W), oq(W);
    auto reclass = [&](int a) {
        std::pair<uint8_t, uint32_t> k{0, 0};
        if (is_alive(a)) {
            const uint64_t* r = gram.row(a);
            uint32_t w = 0;
            for (int q = gram.lo[a]; q < gram.hi[a]; q++) w += (uint32_t)__builtin_popcountll(r[q] & alive[q]);
            if ((r[a >> 6] >> (a & 63)) & 1ull) k = {1, w};
            else if (w > 0) k = {2, w};
        }
        if (k == key[a]) return;
        if (key[a].first == 1) dq.del(key[a].second, a);
        else if (key[a].first == 2) oq.del(key[a].second, a);
        key[a] = k;
        if (k.first == 1) dq.add(k.second, a);
        else if (k.first == 2) oq.add(k.second, a);
    };
    for (int a = 0; a < m; a++) reclass(a);
    SpanVec s(W), sb(W), touched(W);
    auto masked = [&](SpanVec& v, int r) {  // v = gram[r] & alive
        const uint64_t* g = gram.row(r);
        v.lo = gram.lo[r];
        v.hi = gram.hi[r];
        for (int q = v.lo; q < v.hi; q++) v.w[q] = g[q] & alive[q];
    };
    auto kill = [&](int a) { alive[(size_t)a >> 6] &= ~(1ull << (a & 63)); };
    while (true) {
        int a = dq.min();
        if (a >= 0) {  // single_step (normal_form.rs:61-82)
            masked(s, a);
            s.unset(a);
            s.trim();
            const Bits pa = basis.bits(a, m);
            const int plo = basis.lo[a], phi = basis.hi[a];
            s.for_each_one([&](int bi) {
                gram.xor_in(bi, s.w.data(), s.lo, s.hi);
                basis.xor_in(bi, pa.w.data(), plo, phi);
            });
            kill(a);
            st.odd.push_back(pa);
            st.sodd.push_back({plo, phi});
            reclass(a);
            s.for_each_one([&](int bi) { reclass(bi); });
            s.clear();
            continue;
        }
        a = oq.min();
        if (a >= 0) {  // hyper_step (normal_form.rs:87-129)
            masked(s, a);
            s.trim();
            int b = -1;
            for (int q = s.lo; q < s.hi && b < 0; q++)
                if (s.w[q]) b = q * 64 + __builtin_ctzll(s.w[q]);
            s.unset(b);
            s.trim();
            masked(sb, b);
            sb.unset(a);
            sb.trim();
            const Bits pa = basis.bits(a, m), pb = basis.bits(b, m);
            const int alo = basis.lo[a], ahi = basis.hi[a], blo = basis.lo[b], bhi = basis.hi[b];
            touched.lo = std::min(s.lo < s.hi ? s.lo : W, sb.lo < sb.hi ? sb.lo : W);
            touched.hi = std::max(s.hi, sb.hi);
            if (touched.lo > touched.hi) touched.lo = touched.hi;
            for (int q = touched.lo; q < touched.hi; q++) touched.w[q] = s.w[q] | sb.w[q];
            touched.for_each_one([&](int k) {
                if (s.get(k)) { gram.xor_in(k, sb.w.data(), sb.lo, sb.hi); basis.xor_in(k, pb.w.data(), blo, bhi); }
                if (sb.get(k)) { gram.xor_in(k, s.w.data(), s.lo, s.hi); basis.xor_in(k, pa.w.data(), alo, ahi); }
            });
            kill(a);
            kill(b);
            st.pa.push_back(pa);
            st.pb.push_back(pb);
            st.spa.push_back({alo, ahi});
            st.spb.push_back({blo, bhi});
            reclass(a);
            reclass(b);
            touched.for_each_one([&](int k) { reclass(k); });
            s.clear();
            sb.clear();
            touched.clear();
            continue;
        }
        break;
    }
    for (int r = 0; r < m; r++)
        if (is_alive(r)) {
            st.even.push_back(basis.bits(r, m));
            st.seven.push_back({basis.lo[r], basis.hi[r]});
        }
    return st;
}

// z4 value of a basis vector (normal_form.rs:339-348).  The bilinear part p^T B p (B symmetric,
// zero diagonal, a few entries per row) counts every pair {j, k} of p's bits with B_jk = 1
// twice; its half is summed over the upper adjacency lists (neighbours k > j): O(|p| deg / 2)
// bit tests instead of |p| row-wide popcounts.
static unsigned z4_value(const std::vector<std::vector<int>>& upper, const Bits& v0, const Bits& v1, const Bits& p,
                         std::pair<int, int> span) {
    unsigned lin = 0, half = 0;
    for (int q = span.first; q < span.second; q++) {
        const uint64_t x = p.w[(size_t)q];
        lin += (unsigned)__builtin_popcountll(x & v0.w[(size_t)q]) + 2u * (unsigned)__builtin_popcountll(x & v1.w[(size_t)q]);
        for (uint64_t r = x; r; r &= r - 1)
            for (int k : upper[(size_t)(q * 64 + __builtin_ctzll(r))]) half += p.get(k) ? 1u : 0u;
    }
    return (lin + 2 * (half & 1)) & 3u;
}

int HostEngine::phase8(const uint64_t* u) const {  // normal_form.rs:479-493
    int pc1 = 0, pc3 = 0;
    const uint64_t* uo = u + L.off_o();
    for (int i = 0; i < L.wo; i++) {
        pc1 += __builtin_popcountll(uo[i] & dg.o1.w[i]);
        pc3 += __builtin_popcountll(uo[i] & dg.o3.w[i]);
    }
    int n = sigma - 2 * (pc1 - pc3);
    unsigned cnt = 0;
    for (int i = 0; i < L.wg; i++)
        cnt += (unsigned)__builtin_popcountll((dg.wa.w[i] ^ u[L.off_a() + i]) & (dg.wb.w[i] ^ u[L.off_b() + i]));
    if (cnt & 1) n += 4;
    return ((n % 8) + 8) % 8;
}

// ---------------------------------------------------------------- engine build (src/engine.rs:289-390)
std::unique_ptr<HostEngine> build_engine(const PathSum& ps, const std::vector<int>& fixed) {
    auto E = std::make_unique<HostEngine>();
    const int nv = ps.nv, nf = (int)fixed.size();
    E->nv = nv;
    E->nf = nf;
    E->fixed = fixed;
    std::vector<int> fixed_pos((size_t)nv, -1);
    for (int i = 0; i < nf; i++) {
        int f = fixed[i];
        if (f < 0 || f >= nv || ps.dead[f]) throw std::invalid_argument("fixed variable is not live");
        if (fixed_pos[f] != -1) throw std::invalid_argument("duplicate fixed variable");
        fixed_pos[f] = i;
    }
    std::vector<int> fidx((size_t)nv, -1);
    for (int i = 0; i < nv; i++)
        if (!ps.dead[i] && fixed_pos[i] < 0) { fidx[i] = (int)E->freev.size(); E->freev.push_back(i); }
    const int m = (int)E->freev.size();
    E->m = m;
    std::vector<Bits> bff((size_t)m, Bits(m));
    Bits parity(m);
    for (int i = 0; i < m; i++) {
        ps.b[E->freev[i]].for_each_one([&](int j) { if (fidx[j] >= 0) bff[i].set(fidx[j], true); });
        parity.set(i, ps.v[E->freev[i]] & 1);
    }
    E->wf = words_of(nf);
    E->bfixed.assign((size_t)nf * std::max(1, E->wf), 0ull);
    for (int i = 0; i < nf; i++)
        ps.b[fixed[i]].for_each_one([&](int j) {
            int p = fixed_pos[j];
            if (p >= 0) E->bfixed[(size_t)i * E->wf + (p >> 6)] |= 1ull << (p & 63);
        });
    E->st = eliminate(bff, parity);
    const Structure& st = E->st;
    Layout& Lo = E->L;
    Lo.g = st.g(); Lo.nodd = (int)st.odd.size(); Lo.neven = (int)st.even.size();
    Lo.wg = words_of(Lo.g); Lo.wo = words_of(Lo.nodd); Lo.we = words_of(Lo.neven);
    const int W = Lo.full();

    // basis columns for the variables that need them (normal_form.rs:413-433)
    std::vector<uint8_t> needed((size_t)m, 0);
    for (int f : fixed) ps.b[f].for_each_one([&](int j) { if (fidx[j] >= 0) needed[fidx[j]] = 1; });
    for (int i = 0; i < m; i++) if (ps.theta[E->freev[i]] != 0) needed[i] = 1;
    std::vector<int> colpos((size_t)m, -1);
    int ncol = 0;
    for (int i = 0; i < m; i++) if (needed[i]) colpos[i] = ncol++;
    std::vector<uint64_t> cols((size_t)ncol * std::max(1, W), 0ull);
    auto scan = [&](const std::vector<Bits>& vecs, const std::vector<std::pair<int, int>>& span, int off) {
        for (size_t l = 0; l < vecs.size(); l++)
            for (int q = span[l].first; q < span[l].second; q++)
                for (uint64_t x = vecs[l].w[(size_t)q]; x; x &= x - 1) {
                    const int j = q * 64 + __builtin_ctzll(x);
                    if (colpos[j] >= 0) cols[(size_t)colpos[j] * W + off + (l >> 6)] |= 1ull << (l & 63);
                }
    };
    scan(st.pa, st.spa, Lo.off_a());
    scan(st.pb, st.spb, Lo.off_b());
    scan(st.odd, st.sodd, Lo.off_o());
    scan(st.even, st.seven, Lo.off_e());
    E->ucols.assign((size_t)nf * std::max(1, W), 0ull);
    for (int i = 0; i < nf; i++)
        ps.b[fixed[i]].for_each_one([&](int j) {
            int fj = fidx[j];
            if (fj < 0) return;
            const uint64_t* c = &cols[(size_t)colpos[fj] * W];
            for (int w = 0; w < W; w++) E->ucols[(size_t)i * W + w] ^= c[w];
        });
    // branching (engine.rs:372-378)
    for (int i = 0; i < m; i++) if (ps.theta[E->freev[i]] != 0) E->term_vars.push_back(i);
    const int t = (int)E->term_vars.size();
    E->t = t;
    E->mcols.assign((size_t)t * std::max(1, W), 0ull);
    for (int k = 0; k < t; k++) {
        const uint64_t* c = &cols[(size_t)colpos[E->term_vars[k]] * W];
        std::copy(c, c + W, E->mcols.begin() + (size_t)k * W);
    }
    // Elim::new (engine.rs:119-184): RREF of K = M|_even, tracking the row operations R
    const int ne = Lo.neven;
    std::vector<Bits> rk((size_t)ne, Bits(t)), rr((size_t)ne, Bits(ne));
    for (int r = 0; r < ne; r++) {
        rr[r].set(r, true);
        for (int c = 0; c < t; c++)
            if ((E->mcols[(size_t)c * W + Lo.off_e() + (r >> 6)] >> (r & 63)) & 1ull) rk[r].set(c, true);
    }
    int rank = 0;
    for (int col = 0; col < t; col++) {
        int r = -1;
        for (int i = rank; i < ne; i++) if (rk[i].get(col)) { r = i; break; }
        if (r < 0) continue;
        std::swap(rk[rank], rk[r]);
        std::swap(rr[rank], rr[r]);
        for (int r2 = 0; r2 < ne; r2++)
            if (r2 != rank && rk[r2].get(col)) { rk[r2].xor_with(rk[rank]); rr[r2].xor_with(rr[rank]); }
        E->piv_col.push_back(col);
        rank++;
    }
    E->rank = rank;
    for (int i = 0; i < rank; i++) E->piv_row.push_back(rr[i]);
    for (int i = rank; i < ne; i++) E->cons.push_back(rr[i]);
    E->ncons = ne - rank;
    std::vector<uint8_t> is_piv((size_t)t, 0);
    for (int c : E->piv_col) is_piv[c] = 1;
    const int abo = Lo.abo();
    for (int j = 0; j < t; j++) {
        if (is_piv[j]) continue;
        Bits kv(t);
        kv.set(j, true);
        uint64_t rmask = 0;
        for (int i = 0; i < rank; i++)
            if (rk[i].get(j)) { kv.set(E->piv_col[i], true); if (i < 64) rmask |= 1ull << i; }
        std::vector<uint64_t> u((size_t)W, 0ull);
        kv.for_each_one([&](int k) { for (int w = 0; w < W; w++) u[w] ^= E->mcols[(size_t)k * W + w]; });
        for (int w = Lo.off_e(); w < W; w++)
            if (u[w]) throw std::logic_error("kernel column with a radical component");
        E->ku.insert(E->ku.end(), u.begin(), u.begin() + abo);
        E->kernel.push_back(kv);
        E->R.push_back(rmask);
        E->free_col.push_back(j);
    }
    E->d = (int)E->kernel.size();
    // Z4 diagonal (normal_form.rs:354-391)
    Bits v0(m), v1(m);
    for (int i = 0; i < m; i++) { uint8_t x = ps.v[E->freev[i]]; v0.set(i, x & 1); v1.set(i, (x & 2) != 0); }
    std::vector<std::vector<int>> adj((size_t)m);  // upper adjacency: neighbours k > i
    for (int i = 0; i < m; i++)
        bff[(size_t)i].for_each_one([&](int k) {
            if (k > i) adj[(size_t)i].push_back(k);
        });
    Diag& dg = E->dg;
    dg.wa = Bits(Lo.g); dg.wb = Bits(Lo.g); dg.o1 = Bits(Lo.nodd); dg.o3 = Bits(Lo.nodd); dg.we = Bits(Lo.neven);
    for (int j = 0; j < Lo.g; j++) {
        dg.wa.set(j, z4_value(adj, v0, v1, st.pa[j], st.spa[(size_t)j]) == 2);
        dg.wb.set(j, z4_value(adj, v0, v1, st.pb[j], st.spb[(size_t)j]) == 2);
    }
    dg.sigma = 0;
    for (int l = 0; l < Lo.nodd; l++) {
        if (z4_value(adj, v0, v1, st.odd[l], st.sodd[(size_t)l]) == 1) { dg.o1.set(l, true); dg.sigma++; }
        else { dg.o3.set(l, true); dg.sigma--; }
    }
    for (int l = 0; l < Lo.neven; l++) dg.we.set(l, z4_value(adj, v0, v1, st.even[l], st.seven[(size_t)l]) == 2);
    E->sigma = dg.sigma;
    E->mag2 = 2 * Lo.g + 2 * Lo.neven + Lo.nodd;
    // terms (engine.rs:232-238), FP64
    for (int k = 0; k < t; k++) {
        Cplx e = phase_complex(ps.theta[E->freev[E->term_vars[k]]]);
        E->alpha.push_back({(1.0 + e.re) * 0.5, (0.0 + e.im) * 0.5});
        E->beta.push_back({(1.0 - e.re) * 0.5, (0.0 - e.im) * 0.5});
    }
    for (int i = 0; i < nf; i++) { E->fixed_v.push_back(ps.v[fixed[i]]); E->fixed_th.push_back(ps.theta[fixed[i]]); }
    E->num_h = ps.num_h;
    E->global = ps.global;
    E->zero = ps.zero;
    // quadratic part of the Z8 phase over kernel coordinates: 4*G_ij is the second finite
    // difference of phase8 along kernel columns i and j, which does not depend on the base point
    const int d = E->d;
    E->dw = (d + 63) / 64;
    E->Gw.assign((size_t)d * (size_t)E->dw, 0ull);
    {
        std::vector<uint64_t> z((size_t)abo, 0ull), uij((size_t)abo);
        const int p0 = E->phase8(z.data());
        std::vector<int> p1((size_t)d);
        for (int j = 0; j < d; j++) p1[j] = E->phase8(&E->ku[(size_t)j * abo]);
        // Z8 first differences are 2 Lp_j; the parity of Lp_j does not depend on the base point
        E->lp0.assign((size_t)d, 0);
        for (int j = 0; j < d; j++) E->lp0[(size_t)j] = (uint8_t)(((((p1[j] - p0) % 8 + 8) % 8) >> 1) & 1);
        for (int i = 0; i < d; i++)
            for (int j = i + 1; j < d; j++) {
                for (int w = 0; w < abo; w++) uij[w] = E->ku[(size_t)i * abo + w] ^ E->ku[(size_t)j * abo + w];
                int dd = ((E->phase8(uij.data()) - p1[i] - p1[j] + p0) % 8 + 16) % 8;
                if (dd != 0 && dd != 4) throw std::logic_error("phase is not quadratic over the kernel");
                if (dd == 4) {
                    E->Gw[(size_t)i * E->dw + (size_t)(j >> 6)] |= 1ull << (j & 63);
                    E->Gw[(size_t)j * E->dw + (size_t)(i >> 6)] |= 1ull << (i & 63);
                }
            }
    }
    // one word per row, the enumeration's form: complete for d <= 64, coordinates 0..63 above
    E->G.assign((size_t)d, 0ull);
    for (int j = 0; j < d; j++) E->G[(size_t)j] = E->Gw[(size_t)j * E->dw];
    // error-bound factor: sum_s |c(s)| <= prod_j (|a0|+|a1|)(free cols) * prod_i max(|a0|,|a1|)(pivots)
    double bound = 1.0;
    for (int j = 0; j < d; j++) {
        int k = E->free_col[j];
        bound *= std::hypot(E->alpha[k].re, E->alpha[k].im) + std::hypot(E->beta[k].re, E->beta[k].im);
    }
    for (int i = 0; i < rank; i++) {
        int k = E->piv_col[i];
        bound *= std::max(std::hypot(E->alpha[k].re, E->alpha[k].im), std::hypot(E->beta[k].re, E->beta[k].im));
    }
    E->sum_abs_bound = bound;
    return E;
}

// ---------------------------------------------------------------- strategy layer (src/rank.rs)
static const int kMaxPairs = 14;
static const uint32_t kMask30 = (1u << 30) - 1;

std::vector<std::pair<int, int>> pair_candidates(const PathSum& ps, const std::vector<int>& fixed, int& ntclass) {
    std::map<uint32_t, std::vector<int>> groups;  // rank.rs:62-84
    for (int k = 0; k < ps.nv; k++) {
        if (ps.dead[k] || ps.theta[k] == 0) continue;
        if (std::find(fixed.begin(), fixed.end(), k) != fixed.end()) continue;
        uint32_t r = ps.theta[k] & kMask30;
        uint32_t o = (uint32_t)(((uint64_t)kMask30 + 1 - r) & kMask30);
        groups[std::min(r, o)].push_back(k);
    }
    std::vector<std::pair<int, int>> tp, gp;
    for (auto& kv : groups) {
        auto& target = kv.first == (1u << 29) ? tp : gp;
        for (size_t i = 0; i + 1 < kv.second.size(); i += 2) target.push_back({kv.second[i], kv.second[i + 1]});
    }
    ntclass = (int)tp.size();
    tp.insert(tp.end(), gp.begin(), gp.end());
    return tp;
}

int best_pairs(const HostEngine& base, int available, int tclass) {  // rank.rs:205-222
    double m = (double)base.m;
    double words = (double)(base.m / 64 + 1);
    double ldl = 2.0 * m * m * m / 64.0 + 50.0 * m + 2000.0;
    double step = 20.0 + 4.0 * words + (double)base.t / 2.0;
    int best = 0;
    double bestc = INFINITY;
    for (int p = 0; p <= std::min(available, kMaxPairs); p++) {
        int removed = 2 * std::min(p, tclass) + std::max(0, p - tclass);
        int d = std::max(0, base.d - removed);
        double cost = std::pow(2.0, (double)p) * ((p == 0 ? 0.0 : ldl) + std::pow(2.0, (double)d) * step);
        if (cost < bestc) { best = p; bestc = cost; }
    }
    return best;
}

std::unique_ptr<HostEngine> pattern_engine(const PathSum& ps, const std::vector<int>& fixed,
                                           const std::vector<std::pair<int, int>>& cands, int p, uint64_t pattern) {
    PathSum b = ps;
    for (int i = 0; i < p; i++) b.substitute(cands[(size_t)i].first, cands[(size_t)i].second, (pattern >> i) & 1ull);
    return build_engine(b, fixed);
}

// 2^p branch engines built on host threads (rank.rs:88-103 builds them with rayon)
static RankSet rank_new(const PathSum& ps, const std::vector<int>& fixed, int pairs) {
    int nt = 0;
    auto cands = pair_candidates(ps, fixed, nt);
    int p = std::min(std::min(pairs, (int)cands.size()), kMaxPairs);
    RankSet rs;
    rs.pairs = p;
    const int nb = 1 << p;
    rs.branches.resize((size_t)nb);
    std::atomic<int> next{0};
    std::vector<std::string> errs((size_t)nb);
    auto work = [&]() {
        for (int pat = next++; pat < nb; pat = next++) {
            try {
                PathSum b = ps;
                for (int i = 0; i < p; i++) b.substitute(cands[i].first, cands[i].second, (pat >> i) & 1);
                rs.branches[pat] = build_engine(b, fixed);
            } catch (const std::exception& e) {
                errs[pat] = e.what();
            }
        }
    };
    int nth = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)nb);
    if (nth <= 1) work();
    else {
        std::vector<std::thread> th;
        for (int i = 0; i < nth; i++) th.emplace_back(work);
        for (auto& x : th) x.join();
    }
    for (auto& e : errs) if (!e.empty()) throw std::runtime_error(e);
    return rs;
}

RankSet build_rank(const PathSum& ps, const std::vector<int>& fixed, int strategy, int pairs) {
    if (strategy == STRAT_CACHED) return rank_new(ps, fixed, 0);
    if (strategy == STRAT_PAIRS) return rank_new(ps, fixed, pairs);
    // Auto (rank.rs:115-123)
    auto base = build_engine(ps, fixed);
    int nt = 0;
    auto cands = pair_candidates(ps, fixed, nt);
    int p = best_pairs(*base, (int)cands.size(), nt);
    if (p == 0) {
        RankSet rs;
        rs.pairs = 0;
        rs.branches.push_back(std::move(base));
        return rs;
    }
    return rank_new(ps, fixed, p);
}

// ---------------------------------------------------------------- weight tables
static inline Cplx cmul(Cplx a, Cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

EngineTables build_tables(const HostEngine& e, int di_max) {
    EngineTables T;
    const int d = e.d;
    T.DI = std::min(d, di_max);
    T.joint = e.rank <= kJointMaxPivots;
    if (T.joint && T.DI + e.rank > kJointMaxBits) T.DI = std::max(0, kJointMaxBits - e.rank);
    T.pmask = e.rank >= 64 ? ~0ull : ((1ull << e.rank) - 1ull);
    T.plo = e.rank;
    if (!T.joint && e.dev_DI >= 3) {
        // more pivots than one table holds: the table covers the pivots the dev_DI low
        // coordinates (chosen by device_order) touch; the others become a per-chunk factor
        uint64_t pm = 0;
        for (int j = 0; j < e.dev_DI; j++) pm |= e.R[(size_t)j];
        if (e.dev_DI + __builtin_popcountll(pm) <= kJointMaxBits) {
            T.DI = e.dev_DI;
            T.joint = T.partial = true;
            T.pmask = pm;
            T.plo = __builtin_popcountll(pm);
        }
    }
    T.Rc.resize((size_t)d);
    for (int j = 0; j < d; j++) {
        uint64_t r = e.R[(size_t)j];
        if (T.partial && j < T.DI) {
            uint64_t c = 0;
            int k = 0;
            for (uint64_t m = T.pmask; m; m &= m - 1, k++) c |= ((r >> __builtin_ctzll(m)) & 1ull) << k;
            r = c;
        }
        T.Rc[(size_t)j] = r;
    }
    auto xw = [&](int j, int bit) { int k = e.free_col[j]; return bit ? e.beta[k] : e.alpha[k]; };
    auto pw = [&](int i, int bit) { int k = e.piv_col[i]; return bit ? e.beta[k] : e.alpha[k]; };
    const size_t nlo = (size_t)1 << T.DI;
    T.tlo.resize(nlo);
    for (size_t s = 0; s < nlo; s++) {
        Cplx c{1.0, 0.0};
        for (int j = 0; j < T.DI; j++) c = cmul(c, xw(j, (int)((s >> j) & 1)));
        T.tlo[s] = c;
    }
    T.nsl_tp = (e.rank + 7) / 8;
    T.tp.resize((size_t)T.nsl_tp * 256);
    for (int sl = 0; sl < T.nsl_tp; sl++)
        for (int b = 0; b < 256; b++) {
            Cplx c{1.0, 0.0};
            for (int k = 0; k < 8 && 8 * sl + k < e.rank; k++) c = cmul(c, pw(8 * sl + k, (b >> k) & 1));
            T.tp[(size_t)sl * 256 + b] = c;
        }
    T.nsl_th = (d - T.DI + 7) / 8;
    T.th.resize((size_t)T.nsl_th * 256);
    for (int sl = 0; sl < T.nsl_th; sl++)
        for (int b = 0; b < 256; b++) {
            Cplx c{1.0, 0.0};
            for (int k = 0; k < 8 && T.DI + 8 * sl + k < d; k++) c = cmul(c, xw(T.DI + 8 * sl + k, (b >> k) & 1));
            T.th[(size_t)sl * 256 + b] = c;
        }
    if (T.joint) {
        // pivot of table index bit k: the k-th set bit of pmask
        std::vector<int> piv;
        for (int i = 0; i < e.rank; i++)
            if ((T.pmask >> i) & 1ull) piv.push_back(i);
        T.w.resize((size_t)1 << (T.DI + T.plo));
        for (size_t y = 0; y < ((size_t)1 << T.plo); y++) {
            Cplx tpv{1.0, 0.0};
            for (int k = 0; k < T.plo; k++) tpv = cmul(tpv, pw(piv[(size_t)k], (int)((y >> k) & 1)));
            for (size_t s = 0; s < nlo; s++) T.w[(y << T.DI) | s] = cmul(T.tlo[s], tpv);
        }
    }
    if (T.partial) {
        T.thp.resize((size_t)T.nsl_tp * 256);
        for (int sl = 0; sl < T.nsl_tp; sl++)
            for (int b = 0; b < 256; b++) {
                Cplx c{1.0, 0.0};
                for (int k = 0; k < 8 && 8 * sl + k < e.rank; k++)
                    if (!((T.pmask >> (8 * sl + k)) & 1ull)) c = cmul(c, pw(8 * sl + k, (b >> k) & 1));
                T.thp[(size_t)sl * 256 + b] = c;
            }
    }
    return T;
}

// ---------------------------------------------------------------- packing for upload
namespace {
struct Packer {
    std::vector<uint8_t> blob;
    size_t put(const void* p, size_t bytes) {
        size_t off = (blob.size() + 15) & ~(size_t)15;
        blob.resize(off + std::max<size_t>(bytes, 16), 0);
        if (bytes) std::memcpy(blob.data() + off, p, bytes);
        return off;
    }
    template <class T> size_t vec(const std::vector<T>& v) { return put(v.data(), v.size() * sizeof(T)); }
};
template <class T> const T* as_off(size_t o) { return reinterpret_cast<const T*>(o); }
template <class T> const T* shift(const T* p, const uint8_t* base) {
    return reinterpret_cast<const T*>(base + reinterpret_cast<size_t>(p));
}
}  // namespace

PackedEngine pack_engine(const HostEngine& e, const EngineTables& T) {
    PackedEngine P;
    Packer k;
    EngineDev& d = P.off;
    std::memset(&d, 0, sizeof(d));
    const Layout& L = e.L;
    d.nf = e.nf; d.t = e.t; d.d = e.d; d.rank = e.rank; d.ncons = e.ncons;
    d.wg = L.wg; d.wo = L.wo; d.we = L.we; d.wf = e.wf; d.W = L.full(); d.abo = L.abo();
    d.sigma = e.sigma; d.mag2 = e.mag2; d.num_h = e.num_h; d.global = e.global; d.zero = e.zero ? 1 : 0;
    d.DI = T.DI; d.nsl_tp = T.nsl_tp; d.nsl_th = T.nsl_th;
    d.plo = T.plo; d.pmask = T.pmask;
    d.sum_abs_bound = e.sum_abs_bound;
    d.o1 = as_off<uint64_t>(k.vec(e.dg.o1.w));
    d.o3 = as_off<uint64_t>(k.vec(e.dg.o3.w));
    d.wa = as_off<uint64_t>(k.vec(e.dg.wa.w));
    d.wb = as_off<uint64_t>(k.vec(e.dg.wb.w));
    d.wem = as_off<uint64_t>(k.vec(e.dg.we.w));
    d.ucols = as_off<uint64_t>(k.vec(e.ucols));
    d.mcols = as_off<uint64_t>(k.vec(e.mcols));
    d.ku = as_off<uint64_t>(k.vec(e.ku));
    d.bfixed = as_off<uint64_t>(k.vec(e.bfixed));
    d.fixed_v = as_off<uint8_t>(k.vec(e.fixed_v));
    d.fixed_th = as_off<uint32_t>(k.vec(e.fixed_th));
    std::vector<uint64_t> pr, cs;
    for (const auto& r : e.piv_row) pr.insert(pr.end(), r.w.begin(), r.w.end());
    for (const auto& r : e.cons) cs.insert(cs.end(), r.w.begin(), r.w.end());
    d.pivrow = as_off<uint64_t>(k.vec(pr));
    d.cons = as_off<uint64_t>(k.vec(cs));
    std::vector<int32_t> pc(e.piv_col.begin(), e.piv_col.end());
    d.pivcol = as_off<int32_t>(k.vec(pc));
    d.G = as_off<uint64_t>(k.vec(e.G));
    d.Gw = as_off<uint64_t>(k.vec(e.Gw));
    d.dw = e.dw;
    d.R = as_off<uint64_t>(k.vec(e.R));
    d.Rc = as_off<uint64_t>(k.vec(T.Rc));
    d.thp = T.partial ? as_off<double2>(k.vec(T.thp)) : nullptr;
    std::vector<float> tlo32, tp32;
    for (const auto& c : T.tlo) { tlo32.push_back((float)c.re); tlo32.push_back((float)c.im); }
    for (const auto& c : T.tp) { tp32.push_back((float)c.re); tp32.push_back((float)c.im); }
    d.tlo = as_off<float2>(k.vec(tlo32));
    d.tp = as_off<float2>(k.vec(tp32));
    d.th = as_off<double2>(k.vec(T.th));
    d.tlo64 = as_off<double2>(k.vec(T.tlo));
    d.tp64 = as_off<double2>(k.vec(T.tp));
    d.joint = T.joint ? 1 : 0;
    d.npairc = 0;
    d.pairc[0] = d.pairc[1] = d.pairc[2] = -1;
    if (T.joint)
        for (int j = T.DI; j < e.d && d.npairc < 3; j++)
            if (e.R[(size_t)j] == 0) d.pairc[d.npairc++] = j;
    // The high-coordinate weight factors as chi(s) = chi_rest(s) P(bits of s at the pair
    // coordinates): thr is th without the pair coordinates' factors, pf the 2^npairc values of P
    // split into FP32 hi + lo (the walk combines the chunks of a unit with them in FP32 pairs).
    {
        auto xw = [&](int j, int bit) { int kk = e.free_col[(size_t)j]; return bit ? e.beta[kk] : e.alpha[kk]; };
        auto is_pair = [&](int j) { return j == d.pairc[0] || j == d.pairc[1] || j == d.pairc[2]; };
        std::vector<Cplx> thr((size_t)T.nsl_th * 256);
        for (int sl = 0; sl < T.nsl_th; sl++)
            for (int b = 0; b < 256; b++) {
                Cplx c{1.0, 0.0};
                for (int q = 0; q < 8 && T.DI + 8 * sl + q < e.d; q++)
                    if (!is_pair(T.DI + 8 * sl + q)) c = cmul(c, xw(T.DI + 8 * sl + q, (b >> q) & 1));
                thr[(size_t)sl * 256 + b] = c;
            }
        d.thr = as_off<double2>(k.vec(thr));
        std::vector<float> pf;
        for (int pat = 0; pat < (1 << d.npairc); pat++) {
            Cplx c{1.0, 0.0};
            for (int i = 0; i < d.npairc; i++) c = cmul(c, xw(d.pairc[i], (pat >> i) & 1));
            const float hr = (float)c.re, hi = (float)c.im;
            pf.push_back(hr);
            pf.push_back(hi);
            pf.push_back((float)(c.re - (double)hr));
            pf.push_back((float)(c.im - (double)hi));
        }
        d.pf = as_off<float4>(k.vec(pf));
    }
    // hi.re, hi.im, lo.re, lo.im with hi + lo = the FP64 weight.  hi lies on the grid g, a power
    // of two with 2^DI * max|w| <= 2^23 g: any sum of at most 2^DI hi parts (a chunk) is then an
    // integer multiple of g below 2^24 g, i.e. exact in FP32; lo = w - hi (|lo| <= g/2) carries
    // the rest and is summed in plain FP32.
    double wmax = 0.0;
    for (const auto& c : T.w) wmax = std::max(wmax, std::max(std::fabs(c.re), std::fabs(c.im)));
    double grid = 0.0;
    if (wmax > 0.0) grid = std::ldexp(1.0, (int)std::ceil(std::log2(std::ldexp(wmax, T.DI) / 8388608.0)));
    d.grid = grid;
    // Error of one job's chunk sums from the lo parts: per chunk of N <= 2^DI branches the four
    // lo accumulators err by <= N (g/2)(gamma_N + u) each (summation and the FP32 rounding of lo);
    // chunks are scaled by the FP64 weight of the coordinates >= DI, whose absolute sum over
    // chunks is prod_{j >= DI} (|a_j0| + |a_j1|).
    {
        const double u = 5.9604644775390625e-08, n = std::ldexp(1.0, T.DI);
        const double gam = n * u / (1.0 - n * u);
        double hi_abs = 1.0;
        for (int j = T.DI; j < e.d; j++) {
            int kk = e.free_col[j];
            hi_abs *= std::hypot(e.alpha[kk].re, e.alpha[kk].im) + std::hypot(e.beta[kk].re, e.beta[kk].im);
        }
        // the pivots outside the table scale each chunk by at most the product of their
        // larger weights
        if (T.partial)
            for (int i = 0; i < e.rank; i++)
                if (!((T.pmask >> i) & 1ull)) {
                    const int kk = e.piv_col[(size_t)i];
                    hi_abs *= std::max(std::hypot(e.alpha[kk].re, e.alpha[kk].im), std::hypot(e.beta[kk].re, e.beta[kk].im));
                }
        d.errfac = 4.0 * n * (grid / 2.0) * (gam + u) * hi_abs;
    }
    // The table entry of low coordinates s carries the sign (-1)^{q(s)} of the quadratic phase
    // among them, q(s) = sum_{i<j<DI} G_ij s_i s_j, so that the enumeration sees a Z4 index that
    // is linear in the coordinates it walks.
    std::vector<uint8_t> qsign((size_t)1 << T.DI, 0);
    for (size_t s = 1; s < qsign.size(); s++) {
        const int j = __builtin_ctzll((unsigned long long)s);
        const uint64_t rest = (uint64_t)s & ~(1ull << j);
        qsign[s] = (uint8_t)(qsign[rest] ^ (__builtin_popcountll(e.G[(size_t)j] & rest) & 1));
    }
    std::vector<float> w32;
    const size_t lomask = ((size_t)1 << T.DI) - 1;
    for (size_t idx = 0; idx < T.w.size(); idx++) {
        Cplx c = T.w[idx];
        if (qsign[idx & lomask]) c = Cplx{-c.re, -c.im};
        const double hr = grid > 0.0 ? std::nearbyint(c.re / grid) * grid : 0.0;
        const double hi = grid > 0.0 ? std::nearbyint(c.im / grid) * grid : 0.0;
        w32.push_back((float)hr);
        w32.push_back((float)hi);
        w32.push_back((float)(c.re - hr));
        w32.push_back((float)(c.im - hi));
    }
    d.wtab = nullptr;  // uploaded apart, at an address aligned to its size
    P.wtab = std::move(w32);
    // Chunk-sum table: a chunk walks all DI low coordinates, along which the folded Z4 index is
    // linear, i^{m} = i^{m_start} prod_j i^{Lp0_j s_j} (-1)^{b_j s_j}, b_j = (Lp_j >> 1) ^ c_j; so
    // its sum is i^{m_start} T[y_start][b] with
    //   T[u][b] = sum_s i^{<Lp0, s>} (-1)^{<b, s>} W'[u ^ R_lo s][s],
    // a Walsh-Hadamard transform over s for each pivot pattern u (FP64, once per engine).
    d.ctab = nullptr;
    // (A partial table's chunk sums index its pivots the same way, through the packed masks Rc;
    // the other pivots' weight multiplies each chunk's sum on the device.)
    if (T.joint && T.DI >= 1 && T.DI + T.plo <= 16) {
        const size_t nlo = (size_t)1 << T.DI, nu = (size_t)1 << T.plo;
        std::vector<Cplx> ct(nu * nlo);
        for (size_t u = 0; u < nu; u++) {
            Cplx *g = &ct[u * nlo];
            for (size_t s = 0; s < nlo; s++) {
                uint64_t y = u;
                int ph = 0;
                for (int j = 0; j < T.DI; j++)
                    if ((s >> j) & 1) {
                        y ^= T.Rc[(size_t)j];
                        ph += e.lp0[(size_t)j];
                    }
                Cplx w = T.w[(y << T.DI) | s];
                if (qsign[s]) w = Cplx{-w.re, -w.im};
                switch (ph & 3) {  // times i^ph
                    case 0: g[s] = w; break;
                    case 1: g[s] = Cplx{-w.im, w.re}; break;
                    case 2: g[s] = Cplx{-w.re, -w.im}; break;
                    default: g[s] = Cplx{w.im, -w.re}; break;
                }
            }
            for (size_t h = 1; h < nlo; h <<= 1)  // in-place transform, T[b] = sum_s (-1)^{<b,s>} g[s]
                for (size_t i = 0; i < nlo; i += 2 * h)
                    for (size_t k2 = i; k2 < i + h; k2++) {
                        const Cplx a = g[k2], b = g[k2 + h];
                        g[k2] = Cplx{a.re + b.re, a.im + b.im};
                        g[k2 + h] = Cplx{a.re - b.re, a.im - b.im};
                    }
        }
        d.ctab = as_off<double2>(k.vec(ct));
    }
    P.blob.swap(k.blob);
    return P;
}

// Low (walked) coordinates of an engine with more pivots than one joint table holds: the
// pivot-free coordinates first -- all but three, which stay high as the pair coordinates of the
// walk's units -- then, one at a time, the coordinate that touches the fewest pivots not yet
// touched, while DI + (pivots touched) stays within kJointMaxBits.  Returns them ascending.
static std::vector<int> low_coordinates_many_pivots(const HostEngine& e, int di_max) {
    std::vector<int> zero, other;
    for (int j = 0; j < e.d; j++) (e.R[(size_t)j] == 0 ? zero : other).push_back(j);
    const size_t keep = std::min<size_t>(3, zero.size());
    std::vector<int> L(zero.begin(), zero.end() - (long)keep);
    const int cap = std::min(di_max, kJointMaxBits);
    if ((int)L.size() > cap) L.resize((size_t)cap);
    std::vector<char> used((size_t)e.d, 0);
    for (int j : L) used[(size_t)j] = 1;
    uint64_t pm = 0;
    while ((int)L.size() < cap) {
        int best = -1, bestc = 65;
        for (int j : other)
            if (!used[(size_t)j]) {
                const int c = __builtin_popcountll(e.R[(size_t)j] & ~pm);
                if (c < bestc) { bestc = c; best = j; }
            }
        if (best < 0 || (int)L.size() + 1 + __builtin_popcountll(pm | e.R[(size_t)best]) > kJointMaxBits) break;
        L.push_back(best);
        used[(size_t)best] = 1;
        pm |= e.R[(size_t)best];
    }
    std::sort(L.begin(), L.end());
    return L;
}

// Low (walked) coordinates of an engine whose joint table holds all its pivots: any DI
// coordinates will do, so those whose Z4 increment is even come first (an even step is one
// paired FMA per accumulator pair, an odd one four scalar FMA plus a swap), keeping up to three
// pivot-free coordinates high as the pair coordinates of the walk's units (odd ones kept first).
// Returns them ascending.
static std::vector<int> low_coordinates_even_first(const HostEngine& e, int DI) {
    const int d = e.d;
    std::vector<char> kept((size_t)d, 0);
    int keep = 0;
    for (int pass = 0; pass < 2; pass++)  // pivot-free odd coordinates, then pivot-free even ones
        for (int j = d - 1; j >= 0 && keep < 3; j--)
            if (e.R[(size_t)j] == 0 && (int)e.lp0[(size_t)j] == 1 - pass && !kept[(size_t)j]) {
                kept[(size_t)j] = 1;
                keep++;
            }
    std::vector<int> L;
    for (int pass = 0; pass < 3 && (int)L.size() < DI; pass++)  // even, odd, then the kept ones
        for (int j = 0; j < d && (int)L.size() < DI; j++) {
            const bool take = pass == 0 ? (!kept[(size_t)j] && !e.lp0[(size_t)j])
                                        : (pass == 1 ? (!kept[(size_t)j] && e.lp0[(size_t)j]) : kept[(size_t)j] != 0);
            if (take) L.push_back(j);
        }
    std::sort(L.begin(), L.end());
    return L;
}

HostEngine device_order(const HostEngine& e, int di_max, std::vector<int>& perm) {
    // The low DI coordinates (the walked ones) are those of the joint table, moved to the front:
    // for an engine with d <= 62 those low_coordinates_even_first picks, or, with more pivots
    // than one table holds, those low_coordinates_many_pivots picks; else the first DI in the
    // reference order.  Among them the coordinates
    // whose Z4 increment is even come first (stable), then the odd ones: the walk's fixed-
    // position steps are then even quarter turns (paired FMA) for almost every engine.  The
    // other coordinates follow, those that touch no pivot first, each group in reference order.
    // perm[j] = reference coordinate of device coordinate j.
    const int d = e.d;
    std::vector<int> low;
    if (e.rank > kJointMaxPivots && d <= 62) low = low_coordinates_many_pivots(e, di_max);
    else if (d <= 62) {
        int DI = std::min(d, di_max);
        if (DI + e.rank > kJointMaxBits) DI = std::max(0, kJointMaxBits - e.rank);
        if (DI >= 3) low = low_coordinates_even_first(e, DI);
    }
    if (low.size() < 3) {
        low.clear();
        int DI = std::min(d, di_max);
        if (e.rank <= kJointMaxPivots && DI + e.rank > kJointMaxBits) DI = std::max(0, kJointMaxBits - e.rank);
        for (int j = 0; j < DI; j++) low.push_back(j);
    }
    const int DI = (int)low.size();
    // Units of chunks that differ in the pair coordinates (the first three coordinates outside
    // the walked ones that touch no pivot) are walked as sums bucketed by the parities of the
    // walked point with the pair coordinates' G rows (the bucket walk).  Walked coordinates with
    // even Z4 increments whose G bits at the pair coordinates agree, placed first -- two pairs
    // (16-point groups), else three or two and any third (8-point groups) -- keep every group's
    // points in at most four buckets.
    std::vector<int> even;
    for (int j : low)
        if (!e.lp0[(size_t)j]) even.push_back(j);
    {
        std::vector<char> in_low0((size_t)d, 0);
        for (int j : low) in_low0[(size_t)j] = 1;
        std::vector<int> pr;
        for (int j = 0; j < d && pr.size() < 3; j++)
            if (!in_low0[(size_t)j] && e.R[(size_t)j] == 0) pr.push_back(j);
        if (pr.size() >= 2 && even.size() >= 3) {
            auto gof = [&](int j) {
                int g = 0;
                for (size_t i = 0; i < pr.size(); i++)
                    g |= (int)((e.Gw[(size_t)pr[i] * e.dw + (size_t)(j >> 6)] >> (j & 63)) & 1ull) << i;
                return g;
            };
            int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int j : even) cnt[gof(j)]++;
            // 16-point groups: two pairs, coordinates 0, 1 of one value (gam) and 2, 3 of one value
            // (del); fewest buckets first (gam = del = 0: one; gam = del or gam = 0: two; else four)
            int bg = -1, bd = -1, bscore = 99;
            for (int g = 0; g < 8; g++)
                for (int h = 0; h < 8; h++) {
                    if (cnt[g] < 2 || cnt[h] < 2 || (g == h && cnt[g] < 4)) continue;
                    const int score = (g == 0 && h == 0) ? 0 : ((g == h || g == 0) ? 1 : 2);
                    if (score < bscore) { bscore = score; bg = g; bd = h; }
                }
            if (bg >= 0) {
                std::vector<int> p0, p1, rest;
                for (int j : even) {
                    const int v = gof(j);
                    if (v == bg && p0.size() < 2) p0.push_back(j);
                    else if (v == bd && p1.size() < 2) p1.push_back(j);
                    else rest.push_back(j);
                }
                even = p0;
                even.insert(even.end(), p1.begin(), p1.end());
                even.insert(even.end(), rest.begin(), rest.end());
            } else {
                // 8-point groups: three coordinates with one value (two buckets per group, one for
                // the value 0), else two (four buckets) followed by any third
                int best = -1, need = 3;
                for (; need >= 2 && best < 0; need--)
                    for (int g = 0; g < 8; g++)
                        if (cnt[g] >= need && (best < 0 || (best != 0 && cnt[g] > cnt[best]))) best = g;
                if (best >= 0) {
                    std::vector<int> front, rest;
                    for (int j : even) (front.size() < 3 && gof(j) == best ? front : rest).push_back(j);
                    even = front;
                    even.insert(even.end(), rest.begin(), rest.end());
                }
            }
        }
    }
    perm.resize((size_t)d);
    int k = 0;
    for (int j : even) perm[(size_t)k++] = j;
    for (int j : low)
        if (e.lp0[(size_t)j]) perm[(size_t)k++] = j;
    std::vector<char> in_low((size_t)d, 0);
    for (int j : low) in_low[(size_t)j] = 1;
    // high coordinates that touch no pivot first: the lowest chunk-index bits above the pair
    // coordinates are the lane bits of a warp's units, so a warp's 32 lanes then read the same
    // table entry at every step (a warp-wide load costs L1 data-path time per distinct entry)
    // (engines the enumeration handles, d <= 62; above, only the first 64 coordinates may move:
    // the Monte-Carlo sampler maps its draws through a 64-entry coordinate table)
    for (int pass = 0; pass < 2; pass++)
        for (int j = 0; j < d; j++)
            if (!in_low[(size_t)j] && (d > 62 ? pass == 0 : (e.R[(size_t)j] == 0) == (pass == 0)))
                perm[(size_t)k++] = j;
    HostEngine p = e;
    const int abo = e.L.abo();
    std::vector<int> inv((size_t)d);
    for (int j = 0; j < d; j++) inv[(size_t)perm[(size_t)j]] = j;
    for (int j = 0; j < d; j++) {
        const int r = perm[(size_t)j];
        std::copy(e.ku.begin() + (size_t)r * abo, e.ku.begin() + (size_t)(r + 1) * abo, p.ku.begin() + (size_t)j * abo);
        p.kernel[(size_t)j] = e.kernel[(size_t)r];
        p.R[(size_t)j] = e.R[(size_t)r];
        p.free_col[(size_t)j] = e.free_col[(size_t)r];
        p.lp0[(size_t)j] = e.lp0[(size_t)r];
    }
    std::fill(p.Gw.begin(), p.Gw.end(), 0ull);
    for (int i = 0; i < d; i++)
        for (int j = 0; j < d; j++)
            if ((e.Gw[(size_t)i * e.dw + (size_t)(j >> 6)] >> (j & 63)) & 1ull) {
                const int a = inv[(size_t)i], b = inv[(size_t)j];
                p.Gw[(size_t)a * p.dw + (size_t)(b >> 6)] |= 1ull << (b & 63);
            }
    for (int j = 0; j < d; j++) p.G[(size_t)j] = p.Gw[(size_t)j * p.dw];
    p.dev_DI = DI;
    return p;
}

EngineDev rebase_engine(const EngineDev& o, const uint8_t* base) {
    EngineDev d = o;
    d.o1 = shift(o.o1, base); d.o3 = shift(o.o3, base); d.wa = shift(o.wa, base); d.wb = shift(o.wb, base);
    d.wem = shift(o.wem, base); d.ucols = shift(o.ucols, base); d.mcols = shift(o.mcols, base);
    d.ku = shift(o.ku, base); d.bfixed = shift(o.bfixed, base); d.fixed_v = shift(o.fixed_v, base);
    d.fixed_th = shift(o.fixed_th, base); d.pivrow = shift(o.pivrow, base); d.cons = shift(o.cons, base);
    d.pivcol = shift(o.pivcol, base); d.G = shift(o.G, base); d.Gw = shift(o.Gw, base); d.R = shift(o.R, base);
    d.tlo = shift(o.tlo, base); d.tp = shift(o.tp, base); d.th = shift(o.th, base);
    d.thr = shift(o.thr, base); d.pf = shift(o.pf, base);
    d.tlo64 = shift(o.tlo64, base); d.tp64 = shift(o.tp64, base); d.wtab = nullptr;
    d.Rc = shift(o.Rc, base);
    d.thp = o.thp ? shift(o.thp, base) : nullptr;
    d.ctab = o.ctab ? shift(o.ctab, base) : nullptr;
    return d;
}

IoMapHost build_iomap(const std::vector<std::pair<int, int32_t>>& puts) {
    IoMapHost m;
    for (const auto& p : puts) {
        auto it = std::find(m.fixed.begin(), m.fixed.end(), p.first);
        if (it == m.fixed.end()) { m.fixed.push_back(p.first); m.src.push_back(p.second); }
        else { m.cf_pos.push_back((int32_t)(it - m.fixed.begin())); m.cf_src.push_back(p.second); }
    }
    return m;
}

// ---------------------------------------------------------------- canonical dump
std::vector<uint64_t> engine_dump(const HostEngine& e) {
    std::vector<uint64_t> o;
    const Layout& L = e.L;
    o.push_back((uint64_t)e.m); o.push_back((uint64_t)L.g); o.push_back((uint64_t)L.nodd); o.push_back((uint64_t)L.neven);
    o.push_back((uint64_t)e.t); o.push_back((uint64_t)e.d); o.push_back((uint64_t)(int64_t)e.sigma); o.push_back((uint64_t)e.nf);
    auto put = [&](const Bits& b) { o.insert(o.end(), b.w.begin(), b.w.end()); };
    for (auto& b : e.st.pa) put(b);
    for (auto& b : e.st.pb) put(b);
    for (auto& b : e.st.odd) put(b);
    for (auto& b : e.st.even) put(b);
    put(e.dg.wa); put(e.dg.wb); put(e.dg.o1); put(e.dg.o3); put(e.dg.we);
    const int abo = L.abo(), W = L.full();
    o.insert(o.end(), e.ku.begin(), e.ku.begin() + (size_t)e.d * abo);
    for (auto& k : e.kernel) put(k);
    o.insert(o.end(), e.mcols.begin(), e.mcols.begin() + (size_t)e.t * W);
    o.insert(o.end(), e.ucols.begin(), e.ucols.begin() + (size_t)e.nf * W);
    for (int i = 0; i < e.rank; i++) { o.push_back((uint64_t)e.piv_col[i]); put(e.piv_row[i]); }
    for (auto& c : e.cons) put(c);
    return o;
}

}  // namespace pq
