// pq_device.cu -- device runtime and C-ABI of the GB300 amplitude path.
//
// Objects
//   Target   branch engines of one fixed-variable set (a Simulator's <y|C|x> engines, or the
//            sandwich engines of one measured-qubit set), resident in HBM, plus its
//            boundary map.
//   Plan     the job/item layout of one launch shape (targets x boundary counts), its
//            device buffers and the captured CUDA graph (prepare -> counter reset ->
//            persistent enumeration -> job reduce -> output reduce).  Simulator calls
//            cache one plan per boundary count; pq_batch owns one plan over many targets.
//   pq_sim   Simulator::with_options (src/sim.rs:144-148): compiled path sum, rank
//            strategy, main target, cached marginal targets, stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <array>
#include <chrono>
#include <cmath>
#include <complex>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "pq_host.hpp"
#include "pq_kernels.cuh"
#include "polyq_gb300.h"

namespace pq {

thread_local std::string g_err;
static std::mutex g_mu;
static int g_device = 0;
// Library default launch shape (2^10-step chunks, one unit per lane per work item, 8 warps, two
// blocks per SM with 128 registers, units of 8 chunks): measured best across the plain
// per-circuit, per-boundary and served workloads; large single launches are autotuned.
static pq_tuning g_tuning = {10, 1, 8, 48, 2, 8, 0};

// Chunks per unit a tuning allows: eight accumulating chunks per lane only fit the 128-register
// (two blocks per SM) build of the enumeration kernel.
static int unit_max_of(const pq_tuning &tu) {
    const int u = tu.unit_chunks > 0 ? tu.unit_chunks : 4;
    return tu.blocks_per_sm == 2 ? u : std::min(u, 4);
}
// Per engine: chunks summed from the chunk-sum table are visited one by one in Gray order
// (units of one chunk).
static int unit_max_for(const EngineDev &E, const pq_tuning &tu) {
    return (tu.chunk_tables == 1 && E.ctab) ? 1 : unit_max_of(tu);
}

// A launch takes the fused single-kernel path when each of its outputs sums at most this many
// branches (over all of its branch engines): prepare and enumeration of such an output take a
// few microseconds, less than the launches of a four-kernel sequence.
static const double kSmallMaxBranches = 16384.0;

static pq_status fail(pq_status s, const std::string &m) {
    g_err = m;
    return s;
}
static pq_status cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? PQ_ERR_OUT_OF_MEMORY : PQ_ERR_DEVICE,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define CU(x)                                           \
    do {                                                \
        cudaError_t e_ = (x);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x); \
    } while (0)

static double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// ------------------------------------------------------------------------ device memory
struct DevMem {
    void *p = nullptr;
    size_t n = 0;
    cudaStream_t astream = nullptr;  // set: stream-ordered allocation from the device memory pool
    bool view = false;  // a part of another allocation (not freed here)
    DevMem() = default;
    DevMem(const DevMem &) = delete;
    DevMem &operator=(const DevMem &) = delete;
    ~DevMem() { reset(); }
    void reset() {
        if (p && !view) {
            if (astream) cudaFreeAsync(p, astream);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
        view = false;
    }
    void set_view(void *ptr, size_t bytes) {
        reset();
        p = ptr;
        n = bytes;
        view = true;
    }
    cudaError_t alloc(size_t bytes) {
        reset();
        n = std::max<size_t>(bytes, 16);
        return astream ? cudaMallocAsync(&p, n, astream) : cudaMalloc(&p, n);
    }
    template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};
// Pinned host memory, mapped into the device's address space: kernels of small launches read
// their boundaries from it and write their results to it directly (no copies).
struct HostPinned {
    void *p = nullptr;
    void *d = nullptr;  // the device's address of the same memory
    size_t n = 0;
    bool view = false;  // a part of another allocation (not freed here)
    HostPinned() = default;
    HostPinned(const HostPinned &) = delete;
    HostPinned &operator=(const HostPinned &) = delete;
    ~HostPinned() {
        if (p && !view) cudaFreeHost(p);
    }
    void set_view(const HostPinned &whole, size_t off, size_t bytes) {
        if (p && !view) cudaFreeHost(p);
        p = static_cast<uint8_t *>(whole.p) + off;
        d = static_cast<uint8_t *>(whole.d) + off;
        n = bytes;
        view = true;
    }
    cudaError_t alloc(size_t bytes) {
        if (p && !view) cudaFreeHost(p);
        view = false;
        p = d = nullptr;
        n = std::max<size_t>(bytes, 16);
        cudaError_t e = cudaHostAlloc(&p, n, cudaHostAllocMapped);
        if (e != cudaSuccess) return e;
        return cudaHostGetDevicePointer(&d, p, 0);
    }
    template <class T> T *as() const { return reinterpret_cast<T *>(p); }
    template <class T> T *dev() const { return reinterpret_cast<T *>(d); }
};
template <class T> static cudaError_t upload(DevMem &m, const std::vector<T> &v) {
    cudaError_t e = m.alloc(v.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    if (v.empty()) return e;
    // pageable source: the call returns once the data is staged, so `v` may go away after it
    if (m.astream) return cudaMemcpyAsync(m.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, m.astream);
    return cudaMemcpy(m.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// ------------------------------------------------------------------------ targets
struct Target {
    RankSet rs;
    IoMapHost iom;
    std::vector<std::unique_ptr<DevMem>> mem;  // the engines' tables and blobs (one allocation)
    std::vector<EngineDev> dev;                // rebased onto device addresses
    DevMem iom_mem;
    IoMapDev iom_dev{};
    // the engine records and the boundary map as device structs (launch-independent; the
    // allocation-free entry point launches on them directly)
    DevMem rec_mem;
    const EngineDev *dev_rec = nullptr;
    const IoMapDev *map_rec = nullptr;
    int64_t bytes = 0;
    double branches_per_amp = 0.0;
    // Lower bound of the error bound the FP32 walk reports for any boundary whose sum does not
    // vanish, largest over the branch engines (the bound's boundary-independent terms): above
    // 1e-12 it can never certify a marginal probability
    double fp32_floor = 0.0;
    int max_d = 0, max_rank = 0, max_words = 0;
};

static pq_status upload_target(Target &T, int di_max) {
    T.bytes = 0;
    T.branches_per_amp = 0.0;
    const size_t ne = T.rs.branches.size();
    std::vector<PackedEngine> pks(ne);
    // pack each engine (a copy in the device's coordinate order: even-increment low coordinates
    // first) on host threads: targets of 2^14 engines take seconds on one core
    {
        std::atomic<size_t> next{0};
        std::vector<std::string> errs(ne);
        auto work = [&]() {
            for (size_t i = next++; i < ne; i = next++) {
                try {
                    const auto &e = T.rs.branches[i];
                    std::vector<int> perm;
                    const HostEngine pe = device_order(*e, di_max, perm);
                    EngineTables tb = build_tables(pe, di_max);
                    pks[i] = pack_engine(pe, tb);
                    for (int j = 0; j < 64; j++) pks[i].off.cperm[j] = (uint8_t)(j < pe.d ? perm[(size_t)j] : j);
                } catch (const std::exception &ex) {
                    errs[i] = ex.what();
                }
            }
        };
        const size_t nth = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), ne);
        if (nth <= 1) work();
        else {
            std::vector<std::thread> th;
            for (size_t t = 0; t < nth; t++) th.emplace_back(work);
            for (auto &x : th) x.join();
        }
        for (auto &e : errs)
            if (!e.empty()) return fail(PQ_ERR_INTERNAL, "engine packing: " + e);
    }
    // One allocation per target: the weight tables first, each at an offset aligned to its size
    // (a power of two; placed largest first, every offset is a sum of larger powers of two), so
    // that the walk forms entry addresses by XOR with byte strides; then the engine blobs.
    std::vector<size_t> order(ne), toff(ne, 0), doff(ne, 0);
    for (size_t i = 0; i < ne; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return pks[a].wtab.size() > pks[b].wtab.size(); });
    size_t tab = 0, maxw = 16;
    for (size_t i : order) {
        const size_t wb = pks[i].wtab.size() * sizeof(float);
        if (!wb) continue;
        if ((wb & (wb - 1)) != 0 || wb < 16) return fail(PQ_ERR_INTERNAL, "weight table size not a power of two");
        toff[i] = tab;
        tab += wb;
        maxw = std::max(maxw, wb);
    }
    size_t data = 0;
    for (size_t i = 0; i < ne; i++) {
        doff[i] = data;
        data += (pks[i].blob.size() + 15) & ~(size_t)15;
    }
    auto m = std::make_unique<DevMem>();
    CU(m->alloc(maxw + tab + data));
    uint8_t *tbase = reinterpret_cast<uint8_t *>(((uintptr_t)m->p + maxw - 1) & ~(uintptr_t)(maxw - 1));
    uint8_t *dbase = tbase + tab;
    for (size_t i = 0; i < ne; i++) {
        const PackedEngine &pk = pks[i];
        CU(cudaMemcpy(dbase + doff[i], pk.blob.data(), pk.blob.size(), cudaMemcpyHostToDevice));
        EngineDev dev = rebase_engine(pk.off, dbase + doff[i]);
        if (!pk.wtab.empty()) {
            const size_t wb = pk.wtab.size() * sizeof(float);
            CU(cudaMemcpy(tbase + toff[i], pk.wtab.data(), wb, cudaMemcpyHostToDevice));
            dev.wtab = reinterpret_cast<const float4 *>(tbase + toff[i]);
            if (((uintptr_t)dev.wtab & (wb - 1)) != 0) return fail(PQ_ERR_INTERNAL, "weight table not aligned to its size");
        }
        T.dev.push_back(dev);
        const auto &e = T.rs.branches[i];
        T.branches_per_amp += std::ldexp(1.0, e->d);
        {
            // the FP32 walk's bound has a 1e-12 relative term and the lo-sum term (joint
            // tables); FP64 weights at least 2^DI rounding errors of 2^-53 per chunk sum
            const double mag = pow2_half(dev.mag2 - dev.num_h);
            const double fl = dev.joint ? (1e-12 * dev.sum_abs_bound + dev.errfac) * mag
                                        : std::ldexp(1.0, dev.DI) * 2.220446049250313e-16 * dev.sum_abs_bound * mag;
            T.fp32_floor = std::max(T.fp32_floor, fl);
        }
        T.max_d = std::max(T.max_d, e->d);
        T.max_rank = std::max(T.max_rank, e->rank);
        T.max_words = std::max(T.max_words, e->L.full() + e->wf + 2);
    }
    T.bytes += (int64_t)m->n;
    T.mem.push_back(std::move(m));
    // boundary map: src | cf_pos | cf_src in one allocation
    std::vector<int32_t> blob;
    blob.insert(blob.end(), T.iom.src.begin(), T.iom.src.end());
    blob.insert(blob.end(), T.iom.cf_pos.begin(), T.iom.cf_pos.end());
    blob.insert(blob.end(), T.iom.cf_src.begin(), T.iom.cf_src.end());
    CU(upload(T.iom_mem, blob));
    const int32_t *base = T.iom_mem.as<int32_t>();
    T.iom_dev.nf = (int)T.iom.src.size();
    T.iom_dev.ncf = (int)T.iom.cf_pos.size();
    T.iom_dev.src = base;
    T.iom_dev.cf_pos = base + T.iom.src.size();
    T.iom_dev.cf_src = base + T.iom.src.size() + T.iom.cf_pos.size();
    T.bytes += (int64_t)T.iom_mem.n;
    for (auto &e : T.rs.branches)
        if ((int)T.iom.src.size() != e->nf) return fail(PQ_ERR_INTERNAL, "boundary map does not match engine");
    // engine records then the boundary map, one allocation
    const size_t rb = sizeof(EngineDev) * T.dev.size();
    CU(T.rec_mem.alloc(rb + sizeof(IoMapDev)));
    CU(cudaMemcpy(T.rec_mem.p, T.dev.data(), rb, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(T.rec_mem.as<uint8_t>() + rb, &T.iom_dev, sizeof(IoMapDev), cudaMemcpyHostToDevice));
    T.dev_rec = T.rec_mem.as<EngineDev>();
    T.map_rec = reinterpret_cast<const IoMapDev *>(T.rec_mem.as<uint8_t>() + rb);
    T.bytes += (int64_t)T.rec_mem.n;
    return PQ_OK;
}

// ------------------------------------------------------------------------ plans
// `count` boundaries on target tg, each evaluated over branch engines [eb, ee) (ee < 0: all);
// a segment of one engine may cover only work items [ib, ie) of its jobs (ie < 0: all).
struct Segment {
    Target *tg;
    int64_t count;
    int eb = 0, ee = -1;
    long long ib = 0, ie = -1;
    Segment(Target *t, int64_t c) : tg(t), count(c) {}
    Segment(Target *t, int64_t c, int e0, int e1, long long i0, long long i1)
        : tg(t), count(c), eb(e0), ee(e1), ib(i0), ie(i1) {}
    int engines() const { return (ee < 0 ? (int)tg->dev.size() : ee) - eb; }
};

static const int kMaxSlices = 256;  // item slices of a plan's enumeration (one per SM)
static const size_t kSliceMinEngines = 64;  // launches over more branch engines use slices

struct Plan {
    int nw = 1;
    int64_t nreq = 0;
    int njobs = 0, nout = 0;
    long long nitems = 0;
    double branches = 0.0;  // branches enumerated per run (vanishing boundaries included)
    int smem_words = 8;
    int grid_prep = 1, grid_enum = 1, block_enum = 256;
    int minb = 3;  // enum_kernel<0, minb> instantiation (blocks per SM its registers allow)
    bool any_ctab = false;   // some job can take its chunk sums from a chunk-sum table
    bool fp32_any = false;   // some job walks in FP32 (joint table) without tables
    bool fp32_rest = false;  // some job walks in FP32 even with tables (none for its engine)
    double fp32_floor = 0.0;  // largest over the launch's targets of Target::fp32_floor
    uint64_t last_use = 0;  // recency in the owning simulator's plan cache
    bool graph_ready = false;
    bool eager_used = false, eager_host_used = false;  // first launches, enqueued without a graph
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // small launches: one fused kernel (small_kernel) instead of the four-kernel sequence; host-
    // buffer calls run it on mapped pinned memory through their own graph
    bool fused = false;
    int fused_grid = 1, fused_block = 32;
    size_t fused_smem = 0;
    KArgs args_host{};
    bool graph_host_ready = false;
    bool ran = false;           // a graph of this plan has been launched
    bool last_host_io = false;  // the last launch was a fused one on the mapped host buffers
    cudaGraph_t graph_host = nullptr;
    cudaGraphExec_t gexec_host = nullptr;
    // one device allocation and one mapped host allocation hold all of the plan's buffers
    DevMem arena;
    HostPinned harena;
    DevMem engines, maps, jobs, perm, kinv, istart, jdl, jcpi, jnch, partials, counter, job_vals, job_err, out_jobs,
        x, y, out, err, errflag, ioff;
    HostPinned hx, hy, hout, herr, herrflag;
    std::vector<int> job_engine_d;
    std::vector<JobDev> jobs_host;
    KArgs args{};
    // ev_in/ev_out order the plan's stream against a caller's stream; tev[0..3] bracket
    // prepare | enumerate | reductions inside every launch (event-record nodes in the graph)
    cudaEvent_t ev_in = nullptr, ev_out = nullptr, tev[4] = {nullptr, nullptr, nullptr, nullptr};
    ~Plan() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        if (gexec_host) cudaGraphExecDestroy(gexec_host);
        if (graph_host) cudaGraphDestroy(graph_host);
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
        for (auto &e : tev)
            if (e) cudaEventDestroy(e);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

static int sm_count() {
    static int n = 0;
    if (!n) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, g_device) == cudaSuccess) n = p.multiProcessorCount;
        if (n <= 0) n = 1;
    }
    return n;
}

// Work decomposition of one job (fixed per job, so a boundary's result does not depend on
// what else shares the launch): chunks of 2^dl Gray steps, 32 * cpl chunks per item.
// `light`: a one-shot plan (serving waves): device buffers come from the stream-ordered pool
// and are released in stream order; no pinned host staging.
// `prepare_only`: job records for the prepare kernel alone (Monte-Carlo sampling of engines
// beyond the enumeration's limits): no dimension cap, no work items.
static pq_status build_plan(const std::vector<Segment> &segs, int nw, cudaStream_t stream, const pq_tuning &tu,
                            Plan &P, bool light = false, bool prepare_only = false) {
    P.nw = nw;
    P.stream = stream;
    if (!P.stream) {
        CU(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking));
        P.own_stream = true;
    }
    if (light) P.arena.astream = P.stream;  // one-shot plans: from the stream-ordered pool
    {
        // (boundary, branch engine) jobs are indexed with 32-bit integers on the device
        double total = 0.0;
        for (const auto &sg : segs) total += (double)sg.count * (double)sg.engines();
        if (total > (double)(1 << 28))
            return fail(PQ_ERR_INVALID_ARG, "boundaries x branch engines above 2^28 in one launch; split the call");
    }
    for (const auto &sg : segs) P.fp32_floor = std::max(P.fp32_floor, sg.tg->fp32_floor);
    std::vector<EngineDev> eng;
    std::vector<IoMapDev> maps;
    std::vector<JobDev> jobs;
    std::vector<int> out_jobs;
    std::vector<int> jd;
    std::vector<long long> jib, jie;  // per job: work-item range [ib, ie) (ie < 0: all)
    bool ranged = false;
    int64_t req = 0;
    int maxw = 8;
    for (size_t si = 0; si < segs.size(); si++) {
        const Segment &sg = segs[si];
        Target *T = sg.tg;
        const int e0 = sg.eb, e1 = sg.ee < 0 ? (int)T->dev.size() : sg.ee;
        if (e0 < 0 || e1 > (int)T->dev.size() || e0 >= e1 || (sg.ie >= 0 && (e1 - e0 != 1 || sg.ib >= sg.ie)))
            return fail(PQ_ERR_INTERNAL, "bad launch segment");
        ranged = ranged || sg.ie >= 0 || sg.ib > 0;
        const int ebase = (int)eng.size();
        for (int b = e0; b < e1; b++) {
            const EngineDev &e = T->dev[(size_t)b];
            if (e.rank > kMaxPivots || (e.d > kMaxD && !prepare_only))
                return fail(PQ_ERR_UNSUPPORTED, "branch engine outside kernel limits");
            if (e.d > tu.max_branch_dim && !prepare_only)
                return fail(PQ_ERR_ADMISSION_REFUSED, "branch dimension " + std::to_string(e.d) + " above the cap " +
                                                          std::to_string(tu.max_branch_dim));
            eng.push_back(e);
        }
        maps.push_back(T->iom_dev);
        maxw = std::max(maxw, T->max_words);
        for (int64_t r = 0; r < sg.count; r++, req++) {
            out_jobs.push_back((int)jobs.size());
            for (int b = e0; b < e1; b++) {
                JobDev J;
                std::memset(&J, 0, sizeof(J));
                J.engine = ebase + (b - e0);
                J.iomap = (int)si;
                J.req = (int)req;
                J.out = (int)req;
                jobs.push_back(J);
                jd.push_back(T->dev[(size_t)b].d);
                jib.push_back(sg.ib);
                jie.push_back(sg.ie);
            }
        }
    }
    out_jobs.push_back((int)jobs.size());
    P.nreq = req;
    P.njobs = (int)jobs.size();
    P.nout = (int)req;
    P.smem_words = maxw;
    if (P.njobs == 0) return fail(PQ_ERR_INVALID_ARG, "empty launch");
    // item layout: jobs in decreasing branch dimension (longest work first); equal dimensions
    // grouped by engine, so warps running at the same time share that engine's tables in L1
    std::vector<int> perm((size_t)P.njobs), kinv((size_t)P.njobs), jdl((size_t)P.njobs);
    std::vector<unsigned> jcpi((size_t)P.njobs);
    std::vector<unsigned long long> jnch((size_t)P.njobs);
    for (int j = 0; j < P.njobs; j++) perm[j] = j;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) {
        if (jd[a] != jd[b]) return jd[a] > jd[b];
        return jobs[a].engine < jobs[b].engine;
    });
    std::vector<long long> istart((size_t)P.njobs + 1, 0);
    P.branches = 0.0;
    for (int k = 0; k < P.njobs; k++) {
        int j = perm[k];
        kinv[j] = k;
        const EngineDev &E = eng[jobs[j].engine];
        if (prepare_only) {
            jdl[j] = 0;
            jnch[j] = 0;
            jcpi[j] = 1;
        } else {
            job_shape(E, tu.chunks_per_lane, unit_max_for(E, tu), jdl[j], jnch[j], jcpi[j]);
        }
        const long long nit = (long long)((jnch[j] + jcpi[j] - 1) / jcpi[j]);
        const long long i1 = jie[j] < 0 ? nit : std::min<long long>(jie[j], nit);
        const long long i0 = std::min<long long>(jib[j], i1);
        jib[j] = i0;
        istart[k + 1] = istart[k] + (i1 - i0);
        P.branches += prepare_only || nit == 0 ? std::ldexp(1.0, E.d)
                                               : std::ldexp(1.0, E.d) * (double)(i1 - i0) / (double)nit;
        const bool covered = E.ctab && (jdl[j] & 255) == E.DI;
        P.any_ctab = P.any_ctab || covered;
        P.fp32_any = P.fp32_any || E.joint;
        P.fp32_rest = P.fp32_rest || (E.joint && !covered);
    }
    P.nitems = istart[P.njobs];
    {
        // every device buffer is a 256-byte aligned part of one allocation; the records go up in
        // one copy (pageable source: the call returns once the data is staged)
        struct Part {
            DevMem *m;
            size_t bytes;
            const void *src;
        };
        auto vb = [](const auto &v) { return v.size() * sizeof(v[0]); };
        std::vector<Part> parts = {{&P.engines, vb(eng), eng.data()},   {&P.maps, vb(maps), maps.data()},
                                   {&P.jobs, vb(jobs), jobs.data()},    {&P.perm, vb(perm), perm.data()},
                                   {&P.kinv, vb(kinv), kinv.data()},    {&P.istart, vb(istart), istart.data()},
                                   {&P.jdl, vb(jdl), jdl.data()},       {&P.jcpi, vb(jcpi), jcpi.data()},
                                   {&P.jnch, vb(jnch), jnch.data()},    {&P.out_jobs, vb(out_jobs), out_jobs.data()}};
        if (ranged) parts.push_back({&P.ioff, vb(jib), jib.data()});
        const size_t nup = parts.size();
        parts.push_back({&P.partials, (size_t)P.nitems * sizeof(double2), nullptr});
        parts.push_back({&P.counter, sizeof(unsigned long long) * kMaxSlices, nullptr});
        parts.push_back({&P.job_vals, (size_t)P.njobs * sizeof(double2), nullptr});
        parts.push_back({&P.job_err, (size_t)P.njobs * sizeof(double), nullptr});
        parts.push_back({&P.x, (size_t)P.nreq * nw * 8, nullptr});
        parts.push_back({&P.y, (size_t)P.nreq * nw * 8, nullptr});
        parts.push_back({&P.out, (size_t)P.nout * 2 * sizeof(double), nullptr});
        parts.push_back({&P.err, (size_t)P.nout * sizeof(double), nullptr});
        parts.push_back({&P.errflag, sizeof(int), nullptr});
        std::vector<size_t> off(parts.size());
        size_t total = 0, up_end = 0;
        for (size_t i = 0; i < parts.size(); i++) {
            off[i] = total;
            total += (std::max<size_t>(parts[i].bytes, 16) + 255) & ~(size_t)255;
            if (i + 1 == nup) up_end = total;
        }
        CU(P.arena.alloc(total));
        std::vector<uint8_t> stage(up_end, 0);
        for (size_t i = 0; i < nup; i++)
            if (parts[i].bytes) std::memcpy(stage.data() + off[i], parts[i].src, parts[i].bytes);
        for (size_t i = 0; i < parts.size(); i++)
            parts[i].m->set_view(P.arena.as<uint8_t>() + off[i], std::max<size_t>(parts[i].bytes, 16));
        if (light) CU(cudaMemcpyAsync(P.arena.p, stage.data(), up_end, cudaMemcpyHostToDevice, P.stream));
        else CU(cudaMemcpy(P.arena.p, stage.data(), up_end, cudaMemcpyHostToDevice));
    }
    CU(cudaEventCreateWithFlags(&P.ev_in, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&P.ev_out, cudaEventDisableTiming));
    for (auto &e : P.tev) CU(cudaEventCreate(&e));
    if (!light) {
        // mapped host buffers of the fused host-buffer path, parts of one pinned allocation
        const size_t bx = (size_t)P.nreq * nw * 8, bo = (size_t)P.nout * 16, be = (size_t)P.nout * 8;
        auto r = [](size_t b) { return (std::max<size_t>(b, 16) + 255) & ~(size_t)255; };
        CU(P.harena.alloc(2 * r(bx) + r(bo) + r(be) + r(4)));
        size_t o = 0;
        P.hx.set_view(P.harena, o, bx);
        o += r(bx);
        P.hy.set_view(P.harena, o, bx);
        o += r(bx);
        P.hout.set_view(P.harena, o, bo);
        o += r(bo);
        P.herr.set_view(P.harena, o, be);
        o += r(be);
        P.herrflag.set_view(P.harena, o, sizeof(int));
    }
    P.jobs_host = jobs;
    KArgs &a = P.args;
    a.engines = P.engines.as<EngineDev>();
    a.maps = P.maps.as<IoMapDev>();
    a.jobs = P.jobs.as<JobDev>();
    a.njobs = P.njobs;
    a.perm = P.perm.as<int>();
    a.kinv = P.kinv.as<int>();
    a.istart = P.istart.as<long long>();
    a.jdl = P.jdl.as<int>();
    a.jcpi = P.jcpi.as<unsigned>();
    a.jnch = P.jnch.as<unsigned long long>();
    a.nitems = P.nitems;
    a.partials = P.partials.as<double2>();
    a.counter = P.counter.as<unsigned long long>();
    // item slices per SM where the launch spans many engines' tables (batches): with few
    // engines their tables stay in L1 anyway and one counter balances best
    a.nslices = eng.size() > kSliceMinEngines ? std::min(sm_count(), kMaxSlices) : 1;
    a.use_ctab = tu.chunk_tables == 1 ? 1 : 0;
    a.job_vals = P.job_vals.as<double2>();
    a.job_err = P.job_err.as<double>();
    a.out_jobs = P.out_jobs.as<int>();
    a.nout = P.nout;
    a.out = P.out.as<double>();
    a.err = P.err.as<double>();
    a.out_prob = 0;
    a.xs = P.x.as<uint64_t>();
    a.ys = P.y.as<uint64_t>();
    a.nw = nw;
    a.smem_words = P.smem_words;
    a.dbg = nullptr;
    a.errflag = P.errflag.as<int>();
    a.ioff = ranged ? P.ioff.as<long long>() : nullptr;
    const int bw = std::max(1, std::min(8, tu.block_warps));
    P.block_enum = 32 * bw;
    P.minb = (tu.blocks_per_sm >= 2 && tu.blocks_per_sm <= 4) ? tu.blocks_per_sm : 3;
    int occ = 0;
    if (P.minb == 4) CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, enum_kernel<0, 4>, P.block_enum, 0));
    else if (P.minb == 2) CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, enum_kernel<0, 2>, P.block_enum, 0));
    else CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, enum_kernel<0, 3>, P.block_enum, 0));
    occ = std::max(occ, 1);
    long long want = (long long)sm_count() * occ;
    P.grid_enum = (int)std::max(1LL, std::min<long long>(want, (P.nitems + bw - 1) / bw));
    P.grid_prep = std::max(1, std::min((P.njobs + 3) / 4, 65535));
    if ((size_t)4 * P.smem_words * 8 > 48 * 1024) {
        CU(cudaFuncSetAttribute(prepare_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(4 * P.smem_words * 8)));
    }
    // one fused kernel when every output is small: at most kSmallMaxJobs branch engines and
    // kSmallMaxBranches branches summed over them
    if (!prepare_only) {
        bool small = true;
        int maxj = 1;
        for (const auto &sg : segs) {
            const int nb = sg.engines();
            small = small && nb <= kSmallMaxJobs && sg.tg->branches_per_amp <= kSmallMaxBranches;
            maxj = std::max(maxj, nb);
        }
        const int wpb = std::min(maxj, 8);
        const size_t smem = (size_t)(2 * nw + wpb * P.smem_words) * 8;
        // static (SmallShared) plus dynamic shared memory within the 48 KB a launch gets without opt-in
        if (small && smem + sizeof(SmallShared) + 256 <= 48 * 1024) {
            P.fused = true;
            P.fused_block = 32 * wpb;
            P.fused_smem = smem;
            P.fused_grid = (int)std::max<long long>(1, std::min<long long>(P.nout, (long long)sm_count() * 8));
            if (!light) {
                P.args_host = P.args;
                P.args_host.xs = P.hx.dev<uint64_t>();
                P.args_host.ys = P.hy.dev<uint64_t>();
                P.args_host.out = P.hout.dev<double>();
                P.args_host.err = P.herr.dev<double>();
                P.args_host.errflag = P.herrflag.dev<int>();
            }
        }
    }
    return PQ_OK;
}

// Enqueue the core launch sequence on P.stream (capturable).  mode 1 walks in FP64; ctab >= 0
// overrides the plan's use of chunk-sum tables (which, where they apply, are FP64 in either mode).
// `io` (optional) replaces the plan's boundary, result and flag pointers (the mapped host
// buffers of a fused launch).
static cudaError_t enqueue_core(Plan &P, int mode, int ctab = -1, const KArgs *io = nullptr) {
    cudaError_t e;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(P.stream, &cs)) != cudaSuccess) return e;
    // timing events become event-record nodes of the graph while capturing
    const unsigned evflag = cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (P.fused && mode == 0 && (ctab < 0 || ctab == P.args.use_ctab)) {
        KArgs args = io ? *io : P.args;
        if ((e = cudaMemsetAsync(args.errflag, 0, sizeof(int), P.stream)) != cudaSuccess) return e;
        if ((e = cudaEventRecordWithFlags(P.tev[0], P.stream, evflag)) != cudaSuccess) return e;
        if ((e = cudaEventRecordWithFlags(P.tev[1], P.stream, evflag)) != cudaSuccess) return e;
        if (P.minb == 2) small_kernel<2><<<P.fused_grid, P.fused_block, P.fused_smem, P.stream>>>(args);
        else small_kernel<3><<<P.fused_grid, P.fused_block, P.fused_smem, P.stream>>>(args);
        if ((e = cudaEventRecordWithFlags(P.tev[2], P.stream, evflag)) != cudaSuccess) return e;
        if ((e = cudaEventRecordWithFlags(P.tev[3], P.stream, evflag)) != cudaSuccess) return e;
        return cudaGetLastError();
    }
    e = cudaMemsetAsync(P.errflag.p, 0, sizeof(int), P.stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(P.counter.p, 0, P.counter.n, P.stream);
    if (e != cudaSuccess) return e;
    KArgs args = P.args;
    args.fp64_mode = mode == 1 ? 1 : 0;
    if (ctab >= 0) args.use_ctab = ctab;
    if ((e = cudaEventRecordWithFlags(P.tev[0], P.stream, evflag)) != cudaSuccess) return e;
    prepare_kernel<<<P.grid_prep, 128, (size_t)4 * P.smem_words * 8, P.stream>>>(args);
    if ((e = cudaEventRecordWithFlags(P.tev[1], P.stream, evflag)) != cudaSuccess) return e;
    if (mode == 1) enum_kernel<1><<<P.grid_enum, P.block_enum, 0, P.stream>>>(args);
    else if (P.minb == 4) enum_kernel<0, 4><<<P.grid_enum, P.block_enum, 0, P.stream>>>(args);
    else if (P.minb == 2) enum_kernel<0, 2><<<P.grid_enum, P.block_enum, 0, P.stream>>>(args);
    else enum_kernel<0, 3><<<P.grid_enum, P.block_enum, 0, P.stream>>>(args);
    if ((e = cudaEventRecordWithFlags(P.tev[2], P.stream, evflag)) != cudaSuccess) return e;
    job_reduce_kernel<<<(P.njobs + 255) / 256, 256, 0, P.stream>>>(args);
    out_reduce_kernel<<<(P.nout + 255) / 256, 256, 0, P.stream>>>(args);
    if ((e = cudaEventRecordWithFlags(P.tev[3], P.stream, evflag)) != cudaSuccess) return e;
    return cudaGetLastError();
}

static pq_status capture(Plan &P, const KArgs *io, cudaGraph_t &graph, cudaGraphExec_t &gexec) {
    CU(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_core(P, 0, -1, io);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(P.stream, &g);
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(e, "capture"); }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    graph = g;
    CU(cudaGraphInstantiate(&gexec, graph, 0));
    return PQ_OK;
}

// A plan's first launch is enqueued directly (a plan used once pays for no graph); later
// launches replay the graph captured at the second.
static pq_status launch_graph(Plan &P) {
    if (!P.graph_ready && !P.eager_used) {
        CU(enqueue_core(P, 0, -1, nullptr));
        P.eager_used = true;
        P.ran = true;
        P.last_host_io = false;
        return PQ_OK;
    }
    if (!P.graph_ready) {
        pq_status st = capture(P, nullptr, P.graph, P.gexec);
        if (st != PQ_OK) return st;
        P.graph_ready = true;
    }
    CU(cudaGraphLaunch(P.gexec, P.stream));
    P.ran = true;
    P.last_host_io = false;
    return PQ_OK;
}

// Fused plans on host buffers: the kernel reads the boundaries from, and writes the results to,
// the plan's mapped pinned buffers.  The timing events are shared with launch_graph's graph.
static pq_status launch_graph_host(Plan &P) {
    if (!P.graph_host_ready && !P.eager_host_used) {
        CU(enqueue_core(P, 0, -1, &P.args_host));
        P.eager_host_used = true;
        P.ran = true;
        P.last_host_io = true;
        return PQ_OK;
    }
    if (!P.graph_host_ready) {
        pq_status st = capture(P, &P.args_host, P.graph_host, P.gexec_host);
        if (st != PQ_OK) return st;
        P.graph_host_ready = true;
    }
    CU(cudaGraphLaunch(P.gexec_host, P.stream));
    P.ran = true;
    P.last_host_io = true;
    return PQ_OK;
}

// Host-buffer run: H2D boundaries, graph, D2H results, wait.
// What a host run must certify to 1e-12 absolute: nothing (amplitudes carry their bound), the
// probability |a|^2, or the real part (a marginal probability).
enum Certify { CERT_NONE = 0, CERT_PROB = 1, CERT_REAL = 2 };

// Host-buffer run: H2D boundaries, graph, D2H results, wait.  Under CERT_PROB / CERT_REAL, when
// the FP32 bound cannot certify 1e-12 absolute, the same launch shape is re-run from the
// chunk-sum tables (FP64) and then, if still needed, with FP64 weights and accumulation.
static pq_status run_host(Plan &P, const uint64_t *x, const uint64_t *y, double *out, double *err, Certify cert) {
    const size_t bw = (size_t)P.nreq * P.nw * 8;
    std::memcpy(P.hx.p, x, bw);
    std::memcpy(P.hy.p, y, bw);
    pq_status st;
    // a marginal whose FP32 walk cannot show 1e-12 on any boundary (the floor of its bound is
    // above it) starts at the level that can
    const bool ctab0 = P.args.use_ctab != 0;
    const bool skip_fp32 = cert == CERT_REAL && P.fp32_floor > 1e-12 &&
                           ((P.any_ctab && !ctab0) || (ctab0 ? P.fp32_rest : P.fp32_any));
    if (skip_fp32) {
        CU(cudaMemcpyAsync(P.x.p, P.hx.p, bw, cudaMemcpyHostToDevice, P.stream));
        CU(cudaMemcpyAsync(P.y.p, P.hy.p, bw, cudaMemcpyHostToDevice, P.stream));
        *P.herrflag.as<int>() = 0;
    } else if (P.fused) {
        // one graph launch: the fused kernel reads and writes the mapped buffers
        st = launch_graph_host(P);
        if (st != PQ_OK) return st;
    } else {
        CU(cudaMemcpyAsync(P.x.p, P.hx.p, bw, cudaMemcpyHostToDevice, P.stream));
        CU(cudaMemcpyAsync(P.y.p, P.hy.p, bw, cudaMemcpyHostToDevice, P.stream));
        st = launch_graph(P);
        if (st != PQ_OK) return st;
        CU(cudaMemcpyAsync(P.hout.p, P.out.p, (size_t)P.nout * 16, cudaMemcpyDeviceToHost, P.stream));
        CU(cudaMemcpyAsync(P.herr.p, P.err.p, (size_t)P.nout * 8, cudaMemcpyDeviceToHost, P.stream));
        CU(cudaMemcpyAsync(P.herrflag.p, P.errflag.p, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
    }
    if (!skip_fp32) CU(cudaStreamSynchronize(P.stream));
    if (*P.herrflag.as<int>()) return fail(PQ_ERR_INTERNAL, "device self-check failed (odd Z8 increment)");
    const double *ho = P.hout.as<double>();
    const double *he = P.herr.as<double>();
    auto bound_of = [&](int o) {
        if (cert == CERT_PROB) {
            const double a = std::sqrt(ho[2 * o] * ho[2 * o] + ho[2 * o + 1] * ho[2 * o + 1]);
            return he[o] * (2.0 * a + he[o]);
        }
        return he[o];
    };
    auto uncertified = [&]() {
        for (int o = 0; o < P.nout; o++)
            if (bound_of(o) > 1e-12) return true;
        return false;
    };
    bool staged = !P.fused || skip_fp32;  // boundaries in the plan's device buffers
    auto rerun = [&](int mode, int ctab) -> pq_status {
        if (!staged) {
            CU(cudaMemcpyAsync(P.x.p, P.hx.p, bw, cudaMemcpyHostToDevice, P.stream));
            CU(cudaMemcpyAsync(P.y.p, P.hy.p, bw, cudaMemcpyHostToDevice, P.stream));
            staged = true;
        }
        CU(enqueue_core(P, mode, ctab));
        CU(cudaMemcpyAsync(P.hout.p, P.out.p, (size_t)P.nout * 16, cudaMemcpyDeviceToHost, P.stream));
        CU(cudaMemcpyAsync(P.herr.p, P.err.p, (size_t)P.nout * 8, cudaMemcpyDeviceToHost, P.stream));
        CU(cudaStreamSynchronize(P.stream));
        return PQ_OK;
    };
    if (cert != CERT_NONE && (skip_fp32 || uncertified())) {
        bool tables = ctab0;
        bool have = !skip_fp32;  // the host buffers hold an evaluation of these boundaries
        if (P.any_ctab && !tables) {
            st = rerun(0, 1);
            if (st != PQ_OK) return st;
            tables = true;
            have = true;
        }
        // then the FP64 walk for the jobs that walked in FP32 (the tables stay where they
        // apply; jobs without a joint table already used FP64 weights, so a rerun would repeat
        // them)
        if ((!have || uncertified()) && (tables ? P.fp32_rest : P.fp32_any)) {
            st = rerun(1, tables ? 1 : 0);
            if (st != PQ_OK) return st;
            have = true;
        }
        if (!have) {
            st = rerun(0, -1);
            if (st != PQ_OK) return st;
        }
    }
    for (int o = 0; o < P.nout; o++) {
        if (cert == CERT_PROB) {
            double re = ho[2 * o], im = ho[2 * o + 1];
            out[o] = re * re + im * im;
        } else {
            out[2 * o] = ho[2 * o];
            out[2 * o + 1] = ho[2 * o + 1];
        }
        if (err) err[o] = bound_of(o);
    }
    return PQ_OK;
}

// Device-buffer run ordered after, and waited for by, the caller's `stream` (CUDA convention:
// NULL is the legacy default stream).  No host synchronisation.
static pq_status run_device(Plan &P, const uint64_t *x, const uint64_t *y, double *out, double *err,
                            cudaStream_t stream) {
    const size_t bw = (size_t)P.nreq * P.nw * 8;
    CU(cudaEventRecord(P.ev_in, stream));
    CU(cudaStreamWaitEvent(P.stream, P.ev_in, 0));
    if (x != P.x.as<uint64_t>()) CU(cudaMemcpyAsync(P.x.p, x, bw, cudaMemcpyDeviceToDevice, P.stream));
    if (y != P.y.as<uint64_t>()) CU(cudaMemcpyAsync(P.y.p, y, bw, cudaMemcpyDeviceToDevice, P.stream));
    pq_status st = launch_graph(P);
    if (st != PQ_OK) return st;
    if (out && out != P.out.as<double>())
        CU(cudaMemcpyAsync(out, P.out.p, (size_t)P.nout * 16, cudaMemcpyDeviceToDevice, P.stream));
    if (err && err != P.err.as<double>())
        CU(cudaMemcpyAsync(err, P.err.p, (size_t)P.nout * 8, cudaMemcpyDeviceToDevice, P.stream));
    CU(cudaEventRecord(P.ev_out, P.stream));
    CU(cudaStreamWaitEvent(stream, P.ev_out, 0));
    return PQ_OK;
}

// Device times (ms) of the last completed launch: prepare, enumerate, reductions.
static pq_status last_kernel_ms(Plan &P, float *ms) {
    for (int i = 0; i < 3; i++) {
        cudaError_t e = cudaEventElapsedTime(&ms[i], P.tev[i], P.tev[i + 1]);
        if (e != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime");
    }
    return PQ_OK;
}

}  // namespace pq

using namespace pq;

// ------------------------------------------------------------------------ simulator
struct pq_sim {
    int device = 0;
    Circuit circ;
    PathSum ps;
    int strategy = 0, pairs = 0;
    int di_max = 10;
    pq_tuning tu{};  // launch shape of this simulator's plans (library default at creation, or autotuned)
    int nw = 1;
    bool host_only = false;
    Target main;
    cudaStream_t stream = nullptr;
    double build_s = 0.0;
    std::mutex mu;
    std::map<int64_t, std::unique_ptr<Plan>> plans;
    uint64_t use_clock = 0;
    bool have_sw = false;
    PathSum sw;
    std::vector<int> junction;
    std::vector<uint8_t> jneg;
    struct Marg {
        Target tg;
        std::unique_ptr<Plan> plan;                          // one boundary (pq_marginal)
        std::map<int64_t, std::unique_ptr<Plan>> many;       // n boundaries (sampling)
    };
    std::map<std::vector<int>, std::unique_ptr<Marg>> marg;
    // resident mode (pq_sim_set_resident): single-boundary amplitudes served by resident_kernel
    struct Resident {
        std::unique_ptr<Plan> plan;  // its own one-boundary plan (fused)
        HostPinned box;              // ResidentBox + 2 nw boundary words, mapped
        cudaStream_t stream = nullptr;
        cudaEvent_t ev = nullptr;    // recorded after each launch: complete once the kernel returned
        bool launched = false;
        unsigned seq = 0;
        double idle_s = 0.0;
        ~Resident() {
            if (ev) cudaEventDestroy(ev);
            if (stream) cudaStreamDestroy(stream);
        }
    };
    std::unique_ptr<Resident> res;
    ~pq_sim() {
        res.reset();
        plans.clear();
        marg.clear();
        if (stream) cudaStreamDestroy(stream);
    }
};

struct pq_batch {
    std::vector<pq_sim *> sims;
    int nw = 1;
    std::vector<Segment> segs;
    pq_tuning tu{};
    std::unique_ptr<Plan> plan;
    std::mutex mu;
};

static int words_for(int nq) { return std::max(1, (nq + 63) / 64); }
static const size_t kMaxPlans = 16;  // cached launch plans per simulator (boundary counts)
static const size_t kPrepWords = 12;  // u64 words per job of pq_debug_prepare

// puts for <y|C|x> (src/pathsum.rs:430-450)
static IoMapHost main_iomap(const PathSum &ps) {
    std::vector<std::pair<int, int32_t>> puts;
    for (int q = 0; q < ps.nq; q++) puts.push_back({q, io_src(q, 0, 0)});
    for (int q = 0; q < ps.nq; q++) puts.push_back({ps.outputs[q], io_src(q, 1, ps.out_neg[q])});
    return build_iomap(puts);
}

extern "C" {

PQ_API const char *pq_version(void) { return "polyq-gb300 1.0 (sm_103a)"; }
PQ_API const char *pq_last_error(void) { return g_err.c_str(); }

PQ_API pq_status pq_init(int32_t device) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(PQ_ERR_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= n) return fail(PQ_ERR_INVALID_ARG, "device index out of range");
    g_device = device;
    CU(cudaSetDevice(device));
    return PQ_OK;
}

PQ_API pq_status pq_set_default_tuning(const pq_tuning *t) {
    if (!t) return fail(PQ_ERR_INVALID_ARG, "null tuning");
    std::lock_guard<std::mutex> lk(g_mu);
    pq_tuning n = g_tuning;
    if (t->inner_dims) {
        if (t->inner_dims < 4 || t->inner_dims > 14) return fail(PQ_ERR_INVALID_ARG, "inner_dims must be in 4..14");
        n.inner_dims = t->inner_dims;
    }
    if (t->chunks_per_lane) {
        if (t->chunks_per_lane < 1 || t->chunks_per_lane > 64) return fail(PQ_ERR_INVALID_ARG, "chunks_per_lane in 1..64");
        n.chunks_per_lane = t->chunks_per_lane;
    }
    if (t->block_warps) {
        if (t->block_warps < 1 || t->block_warps > 8) return fail(PQ_ERR_INVALID_ARG, "block_warps in 1..8");
        n.block_warps = t->block_warps;
    }
    if (t->max_branch_dim) {
        if (t->max_branch_dim < 1 || t->max_branch_dim > kMaxD) return fail(PQ_ERR_INVALID_ARG, "max_branch_dim in 1..62");
        n.max_branch_dim = t->max_branch_dim;
    }
    if (t->chunk_tables) {
        if (t->chunk_tables != 1 && t->chunk_tables != 2) return fail(PQ_ERR_INVALID_ARG, "chunk_tables is 1 (on) or 2 (off)");
        n.chunk_tables = t->chunk_tables;
    }
    if (t->unit_chunks) {
        if (t->unit_chunks != 1 && t->unit_chunks != 2 && t->unit_chunks != 4 && t->unit_chunks != 8)
            return fail(PQ_ERR_INVALID_ARG, "unit_chunks is 1, 2, 4 or 8");
        n.unit_chunks = t->unit_chunks;
    }
    if (t->blocks_per_sm) {
        if (t->blocks_per_sm < 2 || t->blocks_per_sm > 4) return fail(PQ_ERR_INVALID_ARG, "blocks_per_sm is 2, 3 or 4");
        n.blocks_per_sm = t->blocks_per_sm;
    }
    g_tuning = n;
    return PQ_OK;
}
PQ_API pq_status pq_get_default_tuning(pq_tuning *t) {
    if (!t) return fail(PQ_ERR_INVALID_ARG, "null tuning");
    std::lock_guard<std::mutex> lk(g_mu);
    *t = g_tuning;
    return PQ_OK;
}

static pq_status sim_build_host(const pq_circuit_desc *c, int32_t strategy, int32_t pairs, std::unique_ptr<pq_sim> &S) {
    if (!c) return fail(PQ_ERR_INVALID_ARG, "null argument");
    if (strategy < 0 || strategy > 2) return fail(PQ_ERR_INVALID_ARG, "strategy must be 0 (auto), 1 (cached) or 2 (pairs)");
    if (strategy == 2 && pairs < 0) return fail(PQ_ERR_INVALID_ARG, "negative pair count");
    std::string why = validate_circuit(c->num_qubits, c->num_gates, c->op, c->q0, c->q1);
    if (!why.empty()) return fail(PQ_ERR_INVALID_ARG, why);
    if (c->num_gates > 0 && !c->phase) return fail(PQ_ERR_INVALID_ARG, "null phase array");
    S = std::make_unique<pq_sim>();
    S->device = g_device;
    S->circ.nq = c->num_qubits;
    for (int i = 0; i < c->num_gates; i++) S->circ.gates.push_back(Gate{c->op[i], c->q0[i], c->q1[i], c->phase[i]});
    S->strategy = strategy;
    S->pairs = pairs;
    S->nw = words_for(c->num_qubits);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        S->tu = g_tuning;
        S->di_max = g_tuning.inner_dims;
    }
    try {
        S->ps = PathSum::compile(S->circ);
        S->main.iom = main_iomap(S->ps);
        S->main.rs = build_rank(S->ps, S->main.iom.fixed, strategy, pairs);
    } catch (const std::exception &e) {
        return fail(PQ_ERR_INTERNAL, std::string("engine build: ") + e.what());
    }
    S->main.branches_per_amp = 0.0;
    for (auto &e : S->main.rs.branches) S->main.branches_per_amp += std::ldexp(1.0, e->d);
    return PQ_OK;
}

PQ_API pq_status pq_sim_create(const pq_circuit_desc *c, int32_t strategy, int32_t pairs, pq_sim **out) {
    if (!c || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(PQ_ERR_NO_DEVICE, "no CUDA device visible");
    const double t0 = now_s();
    std::unique_ptr<pq_sim> S;
    pq_status st = sim_build_host(c, strategy, pairs, S);
    if (st != PQ_OK) return st;
    CU(cudaSetDevice(S->device));
    st = upload_target(S->main, S->di_max);
    if (st != PQ_OK) return st;
    CU(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    S->build_s = now_s() - t0;
    *out = S.release();
    return PQ_OK;
}

PQ_API pq_status pq_analyze(const pq_circuit_desc *c, int32_t strategy, int32_t pairs, pq_sim **out) {
    if (!c || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    const double t0 = now_s();
    std::unique_ptr<pq_sim> S;
    pq_status st = sim_build_host(c, strategy, pairs, S);
    if (st != PQ_OK) return st;
    S->host_only = true;
    S->build_s = now_s() - t0;
    *out = S.release();
    return PQ_OK;
}

static pq_status resident_stop(pq_sim *s);

PQ_API void pq_sim_destroy(pq_sim *s) {
    if (!s) return;
    if (s->host_only) {
        delete s;
        return;
    }
    cudaSetDevice(s->device);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        resident_stop(s);
    }
    if (s->stream) cudaStreamSynchronize(s->stream);
    delete s;
}

PQ_API pq_status pq_sim_stats(const pq_sim *s, pq_stats *o) {
    if (!s || !o) return fail(PQ_ERR_INVALID_ARG, "null argument");
    const HostEngine &e = *s->main.rs.branches[0];
    o->free_vars = e.m;
    o->planes = e.L.g;
    o->lines = e.L.nodd;
    o->radical = e.L.neven;
    o->terms = e.t;
    o->branch_dim = e.d;
    o->pairs = s->main.rs.pairs;
    o->num_branches = (int64_t)s->main.rs.branches.size();
    o->branches_per_amplitude = s->main.branches_per_amp;
    {
        std::lock_guard<std::mutex> lk(const_cast<pq_sim *>(s)->mu);
        o->device_bytes = s->main.bytes;
        for (const auto &kv : s->marg) o->device_bytes += kv.second->tg.bytes;
    }
    o->build_seconds = s->build_s;
    return PQ_OK;
}

static pq_status sim_plan(pq_sim *s, int64_t n, Plan **out) {
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    auto it = s->plans.find(n);
    if (it != s->plans.end()) {
        it->second->last_use = ++s->use_clock;
        *out = it->second.get();
        return PQ_OK;
    }
    // plans are cached per boundary count; past kMaxPlans, the least recently used one goes
    // (after the simulator's stream drains: device-pointer calls may still be running on it)
    if (s->plans.size() >= kMaxPlans) {
        auto victim = s->plans.begin();
        for (auto pi = s->plans.begin(); pi != s->plans.end(); ++pi)
            if (pi->second->last_use < victim->second->last_use) victim = pi;
        CU(cudaStreamSynchronize(s->stream));
        s->plans.erase(victim);
    }
    auto P = std::make_unique<Plan>();
    std::vector<Segment> segs{{&s->main, n}};
    pq_status st = build_plan(segs, s->nw, s->stream, s->tu, *P);
    if (st != PQ_OK) return st;
    P->last_use = ++s->use_clock;
    *out = P.get();
    s->plans[n] = std::move(P);
    return PQ_OK;
}

static pq_status check_n(int64_t n) {
    if (n <= 0 || n > (1LL << 24)) return fail(PQ_ERR_INVALID_ARG, "boundary count must be in 1..2^24");
    return PQ_OK;
}

// Resident mode.  Stop the resident kernel (it returns at its next poll) and wait for it.
static pq_status resident_stop(pq_sim *s) {
    if (!s->res || !s->res->launched) return PQ_OK;
    pq_sim::Resident &R = *s->res;
    reinterpret_cast<volatile ResidentBox *>(R.box.p)->stop = 1;
    std::atomic_thread_fence(std::memory_order_seq_cst);
    CU(cudaEventSynchronize(R.ev));
    R.launched = false;
    return PQ_OK;
}

// One boundary through the resident kernel (caller holds s->mu): the boundary and a new request
// number into the mapped box, then a bounded wait for the request number to come back; the
// kernel is launched (again) when it is not running.  The kernel's copy of the boundary it
// evaluated must equal the one sent, else the request is made again (at most 8 times).
static pq_status resident_eval(pq_sim *s, const uint64_t *x, const uint64_t *y, double *out, double *err) {
    pq_sim::Resident &R = *s->res;
    if (!R.plan) {
        auto P = std::make_unique<Plan>();
        std::vector<Segment> segs{{&s->main, 1}};
        pq_status st = build_plan(segs, s->nw, R.stream, s->tu, *P);
        if (st != PQ_OK) return st;
        if (!P->fused) return fail(PQ_ERR_UNSUPPORTED, "resident mode needs single amplitudes of at most 2^14 branches");
        R.plan = std::move(P);
    }
    Plan &P = *R.plan;
    volatile ResidentBox *b = reinterpret_cast<volatile ResidentBox *>(R.box.p);
    const int nw = s->nw;
    for (int w = 0; w < nw; w++) {
        b->words[w] = x[w];
        b->words[nw + w] = y[w];
    }
    auto launch = [&]() -> pq_status {
        b->stop = 0;
        b->exited = 0;
        KArgs a = P.args;
        ResidentBox *bd = R.box.dev<ResidentBox>();
        a.out = bd->out;
        a.err = &bd->err;
        const unsigned long long idle_ns = (unsigned long long)(R.idle_s * 1e9);
        const unsigned long long max_polls = idle_ns + (1ull << 24);  // every poll takes > 1 ns
        if (P.minb == 2)
            resident_kernel<2><<<1, P.fused_block, P.fused_smem, R.stream>>>(a, bd, b->done_seq, idle_ns, max_polls);
        else
            resident_kernel<3><<<1, P.fused_block, P.fused_smem, R.stream>>>(a, bd, b->done_seq, idle_ns, max_polls);
        CU(cudaGetLastError());
        CU(cudaEventRecord(R.ev, R.stream));
        R.launched = true;
        return PQ_OK;
    };
    // `exited` is the kernel's last write: once set, the kernel takes no further request
    if (!R.launched || b->exited) {
        if (R.launched) CU(cudaEventSynchronize(R.ev));
        pq_status st = launch();
        if (st != PQ_OK) return st;
    }
    bool same = false;
    for (int attempt = 0; attempt < 8 && !same; attempt++) {
        const unsigned want = ++R.seq;
        std::atomic_thread_fence(std::memory_order_seq_cst);  // the boundary before the request number
        b->req_seq = want;
        const double t0 = now_s();
        for (unsigned long spins = 0; b->done_seq != want; spins++) {
            if ((spins & 4095) == 4095) {
                if (b->exited && b->done_seq != want) {  // returned (idle) before it saw the request
                    CU(cudaEventSynchronize(R.ev));
                    pq_status st = launch();
                    if (st != PQ_OK) return st;
                }
                if (now_s() - t0 > 10.0) {
                    const cudaError_t q = cudaEventQuery(R.ev);
                    if (q != cudaSuccess && q != cudaErrorNotReady) return cuda_fail(q, "resident kernel");
                    return fail(PQ_ERR_TIMEOUT, "resident kernel did not answer within 10 s");
                }
            }
        }
        std::atomic_thread_fence(std::memory_order_seq_cst);  // the result after the request number
        same = true;
        for (int w = 0; w < nw; w++) same = same && b->words[2 * nw + w] == x[w] && b->words[3 * nw + w] == y[w];
    }
    if (!same) return fail(PQ_ERR_INTERNAL, "resident kernel evaluated a boundary other than the one sent");
    if (b->errflag) return fail(PQ_ERR_INTERNAL, "device self-check failed (odd Z8 increment)");
    out[0] = b->out[0];
    out[1] = b->out[1];
    if (err) err[0] = b->err;
    return PQ_OK;
}

PQ_API pq_status pq_sim_set_resident(pq_sim *s, double idle_seconds) {
    if (!s || !(idle_seconds >= 0.0) || idle_seconds > 3600.0) return fail(PQ_ERR_INVALID_ARG, "idle_seconds in 0..3600");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    pq_status st = resident_stop(s);
    if (st != PQ_OK) return st;
    if (idle_seconds == 0.0) {
        s->res.reset();
        return PQ_OK;
    }
    if (!s->res) {
        auto R = std::make_unique<pq_sim::Resident>();
        CU(R->box.alloc(sizeof(ResidentBox) + (size_t)4 * s->nw * 8));
        std::memset(R->box.p, 0, R->box.n);
        CU(cudaStreamCreateWithFlags(&R->stream, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&R->ev, cudaEventDisableTiming));
        s->res = std::move(R);
    }
    s->res->idle_s = idle_seconds;
    // the plan is built (and its fitness checked) now, so an unsuitable simulator fails here
    std::vector<uint64_t> z((size_t)s->nw, 0ull);
    double o[2];
    st = resident_eval(s, z.data(), z.data(), o, nullptr);
    if (st != PQ_OK) s->res.reset();
    return st;
}

PQ_API pq_status pq_amplitudes(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, double *out,
                               double *errbound) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(n);
    if (st != PQ_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    if (n == 1 && s->res) return resident_eval(s, x, y, out, errbound);
    Plan *P = nullptr;
    st = sim_plan(s, n, &P);
    if (st != PQ_OK) return st;
    return run_host(*P, x, y, out, errbound, CERT_NONE);
}

PQ_API pq_status pq_probabilities(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, double *out) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(n);
    if (st != PQ_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    Plan *P = nullptr;
    st = sim_plan(s, n, &P);
    if (st != PQ_OK) return st;
    return run_host(*P, x, y, out, nullptr, CERT_PROB);
}

PQ_API pq_status pq_amplitudes_device(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, double *out,
                                      double *errbound, void *stream) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(n);
    if (st != PQ_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    Plan *P = nullptr;
    st = sim_plan(s, n, &P);
    if (st != PQ_OK) return st;
    return run_device(*P, x, y, out, errbound, (cudaStream_t)stream);
}

PQ_API pq_status pq_amplitudes_plain(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, double *out) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(n);
    if (st != PQ_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    Plan *P = nullptr;
    st = sim_plan(s, 1, &P);
    if (st != PQ_OK) return st;
    for (int64_t i = 0; i < n; i++) {
        st = run_host(*P, x + (size_t)i * s->nw, y + (size_t)i * s->nw, out + 2 * i, nullptr, CERT_NONE);
        if (st != PQ_OK) return st;
    }
    return PQ_OK;
}

PQ_API pq_status pq_amplitudes_fp64(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, double *out) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(n);
    if (st != PQ_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    Plan *P = nullptr;
    st = sim_plan(s, n, &P);
    if (st != PQ_OK) return st;
    const size_t bw = (size_t)n * s->nw * 8;
    CU(cudaMemcpyAsync(P->x.p, x, bw, cudaMemcpyHostToDevice, P->stream));
    CU(cudaMemcpyAsync(P->y.p, y, bw, cudaMemcpyHostToDevice, P->stream));
    CU(enqueue_core(*P, 1, 0));  // the FP64 walk alone (the precision reference)
    CU(cudaMemcpyAsync(out, P->out.p, (size_t)n * 16, cudaMemcpyDeviceToHost, P->stream));
    CU(cudaStreamSynchronize(P->stream));
    return PQ_OK;
}

// Sandwich engines of one measured-qubit list, built and uploaded on first use and cached
// (caller holds s->mu).  Their fixed set is the first-occurrence order of the variables put
// by Sandwich::assignment: inputs, C^dagger C outputs, measured junctions (src/sim.rs:95-124).
// The sandwich path sum (built once, under s->mu; immutable afterwards).
static void ensure_sandwich(pq_sim *s) {
    if (!s->have_sw) {
        s->sw = PathSum::sandwich(s->circ, s->junction, s->jneg);
        s->have_sw = true;
    }
}

// Build and upload the sandwich engines of one measured-qubit list.  Reads only the simulator's
// immutable parts (circuit, sandwich path sum, strategy), so it runs without s->mu once
// ensure_sandwich has run.
static pq_status marg_build(pq_sim *s, const int32_t *qubits, int nmeas, int di_max, std::unique_ptr<pq_sim::Marg> &M) {
    const int nq = s->circ.nq;
    std::vector<std::pair<int, int32_t>> puts;
    for (int q = 0; q < nq; q++) puts.push_back({q, io_src(q, 0, 0)});
    for (int q = 0; q < nq; q++) puts.push_back({s->sw.outputs[q], io_src(q, 0, s->sw.out_neg[q])});
    for (int i = 0; i < nmeas; i++) puts.push_back({s->junction[qubits[i]], io_src(qubits[i], 1, s->jneg[qubits[i]])});
    M = std::make_unique<pq_sim::Marg>();
    M->tg.iom = build_iomap(puts);
    try {
        M->tg.rs = build_rank(s->sw, M->tg.iom.fixed, s->strategy, s->pairs);
    } catch (const std::exception &e) {
        return fail(PQ_ERR_INTERNAL, std::string("marginal engine build: ") + e.what());
    }
    return upload_target(M->tg, di_max);
}

static pq_status marg_target(pq_sim *s, const int32_t *qubits, int nmeas, pq_sim::Marg **out) {
    std::vector<int> key(qubits, qubits + nmeas);
    auto it = s->marg.find(key);
    if (it != s->marg.end()) {
        *out = it->second.get();
        return PQ_OK;
    }
    ensure_sandwich(s);
    std::unique_ptr<pq_sim::Marg> M;
    pq_status st = marg_build(s, qubits, nmeas, s->di_max, M);
    if (st != PQ_OK) return st;
    *out = M.get();
    s->marg.emplace(key, std::move(M));
    return PQ_OK;
}

PQ_API pq_status pq_marginal(pq_sim *s, const uint64_t *x, int32_t nmeas, const int32_t *qubits,
                             const uint8_t *outcomes, double *out) {
    if (!s || !x || !out || nmeas < 0 || (nmeas > 0 && (!qubits || !outcomes)))
        return fail(PQ_ERR_INVALID_ARG, "null argument");
    const int nq = s->circ.nq;
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    for (int i = 0; i < nmeas; i++)
        if (qubits[i] < 0 || qubits[i] >= nq) return fail(PQ_ERR_INVALID_ARG, "measured qubit out of range");
    std::lock_guard<std::mutex> lk(s->mu);
    CU(cudaSetDevice(s->device));
    pq_sim::Marg *M = nullptr;
    pq_status st = marg_target(s, qubits, nmeas, &M);
    if (st != PQ_OK) return st;
    if (!M->plan) {
        auto P = std::make_unique<Plan>();
        std::vector<Segment> segs{{&M->tg, 1}};
        st = build_plan(segs, s->nw, s->stream, s->tu, *P);
        if (st != PQ_OK) return st;
        M->plan = std::move(P);
    }
    std::vector<uint64_t> yv((size_t)s->nw, 0ull);
    for (int i = 0; i < nmeas; i++)
        if (outcomes[i]) yv[qubits[i] >> 6] |= 1ull << (qubits[i] & 63);
    // repeated measured qubits with different outcomes contradict: the map's check makes it 0
    double amp[2];
    st = run_host(*M->plan, x, yv.data(), amp, nullptr, CERT_REAL);
    if (st != PQ_OK) return st;
    *out = amp[0] > 0.0 ? amp[0] : 0.0;
    return PQ_OK;
}

// ---------------------------------------------------------------- Monte-Carlo estimate
// SplitMix64 (src/rng.rs:12-27).
struct SplitMix {
    uint64_t s;
    explicit SplitMix(uint64_t seed) : s(seed + 0x9E3779B97F4A7C15ull) {}
    uint64_t u64() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double f64() { return (double)(u64() >> 11) / 9007199254740992.0; }
};

static std::complex<double> phase_value(uint32_t p) {  // src/phase.rs:60-66
    static const double h = 0.70710678118654752440;
    static const double r8[16] = {1, 0, h, h, 0, 1, -h, h, -1, 0, -h, -h, 0, -1, h, -h};
    if ((p & ((1u << 29) - 1u)) == 0) {
        const int k = (int)(p >> 29);
        return {r8[2 * k], r8[2 * k + 1]};
    }
    const double th = 2.0 * M_PI * (double)p / 4294967296.0;
    return {std::cos(th), std::sin(th)};
}

// Estimate and standard error from the per-block (sum, sum |x|^2) of the sampled points:
// norm * 2^d * mean and |norm| * 2^d * sqrt(var / n) (src/engine.rs:650-658).
static pq_status mc_finish(const EngineDev &E, const JobDev &J, const std::vector<double> &hp, int grid,
                           int64_t samples, double *out, double *stderr_out) {
    if (J.vanish) return PQ_OK;  // prepare found no surviving subspace: (0, 0), src/engine.rs:618
    double sx = 0.0, sy = 0.0, sq = 0.0;
    for (int b = 0; b < grid; b++) {
        sx += hp[3 * b];
        sy += hp[3 * b + 1];
        sq += hp[3 * b + 2];
    }
    const double n = (double)samples;
    const std::complex<double> mean(sx / n, sy / n);
    const double var = std::max(sq / n - std::norm(mean), 0.0);
    const double scale = std::ldexp(1.0, E.d);
    // norm = phase * magnitude (src/engine.rs:620), and the Z8 root of the index at s = 0
    const std::complex<double> norm = phase_value(J.phase) * phase_value((J.k0 & 7u) << 29) * pow2_half(E.mag2 - E.num_h);
    const std::complex<double> val = norm * mean * scale;
    out[0] = val.real();
    out[1] = val.imag();
    if (stderr_out) *stderr_out = std::abs(norm) * scale * std::sqrt(var / n);
    return PQ_OK;
}

// Simulator::amplitude_estimate (src/sim.rs:184-193) -> RankEngine::estimate (src/rank.rs:149-171).
PQ_API pq_status pq_amplitude_estimate(pq_sim *s, const uint64_t *x, const uint64_t *y, int64_t samples,
                                       uint64_t seed, double *out, double *stderr_out) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    if (samples <= 0 || samples > (1LL << 40)) return fail(PQ_ERR_INVALID_ARG, "samples must be in 1..2^40");
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    std::lock_guard<std::mutex> lk(s->mu);
    CU(cudaSetDevice(s->device));
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    const int nb = (int)s->main.dev.size();
    const int nw = s->nw;
    out[0] = out[1] = 0.0;
    if (stderr_out) *stderr_out = 0.0;
    if (nb > 1) {
        // 2^p stabiliser branches: sample branch indices, evaluate each distinct one exactly
        std::map<int, int64_t> mult;
        for (int64_t i = 0; i < samples; i++) {
            SplitMix r(seed ^ ((uint64_t)i * golden));
            mult[(int)(r.u64() % (uint64_t)nb)]++;
        }
        std::vector<Target> views(mult.size());
        std::vector<Segment> segs;
        std::vector<int64_t> counts;
        size_t v = 0;
        for (const auto &kv : mult) {
            views[v].dev.push_back(s->main.dev[(size_t)kv.first]);
            views[v].iom_dev = s->main.iom_dev;
            views[v].max_words = s->main.max_words;
            segs.push_back({&views[v], 1});
            counts.push_back(kv.second);
            v++;
        }
        Plan P;
        pq_status st = build_plan(segs, nw, s->stream, s->tu, P);
        if (st != PQ_OK) return st;
        std::vector<uint64_t> X(segs.size() * nw), Y(segs.size() * nw);
        for (size_t k = 0; k < segs.size(); k++) {
            std::memcpy(&X[k * nw], x, sizeof(uint64_t) * nw);
            std::memcpy(&Y[k * nw], y, sizeof(uint64_t) * nw);
        }
        std::vector<double> amp(2 * segs.size());
        st = run_host(P, X.data(), Y.data(), amp.data(), nullptr, CERT_NONE);
        if (st != PQ_OK) return st;
        double sx = 0.0, sy = 0.0, sq = 0.0;
        for (size_t k = 0; k < segs.size(); k++) {
            const double m = (double)counts[k];
            sx += m * amp[2 * k];
            sy += m * amp[2 * k + 1];
            sq += m * (amp[2 * k] * amp[2 * k] + amp[2 * k + 1] * amp[2 * k + 1]);
        }
        const double n = (double)samples, mx = sx / n, my = sy / n;
        const double var = std::max(sq / n - (mx * mx + my * my), 0.0);
        out[0] = mx * nb;
        out[1] = my * nb;
        if (stderr_out) *stderr_out = nb * std::sqrt(var / n);
        return PQ_OK;
    }
    const EngineDev &E = s->main.dev[0];
    if (E.d < 63 && (1LL << E.d) <= samples) {  // small subspace: the exact sum
        Plan *P = nullptr;
        pq_status st = sim_plan(s, 1, &P);
        if (st != PQ_OK) return st;
        return run_host(*P, x, y, out, nullptr, CERT_NONE);
    }
    if (E.d > kMaxD) {
        // beyond the enumeration's limits: prepare alone, then the multi-word sampler
        if (E.d > 64 * MC_WORDS) return fail(PQ_ERR_UNSUPPORTED, "Monte-Carlo estimate supports branch dimensions up to 512");
        Plan Q;
        std::vector<Segment> segs{{&s->main, 1}};
        pq_status st = build_plan(segs, nw, s->stream, s->tu, Q, false, true);
        if (st != PQ_OK) return st;
        DevMem lpx;
        CU(lpx.alloc((size_t)E.d));
        Q.args.lpx = lpx.as<uint8_t>();
        Q.args.lpx_stride = E.d;
        const size_t bwb = (size_t)nw * 8;
        CU(cudaMemcpyAsync(Q.x.p, x, bwb, cudaMemcpyHostToDevice, Q.stream));
        CU(cudaMemcpyAsync(Q.y.p, y, bwb, cudaMemcpyHostToDevice, Q.stream));
        prepare_kernel<<<Q.grid_prep, 128, (size_t)4 * Q.smem_words * 8, Q.stream>>>(Q.args);
        CU(cudaGetLastError());
        const int grid = (int)std::max<long long>(1, std::min<long long>((samples + 255) / 256, (long long)sm_count() * 8));
        DevMem part;
        CU(part.alloc((size_t)grid * 3 * sizeof(double)));
        mc_big_kernel<<<grid, 256, 0, Q.stream>>>(Q.engines.as<EngineDev>(), Q.jobs.as<JobDev>(), lpx.as<uint8_t>(),
                                                   seed, (long long)samples, part.as<double>());
        CU(cudaGetLastError());
        JobDev J;
        std::vector<double> hp((size_t)grid * 3);
        CU(cudaMemcpyAsync(&J, Q.jobs.p, sizeof(JobDev), cudaMemcpyDeviceToHost, Q.stream));
        CU(cudaMemcpyAsync(hp.data(), part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, Q.stream));
        CU(cudaStreamSynchronize(Q.stream));
        return mc_finish(E, J, hp, grid, samples, out, stderr_out);
    }
    Plan *P = nullptr;
    pq_status st = sim_plan(s, 1, &P);
    if (st != PQ_OK) return st;
    const size_t bw = (size_t)nw * 8;
    CU(cudaMemcpyAsync(P->x.p, x, bw, cudaMemcpyHostToDevice, P->stream));
    CU(cudaMemcpyAsync(P->y.p, y, bw, cudaMemcpyHostToDevice, P->stream));
    prepare_kernel<<<P->grid_prep, 128, (size_t)4 * P->smem_words * 8, P->stream>>>(P->args);
    CU(cudaGetLastError());
    const int grid = (int)std::max<long long>(1, std::min<long long>((samples + 255) / 256, (long long)sm_count() * 8));
    DevMem part;
    CU(part.alloc((size_t)grid * 3 * sizeof(double)));
    mc_kernel<<<grid, 256, 0, P->stream>>>(P->engines.as<EngineDev>(), P->jobs.as<JobDev>(), seed, (long long)samples,
                                            part.as<double>());
    CU(cudaGetLastError());
    JobDev J;
    std::vector<double> hp((size_t)grid * 3);
    CU(cudaMemcpyAsync(&J, P->jobs.p, sizeof(JobDev), cudaMemcpyDeviceToHost, P->stream));
    CU(cudaMemcpyAsync(hp.data(), part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, P->stream));
    CU(cudaStreamSynchronize(P->stream));
    return mc_finish(E, J, hp, grid, samples, out, stderr_out);
}

// Lazy pair sampling (src/approx.rs:96-135, estimate_amplitude): sample i draws
// Rng::new(seed ^ i * golden), takes one bit per pair for the first p pair candidates, builds
// that branch engine (substitutions + one elimination, on host threads; equal patterns share
// one engine) and evaluates it exactly when its dimension is at most exact_dim_limit, else by
// Engine::estimate with 2^14 points and the sample's next draw as seed.  The estimate is
// 2^p mean and its standard error 2^p sqrt(var / n).
PQ_API pq_status pq_amplitude_estimate_pairs(pq_sim *s, const uint64_t *x, const uint64_t *y, int32_t pairs,
                                             int64_t samples, uint64_t seed, int32_t exact_dim_limit, double *out,
                                             double *stderr_out) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    if (pairs < 0) return fail(PQ_ERR_INVALID_ARG, "negative pair count");
    if (samples <= 0 || samples > (1LL << 24)) return fail(PQ_ERR_INVALID_ARG, "samples must be in 1..2^24");
    if (exact_dim_limit < 0) return fail(PQ_ERR_INVALID_ARG, "negative exact dimension limit");
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    std::lock_guard<std::mutex> lk(s->mu);
    CU(cudaSetDevice(s->device));
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    const int nw = s->nw;
    out[0] = out[1] = 0.0;
    if (stderr_out) *stderr_out = 0.0;
    int ntc = 0;
    const std::vector<int> &fixed = s->main.iom.fixed;
    const auto cands = pair_candidates(s->ps, fixed, ntc);
    const int p = std::min(std::min((int)pairs, (int)cands.size()), 62);
    const size_t ns = (size_t)samples;
    std::vector<uint64_t> mseed(ns);
    std::map<uint64_t, int> index;  // pattern -> distinct engine
    std::vector<uint64_t> distinct;
    std::vector<int> eng_of(ns);
    for (size_t i = 0; i < ns; i++) {
        SplitMix r(seed ^ ((uint64_t)i * golden));
        uint64_t b = 0;
        for (int j = 0; j < p; j++) b |= (r.u64() & 1ull) << j;
        mseed[i] = r.u64();
        auto it = index.find(b);
        if (it == index.end()) {
            it = index.emplace(b, (int)distinct.size()).first;
            distinct.push_back(b);
        }
        eng_of[i] = it->second;
    }
    // every distinct pattern's engine is held (host and device) for the call, as the 2^p
    // engines of a rank strategy are: the same cap, 2^14
    if (distinct.size() > ((size_t)1 << 14))
        return fail(PQ_ERR_INVALID_ARG, "more than 2^14 distinct sampled branch engines in one call; split the samples");
    // one engine per distinct pattern, on host threads
    Target T;
    T.iom = s->main.iom;
    T.rs.pairs = p;
    T.rs.branches.resize(distinct.size());
    {
        std::atomic<size_t> next{0};
        std::vector<std::string> errs(distinct.size());
        auto work = [&]() {
            for (size_t k = next++; k < distinct.size(); k = next++) {
                try {
                    T.rs.branches[k] = pattern_engine(s->ps, fixed, cands, p, distinct[k]);
                } catch (const std::exception &e) {
                    errs[k] = e.what();
                }
            }
        };
        const size_t nth = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), distinct.size());
        if (nth <= 1) work();
        else {
            std::vector<std::thread> th;
            for (size_t t = 0; t < nth; t++) th.emplace_back(work);
            for (auto &t : th) t.join();
        }
        for (auto &e : errs)
            if (!e.empty()) return fail(PQ_ERR_INTERNAL, "engine build: " + e);
    }
    pq_status st = upload_target(T, s->di_max);
    if (st != PQ_OK) return st;
    const int64_t kMcPoints = 1 << 14;
    std::vector<std::complex<double>> val(distinct.size());  // exact values
    std::vector<char> exact(distinct.size(), 0);
    std::vector<Target> views(distinct.size());
    std::vector<Segment> segs;
    std::vector<size_t> seg_engine;
    for (size_t k = 0; k < distinct.size(); k++) {
        views[k].dev.push_back(T.dev[k]);
        views[k].iom_dev = T.iom_dev;
        views[k].max_words = T.max_words;
        const EngineDev &E = T.dev[k];
        // the reference's own rule, and Engine::estimate's exact sum for subspaces of at most
        // as many points as it would sample
        const bool ex = E.d <= exact_dim_limit || (E.d < 63 && (1LL << E.d) <= kMcPoints);
        if (ex && (E.d > s->tu.max_branch_dim || E.rank > kMaxPivots))
            return fail(PQ_ERR_ADMISSION_REFUSED, "sampled branch engine above the enumeration's limits");
        if (ex) {
            exact[k] = 1;
            segs.push_back({&views[k], 1});
            seg_engine.push_back(k);
        }
    }
    if (!segs.empty()) {
        Plan P;
        st = build_plan(segs, nw, s->stream, s->tu, P);
        if (st != PQ_OK) return st;
        std::vector<uint64_t> X(segs.size() * nw), Y(segs.size() * nw);
        for (size_t k = 0; k < segs.size(); k++) {
            std::memcpy(&X[k * nw], x, sizeof(uint64_t) * nw);
            std::memcpy(&Y[k * nw], y, sizeof(uint64_t) * nw);
        }
        std::vector<double> amp(2 * segs.size());
        st = run_host(P, X.data(), Y.data(), amp.data(), nullptr, CERT_NONE);
        if (st != PQ_OK) return st;
        for (size_t k = 0; k < segs.size(); k++) val[seg_engine[k]] = {amp[2 * k], amp[2 * k + 1]};
    }
    // exact samples: their engine's value; Monte-Carlo samples: per distinct engine, prepare
    // once, then one sampler launch per sample
    std::complex<double> sum(0.0, 0.0);
    double sq = 0.0;
    for (size_t i = 0; i < ns; i++)
        if (exact[(size_t)eng_of[i]]) {
            const std::complex<double> a = val[(size_t)eng_of[i]];
            sum += a;
            sq += std::norm(a);
        }
    for (size_t k = 0; k < distinct.size(); k++) {
        if (exact[k]) continue;
        const EngineDev &E = T.dev[k];
        if (E.d > 64 * MC_WORDS) return fail(PQ_ERR_UNSUPPORTED, "Monte-Carlo estimate supports branch dimensions up to 512");
        Plan Q;
        std::vector<Segment> one{{&views[k], 1}};
        st = build_plan(one, nw, s->stream, s->tu, Q, false, true);
        if (st != PQ_OK) return st;
        DevMem lpx;
        if (E.d > kMaxD) {
            CU(lpx.alloc((size_t)E.d));
            Q.args.lpx = lpx.as<uint8_t>();
            Q.args.lpx_stride = E.d;
        }
        const size_t bwb = (size_t)nw * 8;
        CU(cudaMemcpyAsync(Q.x.p, x, bwb, cudaMemcpyHostToDevice, Q.stream));
        CU(cudaMemcpyAsync(Q.y.p, y, bwb, cudaMemcpyHostToDevice, Q.stream));
        prepare_kernel<<<Q.grid_prep, 128, (size_t)4 * Q.smem_words * 8, Q.stream>>>(Q.args);
        CU(cudaGetLastError());
        const int grid = (int)std::max<long long>(1, std::min<long long>((kMcPoints + 255) / 256, (long long)sm_count() * 8));
        DevMem part;
        CU(part.alloc((size_t)grid * 3 * sizeof(double)));
        JobDev J;
        CU(cudaMemcpyAsync(&J, Q.jobs.p, sizeof(JobDev), cudaMemcpyDeviceToHost, Q.stream));
        std::vector<double> hp((size_t)grid * 3);
        for (size_t i = 0; i < ns; i++) {
            if (eng_of[i] != (int)k) continue;
            if (E.d > kMaxD)
                mc_big_kernel<<<grid, 256, 0, Q.stream>>>(Q.engines.as<EngineDev>(), Q.jobs.as<JobDev>(),
                                                          lpx.as<uint8_t>(), mseed[i], (long long)kMcPoints,
                                                          part.as<double>());
            else
                mc_kernel<<<grid, 256, 0, Q.stream>>>(Q.engines.as<EngineDev>(), Q.jobs.as<JobDev>(), mseed[i],
                                                      (long long)kMcPoints, part.as<double>());
            CU(cudaGetLastError());
            CU(cudaMemcpyAsync(hp.data(), part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, Q.stream));
            CU(cudaStreamSynchronize(Q.stream));
            double v[2] = {0.0, 0.0};
            st = mc_finish(E, J, hp, grid, kMcPoints, v, nullptr);
            if (st != PQ_OK) return st;
            const std::complex<double> a(v[0], v[1]);
            sum += a;
            sq += std::norm(a);
        }
    }
    const double n = (double)samples;
    const std::complex<double> mean = sum / n;
    const double var = std::max(sq / n - std::norm(mean), 0.0);
    const double scale = std::ldexp(1.0, p);
    out[0] = mean.real() * scale;
    out[1] = mean.imag() * scale;
    if (stderr_out) *stderr_out = scale * std::sqrt(var / n);
    return PQ_OK;
}

// ---------------------------------------------------------------- sampling
// Simulator::sample_many (src/sim.rs:253-284) with the shots batched per qubit: level l
// evaluates, for every shot at once, the marginal of qubits 0..l with the shot's decided prefix
// and bit l = 0 (the sandwich engines of prefix l, src/sim.rs:232-249), in one launch; each
// shot then draws its uniform and takes bit l exactly as the reference does.  A decision whose
// margin |u * p_prev - p0| lies within the FP32 path's error bound is re-taken on that
// level's FP64 evaluation, so decisions follow FP64 marginals.
PQ_API pq_status pq_sample_many(pq_sim *s, const uint64_t *x, int64_t shots, uint64_t seed, uint64_t *out) {
    if (!s || !x || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(shots);
    if (st != PQ_OK) return st;
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    std::lock_guard<std::mutex> lk(s->mu);
    CU(cudaSetDevice(s->device));
    const int nq = s->circ.nq, nw = s->nw;
    const size_t ns = (size_t)shots;
    SplitMix root(seed);
    std::vector<SplitMix> rng;
    rng.reserve(ns);
    for (size_t i = 0; i < ns; i++) rng.emplace_back(root.u64());
    std::vector<uint64_t> X(ns * nw), Y(ns * nw, 0ull);
    for (size_t i = 0; i < ns; i++) std::memcpy(&X[i * nw], x, sizeof(uint64_t) * nw);
    std::vector<double> p_prev(ns, 1.0), amp(2 * ns), err(ns), u(ns);
    std::vector<char> tie(ns, 0);
    std::vector<int32_t> qs(nq);
    for (int q = 0; q < nq; q++) qs[q] = q;
    for (int l = 0; l < nq; l++) {
        pq_sim::Marg *M = nullptr;
        st = marg_target(s, qs.data(), l + 1, &M);
        if (st != PQ_OK) return st;
        auto &slot = M->many[shots];
        if (!slot) {
            auto P = std::make_unique<Plan>();
            std::vector<Segment> segs{{&M->tg, shots}};
            st = build_plan(segs, nw, s->stream, s->tu, *P);
            if (st != PQ_OK) return st;
            slot = std::move(P);
        }
        Plan &P = *slot;
        st = run_host(P, X.data(), Y.data(), amp.data(), err.data(), CERT_NONE);
        if (st != PQ_OK) return st;
        bool any_tie = false;
        for (size_t i = 0; i < ns; i++) {
            u[i] = rng[i].f64();
            const double p0 = std::min(std::max(amp[2 * i], 0.0), p_prev[i]);
            tie[i] = std::fabs(u[i] * p_prev[i] - p0) <= err[i] + 1e-15 * p0;
            any_tie = any_tie || tie[i];
        }
        if (any_tie) {
            if (P.fused) {  // the fused launch read the boundaries from the mapped buffers
                const size_t bwb = ns * (size_t)nw * 8;
                CU(cudaMemcpyAsync(P.x.p, P.hx.p, bwb, cudaMemcpyHostToDevice, P.stream));
                CU(cudaMemcpyAsync(P.y.p, P.hy.p, bwb, cudaMemcpyHostToDevice, P.stream));
            }
            CU(enqueue_core(P, 1));
            CU(cudaMemcpyAsync(P.hout.p, P.out.p, ns * 16, cudaMemcpyDeviceToHost, P.stream));
            CU(cudaStreamSynchronize(P.stream));
            const double *ho = P.hout.as<double>();
            for (size_t i = 0; i < ns; i++)
                if (tie[i]) amp[2 * i] = ho[2 * i];
        }
        for (size_t i = 0; i < ns; i++) {
            const double p0 = std::min(std::max(amp[2 * i], 0.0), p_prev[i]);
            if (u[i] * p_prev[i] >= p0) {
                Y[i * nw + (l >> 6)] |= 1ull << (l & 63);
                p_prev[i] = std::max(p_prev[i] - p0, 0.0);
            } else {
                p_prev[i] = p0;
            }
        }
    }
    std::memcpy(out, Y.data(), sizeof(uint64_t) * ns * nw);
    return PQ_OK;
}

// ---------------------------------------------------------------- batches
PQ_API pq_status pq_batch_create(int32_t nsims, pq_sim *const *sims, const int64_t *counts, pq_batch **out) {
    if (nsims <= 0 || !sims || !counts || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    auto B = std::make_unique<pq_batch>();
    std::vector<Segment> segs;
    int nw = 1;
    int64_t tot = 0;
    for (int i = 0; i < nsims; i++) {
        if (!sims[i] || counts[i] < 0) return fail(PQ_ERR_INVALID_ARG, "bad simulator or count");
        if (sims[i]->host_only) return fail(PQ_ERR_NO_DEVICE, "host-only simulator in a batch");
        if (sims[i]->device != g_device) return fail(PQ_ERR_INVALID_ARG, "simulators on different devices");
        B->sims.push_back(sims[i]);
        segs.push_back({&sims[i]->main, counts[i]});
        nw = std::max(nw, sims[i]->nw);
        tot += counts[i];
    }
    if (tot <= 0 || tot > (1LL << 24)) return fail(PQ_ERR_INVALID_ARG, "total boundary count must be in 1..2^24");
    pq_tuning tu;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        tu = g_tuning;
    }
    CU(cudaSetDevice(g_device));
    B->segs = segs;
    B->nw = nw;
    B->tu = tu;
    B->plan = std::make_unique<Plan>();
    pq_status st = build_plan(segs, nw, nullptr, tu, *B->plan);
    if (st != PQ_OK) return st;
    *out = B.release();
    return PQ_OK;
}
PQ_API void pq_batch_destroy(pq_batch *b) {
    if (!b) return;
    if (b->plan && b->plan->stream) cudaStreamSynchronize(b->plan->stream);
    delete b;
}
PQ_API int32_t pq_batch_words(const pq_batch *b) { return b ? b->nw : 0; }
PQ_API int64_t pq_batch_branches(const pq_batch *b) { return b && b->plan ? (int64_t)b->plan->branches : 0; }
PQ_API pq_status pq_batch_run(pq_batch *b, const uint64_t *x, const uint64_t *y, double *out, double *err) {
    if (!b || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(b->mu);
    if (!b->plan) return fail(PQ_ERR_INTERNAL, "batch has no launch plan (a failed autotune left none)");
    return run_host(*b->plan, x, y, out, err, CERT_NONE);
}
PQ_API pq_status pq_batch_run_device(pq_batch *b, const uint64_t *x, const uint64_t *y, double *out, double *err,
                                     void *stream) {
    if (!b || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(b->mu);
    if (!b->plan) return fail(PQ_ERR_INTERNAL, "batch has no launch plan (a failed autotune left none)");
    return run_device(*b->plan, x, y, out, err, (cudaStream_t)stream);
}

PQ_API pq_status pq_sim_device_check(pq_sim *s, int64_t n, int32_t *failed) {
    if (!s || !failed) return fail(PQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->plans.find(n);
    if (it == s->plans.end() || !it->second->ran) return fail(PQ_ERR_INVALID_ARG, "no launch of that size yet");
    Plan &P = *it->second;
    CU(cudaSetDevice(s->device));
    CU(cudaStreamSynchronize(P.stream));
    int f = 0;
    if (P.last_host_io) f = *P.herrflag.as<int>();
    else CU(cudaMemcpy(&f, P.errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
    *failed = f ? 1 : 0;
    return PQ_OK;
}

PQ_API pq_status pq_sim_kernel_ms(pq_sim *s, int64_t n, float *ms) {
    if (!s || !ms) return fail(PQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->plans.find(n);
    if (it == s->plans.end() || !it->second->ran) return fail(PQ_ERR_INVALID_ARG, "no launch of that size yet");
    CU(cudaEventSynchronize(it->second->tev[3]));
    return last_kernel_ms(*it->second, ms);
}
PQ_API pq_status pq_batch_kernel_ms(pq_batch *b, float *ms) {
    if (!b || !ms) return fail(PQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(b->mu);
    if (!b->plan || !b->plan->ran) return fail(PQ_ERR_INVALID_ARG, "batch has not run yet");
    CU(cudaEventSynchronize(b->plan->tev[3]));
    return last_kernel_ms(*b->plan, ms);
}
// Branches actually enumerated by the last launch of the simulator's size-n plan: 2^d of every
// (boundary, branch engine) job whose boundary did not make the sum vanish (a vanishing job --
// contradictory boundary or inconsistent radical system -- is a zero, not enumerated).
// out[0] branches, out[1] reference-form int64 ops (5 W_o + 6 W_g per branch), out[2] of which
// 64-bit popcounts (2 W_o + W_g), out[3] of which 64-bit logic ops (3 W_o + 5 W_g).
static pq_status plan_enumerated(Plan &P, double *out, double *per_out) {
    CU(cudaStreamSynchronize(P.stream));
    std::vector<JobDev> jobs((size_t)P.njobs);
    CU(cudaMemcpy(jobs.data(), P.jobs.p, sizeof(JobDev) * jobs.size(), cudaMemcpyDeviceToHost));
    std::vector<EngineDev> eng(P.engines.n / sizeof(EngineDev));
    CU(cudaMemcpy(eng.data(), P.engines.p, sizeof(EngineDev) * eng.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 4; i++) out[i] = 0.0;
    if (per_out)
        for (int o = 0; o < P.nout; o++) per_out[o] = 0.0;
    for (const auto &J : jobs) {
        if (J.vanish) continue;
        const EngineDev &E = eng[J.engine];
        const double b = std::ldexp(1.0, E.d);
        out[0] += b;
        out[1] += b * (5.0 * E.wo + 6.0 * E.wg);
        out[2] += b * (2.0 * E.wo + E.wg);
        out[3] += b * (3.0 * E.wo + 5.0 * E.wg);
        if (per_out) per_out[J.out] += b;
    }
    return PQ_OK;
}
PQ_API pq_status pq_sim_enumerated(pq_sim *s, int64_t n, double *out, double *per_boundary) {
    if (!s || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->plans.find(n);
    if (it == s->plans.end() || !it->second->ran) return fail(PQ_ERR_INVALID_ARG, "no launch of that size yet");
    return plan_enumerated(*it->second, out, per_boundary);
}
PQ_API pq_status pq_batch_enumerated(pq_batch *b, double *out) {
    if (!b || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(b->mu);
    if (!b->plan || !b->plan->ran) return fail(PQ_ERR_INVALID_ARG, "batch has not run yet");
    return plan_enumerated(*b->plan, out, nullptr);
}
PQ_API int64_t pq_sim_launch_items(pq_sim *s, int64_t n) {
    if (!s) return -1;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->plans.find(n);
    return it == s->plans.end() ? -1 : (int64_t)it->second->nitems;
}

// ---------------------------------------------------------------- autotuner
// Rebuilds a simulator's resident weight tables for a new low-coordinate count (the tables'
// layout depends on it); cached plans point into the old tables and are dropped first.
static pq_status retable_sim(pq_sim *s, int di) {
    CU(cudaStreamSynchronize(s->stream));
    if (s->res) {  // its plan points into the tables about to be rebuilt
        pq_status st = resident_stop(s);
        if (st != PQ_OK) return st;
        s->res->plan.reset();
    }
    s->plans.clear();
    s->main.dev.clear();
    s->main.mem.clear();
    s->main.max_d = s->main.max_rank = s->main.max_words = 0;
    pq_status st = upload_target(s->main, di);
    if (st != PQ_OK) return st;
    s->di_max = di;
    return PQ_OK;
}

// Device time (ms, best of `reps` after one warm-up) of one launch of the simulator's
// evaluation of n boundaries under tuning `tu`.
static pq_status time_tuning(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, int reps,
                             const pq_tuning &tu, std::vector<double> &scratch, double *ms_out) {
    if (tu.inner_dims != s->di_max) {
        pq_status st = retable_sim(s, tu.inner_dims);
        if (st != PQ_OK) return st;
    }
    Plan P;
    std::vector<Segment> segs{{&s->main, n}};
    pq_status st = build_plan(segs, s->nw, s->stream, tu, P);
    if (st != PQ_OK) return st;
    scratch.resize((size_t)2 * n);
    double best = 1e300;
    for (int r = 0; r <= reps; r++) {
        st = run_host(P, x, y, scratch.data(), nullptr, CERT_NONE);
        if (st != PQ_OK) return st;
        float ms[3];
        st = last_kernel_ms(P, ms);
        if (st != PQ_OK) return st;
        if (r > 0) best = std::min(best, (double)ms[0] + ms[1] + ms[2]);
    }
    *ms_out = best;
    return PQ_OK;
}

}  // extern "C"

// Coordinate descent over the launch shape from `start`: one field at a time over its
// candidate values, keeping the fastest (by more than 2%, so timing noise does not flip
// choices), until a full pass changes nothing (at most three passes).  `time_of` returns the
// device time of one launch under a tuning.  Lane chunks stop at 2^10 steps: the plain-FP32
// low-part sums lose accuracy as 4^inner_dims (more terms on a coarser exact grid), and 2^12
// already costs an order of magnitude.  The register budget and the chunks per unit move
// together: eight chunks per unit need two blocks per SM.
template <class TimeOf>
static pq_status tune_search(pq_tuning start, bool tune_inner, TimeOf time_of, pq_tuning &best, double &best_t) {
    const std::vector<int> axes[4] = {{8, 9, 10}, {1, 2, 4, 8, 16}, {2, 4, 8}, {28, 24, 34, 32, 44, 42}};
    auto set_field = [](pq_tuning &t, int k, int v) {
        if (k == 0) t.inner_dims = v;
        else if (k == 1) t.chunks_per_lane = v;
        else if (k == 2) t.block_warps = v;
        else {
            t.blocks_per_sm = v / 10;
            t.unit_chunks = v % 10;
        }
    };
    std::map<std::array<int, 5>, double> seen;
    auto eval = [&](const pq_tuning &t, double *ms) -> pq_status {
        std::array<int, 5> key{t.inner_dims, t.chunks_per_lane, t.block_warps, t.blocks_per_sm, unit_max_of(t)};
        auto it = seen.find(key);
        if (it != seen.end()) {
            *ms = it->second;
            return PQ_OK;
        }
        pq_status e = time_of(t, ms);
        if (e == PQ_OK) seen[key] = *ms;
        return e;
    };
    best = start;
    pq_status st = eval(best, &best_t);
    for (int pass = 0; st == PQ_OK && pass < 3; pass++) {
        bool changed = false;
        for (int k = tune_inner ? 0 : 1; k < 4 && st == PQ_OK; k++) {
            for (int v : axes[k]) {
                pq_tuning t = best;
                set_field(t, k, v);
                double ms = 0.0;
                st = eval(t, &ms);
                if (st != PQ_OK) break;
                if (ms < best_t * 0.995) {  // event-timed launches repeat to ~0.1%
                    best = t;
                    best_t = ms;
                    changed = true;
                }
            }
        }
        if (!changed) break;
    }
    return st;
}

extern "C" {

PQ_API pq_status pq_sim_autotune(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, int32_t reps,
                                 pq_tuning *best_out, double *best_ms) {
    if (!s || !x || !y) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(n);
    if (st != PQ_OK) return st;
    if (reps < 0 || reps > 1000) return fail(PQ_ERR_INVALID_ARG, "reps in 0..1000");
    if (reps == 0) reps = 3;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    std::vector<double> scratch;
    pq_tuning start = s->tu, best;
    start.inner_dims = s->di_max;
    double best_t = 0.0;
    st = tune_search(start, true,
                     [&](const pq_tuning &t, double *ms) { return time_tuning(s, n, x, y, reps, t, scratch, ms); },
                     best, best_t);
    // whatever happened, leave the simulator on its best known tuning
    pq_status st2 = PQ_OK;
    if (best.inner_dims != s->di_max) st2 = retable_sim(s, best.inner_dims);
    s->tu = best;
    s->plans.clear();
    if (st != PQ_OK) return st;
    if (st2 != PQ_OK) return st2;
    if (best_out) *best_out = best;
    if (best_ms) *best_ms = best_t;
    return PQ_OK;
}

PQ_API pq_status pq_batch_autotune(pq_batch *b, const uint64_t *x, const uint64_t *y, int32_t reps, pq_tuning *best_out,
                                   double *best_ms) {
    if (!b || !x || !y) return fail(PQ_ERR_INVALID_ARG, "null argument");
    if (reps < 0 || reps > 1000) return fail(PQ_ERR_INVALID_ARG, "reps in 0..1000");
    if (reps == 0) reps = 3;
    std::lock_guard<std::mutex> lk(b->mu);
    CU(cudaSetDevice(g_device));
    std::vector<double> scratch((size_t)2 * b->plan->nout);
    // the lane chunk length is a property of each member simulator's weight tables: a candidate
    // with another length rebuilds them (and drops the simulators' own cached plans)
    int cur_di = b->sims[0]->di_max;
    auto retable_all = [&](int di) -> pq_status {
        std::set<pq_sim *> seen;
        for (pq_sim *sp : b->sims) {
            if (!seen.insert(sp).second) continue;
            std::lock_guard<std::mutex> l2(sp->mu);
            if (sp->di_max != di) {
                pq_status e = retable_sim(sp, di);
                if (e != PQ_OK) return e;
            }
        }
        cur_di = di;
        return PQ_OK;
    };
    if (b->plan) {
        CU(cudaStreamSynchronize(b->plan->stream));
        b->plan.reset();  // its engine records point into tables that may be rebuilt
    }
    auto time_of = [&](const pq_tuning &t, double *ms_out) -> pq_status {
        if (t.inner_dims != cur_di) {
            pq_status e = retable_all(t.inner_dims);
            if (e != PQ_OK) return e;
        }
        Plan P;
        pq_status e = build_plan(b->segs, b->nw, nullptr, t, P);
        if (e != PQ_OK) return e;
        double bt = 1e300;
        for (int r = 0; r <= reps; r++) {
            e = run_host(P, x, y, scratch.data(), nullptr, CERT_NONE);
            if (e != PQ_OK) return e;
            float ms[3];
            e = last_kernel_ms(P, ms);
            if (e != PQ_OK) return e;
            if (r > 0) bt = std::min(bt, (double)ms[0] + ms[1] + ms[2]);
        }
        *ms_out = bt;
        return PQ_OK;
    };
    pq_tuning start = b->tu, best = b->tu;
    start.inner_dims = cur_di;
    double best_t = 0.0;
    pq_status st = tune_search(start, true, time_of, best, best_t);
    // whatever happened, leave the batch on its best known shape
    pq_status st2 = best.inner_dims != cur_di ? retable_all(best.inner_dims) : PQ_OK;
    auto P = std::make_unique<Plan>();
    pq_status st3 = st2 == PQ_OK ? build_plan(b->segs, b->nw, nullptr, best, *P) : st2;
    if (st3 == PQ_OK) {
        b->plan = std::move(P);
        b->tu = best;
    }
    if (st != PQ_OK) return st;
    if (st3 != PQ_OK) return st3;
    if (best_out) *best_out = best;
    if (best_ms) *best_ms = best_t;
    return PQ_OK;
}

PQ_API pq_status pq_sim_get_tuning(const pq_sim *s, pq_tuning *out) {
    if (!s || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    *out = s->tu;
    out->inner_dims = s->di_max;
    return PQ_OK;
}

// ---------------------------------------------------------------- checks
PQ_API int64_t pq_debug_engine_dump(const pq_sim *s, int32_t branch, uint64_t *out, int64_t cap) {
    if (!s || branch < 0 || branch >= (int)s->main.rs.branches.size()) {
        g_err = "bad simulator or branch";
        return -1;
    }
    std::vector<uint64_t> v = engine_dump(*s->main.rs.branches[branch]);
    if (out) std::memcpy(out, v.data(), sizeof(uint64_t) * (size_t)std::min<int64_t>(cap, (int64_t)v.size()));
    return (int64_t)v.size();
}

PQ_API pq_status pq_debug_engine_shape(const pq_sim *s, int32_t branch, int64_t *out) {
    if (!s || !out || branch < 0 || branch >= (int)s->main.rs.branches.size())
        return fail(PQ_ERR_INVALID_ARG, "bad simulator or branch");
    std::vector<int> perm;
    const HostEngine e = device_order(*s->main.rs.branches[branch], s->di_max, perm);
    EngineTables tb = build_tables(e, s->di_max);
    PackedEngine pk = pack_engine(e, tb);
    int64_t r0 = 0, r0hi = 0;
    for (int j = 0; j < e.d; j++)
        if (e.R[(size_t)j] == 0) {
            r0++;
            if (j >= tb.DI) r0hi++;
        }
    const int64_t v[8] = {e.d, e.rank, tb.DI, tb.joint ? 1 : 0, pk.off.npairc ? pk.off.pairc[0] : -1, r0, r0hi, e.t};
    for (int i = 0; i < 8; i++) out[i] = v[i];
    return PQ_OK;
}

PQ_API int32_t pq_debug_branch_phases(pq_sim *s, int32_t branch, const uint64_t *x, const uint64_t *y, uint8_t *out) {
    if (!s || !x || !y || !out || branch < 0 || branch >= (int)s->main.rs.branches.size()) {
        g_err = "bad argument";
        return -2;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) {
        g_err = "simulator was created by pq_analyze (host structures only)";
        return -2;
    }
    if (cudaSetDevice(s->device) != cudaSuccess) return -2;
    const int d = s->main.rs.branches[branch]->d;
    if (d > 24) {
        g_err = "branch dimension above 24";
        return -2;
    }
    // a single-engine target view of branch `branch`
    Target view;
    view.dev.push_back(s->main.dev[branch]);
    view.iom_dev = s->main.iom_dev;
    view.max_words = s->main.max_words;
    pq_tuning tu;
    {
        std::lock_guard<std::mutex> lk2(g_mu);
        tu = g_tuning;
    }
    tu.max_branch_dim = kMaxD;
    Plan P;
    std::vector<Segment> segs{{&view, 1}};
    if (build_plan(segs, s->nw, s->stream, tu, P) != PQ_OK) return -2;
    DevMem dbg;
    if (dbg.alloc((size_t)1 << d) != cudaSuccess) return -2;
    P.args.dbg = dbg.as<uint8_t>();
    const size_t bw = (size_t)s->nw * 8;
    if (cudaMemcpyAsync(P.x.p, x, bw, cudaMemcpyHostToDevice, P.stream) != cudaSuccess) return -2;
    if (cudaMemcpyAsync(P.y.p, y, bw, cudaMemcpyHostToDevice, P.stream) != cudaSuccess) return -2;
    prepare_kernel<<<P.grid_prep, 128, (size_t)4 * P.smem_words * 8, P.stream>>>(P.args);
    cudaMemsetAsync(P.counter.p, 0, P.counter.n, P.stream);
    enum_kernel<2><<<P.grid_enum, P.block_enum, 0, P.stream>>>(P.args);
    JobDev J;
    std::vector<uint8_t> dev((size_t)1 << d);
    if (cudaMemcpyAsync(&J, P.jobs.p, sizeof(JobDev), cudaMemcpyDeviceToHost, P.stream) != cudaSuccess) return -2;
    if (cudaMemcpyAsync(dev.data(), dbg.p, (size_t)1 << d, cudaMemcpyDeviceToHost, P.stream) != cudaSuccess) return -2;
    cudaError_t e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) {
        g_err = cudaGetErrorString(e);
        return -2;
    }
    // the kernel indexes branches in the device's coordinate order: back to the reference's
    const EngineDev &E = view.dev[0];
    for (uint64_t sr = 0; sr < (1ull << d); sr++) out[sr] = dev[(size_t)to_device_order(E, sr)];
    return J.vanish ? -1 : d;
}

PQ_API pq_status pq_debug_prepare(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y, uint64_t *out) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    pq_status st = check_n(n);
    if (st != PQ_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    CU(cudaSetDevice(s->device));
    Plan *P = nullptr;
    st = sim_plan(s, n, &P);
    if (st != PQ_OK) return st;
    const size_t bw = (size_t)n * s->nw * 8;
    CU(cudaMemcpyAsync(P->x.p, x, bw, cudaMemcpyHostToDevice, P->stream));
    CU(cudaMemcpyAsync(P->y.p, y, bw, cudaMemcpyHostToDevice, P->stream));
    CU(cudaMemsetAsync(P->errflag.p, 0, sizeof(int), P->stream));
    prepare_kernel<<<P->grid_prep, 128, (size_t)4 * P->smem_words * 8, P->stream>>>(P->args);
    CU(cudaGetLastError());
    std::vector<JobDev> jobs((size_t)P->njobs);
    CU(cudaMemcpyAsync(jobs.data(), P->jobs.p, sizeof(JobDev) * jobs.size(), cudaMemcpyDeviceToHost, P->stream));
    CU(cudaStreamSynchronize(P->stream));
    // jobs are laid out boundary-major, then branch engine (build_plan); the Z4 increments of
    // the low coordinates are mapped from the device's coordinate order back to the reference's
    const size_t nb = s->main.dev.size();
    for (size_t j = 0; j < jobs.size(); j++) {
        const JobDev &J = jobs[j];
        const EngineDev &E = s->main.dev[j % nb];
        uint64_t *rec = out + j * kPrepWords;
        std::memset(rec, 0, sizeof(uint64_t) * kPrepWords);
        if (J.vanish) {
            rec[0] = 1;
            continue;
        }
        if (J.err) return fail(PQ_ERR_INTERNAL, "device self-check failed (odd Z8 increment)");
        rec[1] = J.phase;
        rec[2] = J.k0;
        rec[3] = J.y0;
        for (int jd = 0; jd < E.d && jd < 64; jd++) {
            const int jr = jd < 64 ? E.cperm[jd] : jd;
            rec[4 + (jr >> 3)] |= (uint64_t)J.Lp[jd] << (8 * (jr & 7));
        }
    }
    return PQ_OK;
}

}  // extern "C"

// ========================================================================================
// Allocation-free evaluation
//
// Some callers cannot allocate device memory at the point where they need amplitudes: hosts
// whose device memory is owned by an outer allocator with a fixed budget (a framework's
// caching allocator, a serving process that has reserved its memory up front), and plugin or
// callback code that is called from a context where allocating would block, fragment the
// caller's pool or fail.  For them, pq_amplitudes_noalloc evaluates a resident simulator's
// amplitudes using only the simulator's already-uploaded structures (engine tables, engine
// records and boundary map, all allocated when the simulator was created) plus one fixed
// scratch array that lives in this file as a static __device__ variable (it exists on every
// GPU that loads the library, until the process exits).  The caller passes device pointers
// for the boundaries and the results.  The scratch holds the per-call job records, work-item
// layout and partial sums; every call overwrites it, so calls that overlap on the GPU (two
// streams, or two host threads) race on it and must be serialised by the caller.
// ========================================================================================
namespace pq {

static const int kNaMaxJobs = 4096;     // boundaries x branch engines per call
static const int kNaMaxItems = 65536;   // work items (chunk ranges) per call

struct NoAllocScratch {
    JobDev jobs[kNaMaxJobs];
    int perm[kNaMaxJobs], kinv[kNaMaxJobs], jdl[kNaMaxJobs];
    unsigned jcpi[kNaMaxJobs];
    unsigned long long jnch[kNaMaxJobs];
    long long istart[kNaMaxJobs + 1];
    int out_jobs[kNaMaxJobs + 1];
    double2 partials[kNaMaxItems];
    double2 job_vals[kNaMaxJobs];
    double job_err[kNaMaxJobs];
    unsigned long long counter;
    int errflag;
};

// The scratch array (about 1.6 MiB).  Host code must not take its address directly: the
// host-side symbol is only a stand-in; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

static std::mutex g_na_mu;
static NoAllocScratch *g_na_ptr[64] = {nullptr};  // device address of the scratch, per device

// One block: job records (boundary-major, then branch engine, as build_plan lays them out),
// identity item order, per-job shapes and the item prefix sums.  Each job gets the work shape
// the simulator's own launch plans give it, so its partial sums are the same numbers in the
// same order.
__global__ void __launch_bounds__(1024) na_layout_kernel(NoAllocScratch *S, const EngineDev *eng, int nreq, int nb,
                                                         int cpl, int umax, int umax_ctab, int use_ctab) {
    __shared__ long long part[1024];
    const int njobs = nreq * nb;
    const int per = (njobs + 1023) / 1024;
    const int j0 = threadIdx.x * per;
    long long local = 0;
    for (int j = j0; j < j0 + per && j < njobs; j++) {
        JobDev &J = S->jobs[j];
        J.engine = j % nb;
        J.iomap = 0;
        J.req = j / nb;
        J.out = j / nb;
        S->perm[j] = j;
        S->kinv[j] = j;
        const EngineDev &E = eng[j % nb];
        job_shape(E, cpl, (use_ctab && E.ctab) ? umax_ctab : umax, S->jdl[j], S->jnch[j], S->jcpi[j]);
        local += (long long)((S->jnch[j] + S->jcpi[j] - 1) / S->jcpi[j]);
    }
    part[threadIdx.x] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long acc = 0;
        for (int t = 0; t < 1024; t++) {
            long long v = part[t];
            part[t] = acc;
            acc += v;
        }
    }
    __syncthreads();
    long long acc = part[threadIdx.x];
    for (int j = j0; j < j0 + per && j < njobs; j++) {
        S->istart[j] = acc;
        acc += (long long)((S->jnch[j] + S->jcpi[j] - 1) / S->jcpi[j]);
    }
    if (threadIdx.x == 1023) S->istart[njobs] = acc;
    for (int o = threadIdx.x; o <= nreq; o += 1024) S->out_jobs[o] = o * nb;
}

}  // namespace pq

extern "C" PQ_API pq_status pq_amplitudes_noalloc(pq_sim *s, int64_t n, const uint64_t *x, const uint64_t *y,
                                                  double *out, double *errbound, void *stream) {
    if (!s || !x || !y || !out) return fail(PQ_ERR_INVALID_ARG, "null argument");
    if (s->host_only) return fail(PQ_ERR_NO_DEVICE, "simulator was created by pq_analyze (host structures only)");
    std::lock_guard<std::mutex> lk(s->mu);
    const int nb = (int)s->main.dev.size();
    if (n <= 0 || n > kNaMaxJobs || n * nb > kNaMaxJobs)
        return fail(PQ_ERR_INVALID_ARG, "pq_amplitudes_noalloc: boundaries x branch engines = " +
                                            std::to_string(n * (int64_t)nb) + " outside 1..4096 (fixed scratch size)");
    // the simulator's own launch shape, as its plans use it
    const pq_tuning tu = s->tu;
    const int umax = unit_max_of(tu);
    const int use_ctab = tu.chunk_tables == 1 ? 1 : 0;
    long long nitems = 0;
    for (int b = 0; b < nb; b++) {
        const EngineDev &E = s->main.dev[b];
        if (E.d > kMaxD || E.rank > kMaxPivots) return fail(PQ_ERR_UNSUPPORTED, "branch engine outside kernel limits");
        if (E.d > tu.max_branch_dim) return fail(PQ_ERR_ADMISSION_REFUSED, "branch dimension above the cap");
        int dl;
        unsigned long long nch;
        unsigned cpi;
        job_shape(E, tu.chunks_per_lane, unit_max_for(E, tu), dl, nch, cpi);
        nitems += n * (long long)((nch + cpi - 1) / cpi);
    }
    if (nitems > kNaMaxItems)
        return fail(PQ_ERR_INVALID_ARG, "pq_amplitudes_noalloc: " + std::to_string(nitems) +
                                            " work items exceed the fixed scratch (65536); pass fewer boundaries");
    CU(cudaSetDevice(s->device));
    if (s->device < 0 || s->device >= 64) return fail(PQ_ERR_INVALID_ARG, "device index above 63");
    NoAllocScratch *S = nullptr;
    {
        // First call on this device: look up the scratch's device address (with this
        // device current).  Make that first call before any stream capture begins.
        std::lock_guard<std::mutex> lk2(g_na_mu);
        if (!g_na_ptr[s->device]) {
            void *p = nullptr;
            CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            g_na_ptr[s->device] = reinterpret_cast<NoAllocScratch *>(p);
        }
        S = g_na_ptr[s->device];
    }
    cudaStream_t st = (cudaStream_t)stream;
    // counter and error flag must start at zero; everything else is fully rewritten below
    CU(cudaMemsetAsync(&S->counter, 0, sizeof(unsigned long long) + sizeof(int), st));
    na_layout_kernel<<<1, 1024, 0, st>>>(S, s->main.dev_rec, (int)n, nb, tu.chunks_per_lane, umax, 1, use_ctab);
    KArgs a{};
    a.engines = s->main.dev_rec;
    a.maps = s->main.map_rec;
    a.jobs = S->jobs;
    a.njobs = (int)(n * nb);
    a.perm = S->perm;
    a.kinv = S->kinv;
    a.istart = S->istart;
    a.jdl = S->jdl;
    a.jcpi = S->jcpi;
    a.jnch = S->jnch;
    a.nitems = nitems;
    a.partials = S->partials;
    a.counter = &S->counter;
    a.job_vals = S->job_vals;
    a.job_err = S->job_err;
    a.out_jobs = S->out_jobs;
    a.nout = (int)n;
    a.out = out;
    a.err = errbound;
    a.out_prob = 0;
    a.xs = x;
    a.ys = y;
    a.nw = s->nw;
    a.smem_words = std::max(8, s->main.max_words);
    a.dbg = nullptr;
    a.errflag = &S->errflag;
    a.use_ctab = use_ctab;
    const size_t psmem = (size_t)4 * a.smem_words * 8;
    if (psmem > 48 * 1024) CU(cudaFuncSetAttribute(prepare_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
    const int bw = std::max(1, std::min(8, tu.block_warps));
    const int minb = (tu.blocks_per_sm >= 2 && tu.blocks_per_sm <= 4) ? tu.blocks_per_sm : 3;
    int occ = 0;
    if (minb == 4) CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, enum_kernel<0, 4>, 32 * bw, 0));
    else if (minb == 2) CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, enum_kernel<0, 2>, 32 * bw, 0));
    else CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, enum_kernel<0, 3>, 32 * bw, 0));
    const long long want = (long long)sm_count() * std::max(occ, 1);
    const int grid_enum = (int)std::max(1LL, std::min<long long>(want, (nitems + bw - 1) / bw));
    prepare_kernel<<<std::max(1, std::min(a.njobs / 4 + 1, 65535)), 128, psmem, st>>>(a);
    if (minb == 4) enum_kernel<0, 4><<<grid_enum, 32 * bw, 0, st>>>(a);
    else if (minb == 2) enum_kernel<0, 2><<<grid_enum, 32 * bw, 0, st>>>(a);
    else enum_kernel<0, 3><<<grid_enum, 32 * bw, 0, st>>>(a);
    job_reduce_kernel<<<(a.njobs + 255) / 256, 256, 0, st>>>(a);
    out_reduce_kernel<<<(a.nout + 255) / 256, 256, 0, st>>>(a);
    CU(cudaGetLastError());
    return PQ_OK;
}

// ========================================================================================
// Serving loop: continuous batching over resident simulators
//
// pq_server_submit queues requests (amplitude, probability, single-qubit-set marginal).  A
// worker thread forms a wave from the queue head -- at most max_slots requests whose launch
// memory fits what the budget has left -- and launches it on a free stream of a small pool,
// then keeps admitting: requests that arrive while earlier waves run go into the next wave on
// another stream, so their work overlaps on the device.  Finished waves are retired in
// completion order; every result carries its submit and completion time.  A request whose
// work (branches over its branch engines) exceeds 2^cap, or whose own launch would not fit the
// budget, is completed at once with PQ_ERR_ADMISSION_REFUSED.  Each boundary's result is the same as
// when evaluated alone: a job's work decomposition does not depend on the rest of the wave.
// ========================================================================================
namespace pq {
static const int kSrvStreams = 4;

// A request whose work is above 2^split_log2 branches (pq_server::split_log2, default 28) is
// evaluated in the background, in pieces -- ranges of its branch engines, or of one engine's work
// items -- of at most 2^piece_log2 branches each (default 32: about 1.5 ms on half the SMs), one
// piece per background wave on a reduced grid, so that it never holds the whole device for long.

struct SrvReq {
    pq_request r;
    double t_submit = 0.0;
    Target *tg = nullptr;
    int64_t bytes = 0;
    int precise = 0;  // 0 the FP32 walk; 1 chunk-sum tables; 2 FP64 walk (probability re-evaluation)
    int64_t group = -1;  // piece of a split request (see pq_server::groups), else -1
    int pieces = 0;      // of a completed split request: how many pieces it took
    int eb = 0, ee = -1;
    long long ib = 0, ie = -1;
};
struct SrvWave {
    std::vector<SrvReq> reqs;
    std::unique_ptr<Plan> plan;
    pq_tuning tu{};  // launch shape of the wave
    int slot = -1;
    int precise = 0;
    bool background = false;  // one piece of a split request
    int64_t bytes = 0;
    cudaEvent_t done = nullptr;
};
// The running sum of a split request's pieces.
struct SrvGroup {
    SrvReq base;
    int remaining = 0, npieces = 0;
    int32_t status = PQ_OK;
    double re = 0.0, im = 0.0, eb = 0.0;
};

// Pieces of a request on target T under launch shape tu: consecutive branch engines while their
// branches stay within `piece`; an engine above it alone, split into ranges of its work
// items of at most `piece` branches each.
static std::vector<SrvReq> srv_split(const SrvReq &q, const pq_tuning &tu, double piece) {
    std::vector<SrvReq> out;
    const Target &T = *q.tg;
    const int nb = (int)T.dev.size();
    int b = 0;
    while (b < nb) {
        const EngineDev &E = T.dev[(size_t)b];
        const double w = std::ldexp(1.0, E.d);
        if (w > piece) {
            int dl;
            unsigned long long nch;
            unsigned cpi;
            job_shape(E, tu.chunks_per_lane, unit_max_for(E, tu), dl, nch, cpi);
            const long long nit = (long long)((nch + cpi - 1) / cpi);
            const long long per = std::max<long long>(1, (long long)(piece / (w / (double)nit)));
            for (long long i = 0; i < nit; i += per) {
                SrvReq p = q;
                p.eb = b;
                p.ee = b + 1;
                p.ib = i;
                p.ie = std::min(nit, i + per);
                out.push_back(p);
            }
            b++;
            continue;
        }
        double acc = 0.0;
        int e = b;
        while (e < nb && std::ldexp(1.0, T.dev[(size_t)e].d) <= piece &&
               acc + std::ldexp(1.0, T.dev[(size_t)e].d) <= piece) {
            acc += std::ldexp(1.0, T.dev[(size_t)e].d);
            e++;
        }
        SrvReq p = q;
        p.eb = b;
        p.ee = e;
        out.push_back(p);
        b = e;
    }
    return out;
}

// The launch shape of a request at a re-evaluation level (1: chunk-sum tables where they apply,
// the FP32 walk elsewhere; 2: the tables, the FP64 walk elsewhere).
static pq_tuning srv_tuning(const pq_tuning &tu, int precise) {
    pq_tuning t = tu;
    if (precise >= 1) t.chunk_tables = 1;
    return t;
}

// Which evaluations a target's branch engines take under a launch shape: some sum their chunks
// from chunk-sum tables (any_ctab), some walk in FP32 without tables (fp32_any), some walk in
// FP32 even with tables (fp32_rest).  Engines without a joint table use FP64 weights always.
static void eval_cover(const Target &T, const pq_tuning &tu, bool &any_ctab, bool &fp32_any, bool &fp32_rest) {
    any_ctab = fp32_any = fp32_rest = false;
    for (const auto &E : T.dev) {
        int dl;
        unsigned long long nch;
        unsigned cpi;
        job_shape(E, tu.chunks_per_lane, unit_max_for(E, tu), dl, nch, cpi);
        const bool covered = E.ctab != nullptr && (dl & 255) == E.DI;
        any_ctab = any_ctab || covered;
        fp32_any = fp32_any || E.joint;
        fp32_rest = fp32_rest || (E.joint && !covered);
    }
}

// Device bytes of one request's launch state (jobs, item partials, outputs).
static int64_t request_bytes(const Target &T, const pq_tuning &tu) {
    int64_t b = 64 + 2 * 2 * 8 + 3 * 8;  // boundaries, outputs
    for (const auto &E : T.dev) {
        int dl;
        unsigned long long nch;
        unsigned cpi;
        job_shape(E, tu.chunks_per_lane, unit_max_for(E, tu), dl, nch, cpi);
        b += (int64_t)sizeof(JobDev) + 64 + 16 * (int64_t)((nch + cpi - 1) / cpi);
    }
    return b;
}
}  // namespace pq

struct pq_server {
    std::vector<pq_sim *> sims;
    int max_slots = 256;
    int64_t budget = 0;
    int max_d = 48;
    int device = 0;
    double t0 = 0.0;
    std::vector<cudaStream_t> streams;
    std::vector<double *> hbuf;  // pinned per stream: max_slots x (re, im, err)
    std::vector<char> busy;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<pq::SrvReq> pending;
    std::vector<pq_result> finished;
    std::vector<std::unique_ptr<pq::SrvWave>> inflight;
    int64_t inflight_bytes = 0;
    bool stop = false;
    std::thread worker;
    // marginal requests whose sandwich engines are not built yet wait here, by (simulator,
    // qubit), while the builder thread builds them; the worker keeps admitting other requests
    std::map<std::pair<int, int>, std::vector<pq::SrvReq>> parked;
    std::deque<std::pair<int, int>> build_q;
    std::condition_variable cv_build;
    std::thread builder;
    bool stop_builder = false;  // set once the worker has exited
    // pieces of split requests, launched one per background wave while a stream is free
    std::deque<pq::SrvReq> bg;
    std::map<int64_t, pq::SrvGroup> groups;
    int64_t next_group = 0;
    bool bg_inflight = false;
    int split_log2 = 28, piece_log2 = 32;
    ~pq_server() {
        for (auto s : streams) cudaStreamDestroy(s);
        for (auto p : hbuf) cudaFreeHost(p);
    }
};

namespace pq {
static double srv_now(const pq_server *S) { return now_s() - S->t0; }

static pq_result srv_result(const SrvReq &q, int32_t status, double t) {
    pq_result r;
    std::memset(&r, 0, sizeof(r));
    r.tag = q.r.tag;
    r.status = status;
    r.kind = q.r.kind;
    r.submit_s = q.t_submit;
    r.done_s = t;
    r.level = q.precise;
    r.pieces = q.pieces;
    return r;
}

// Resolve a request's target.  A marginal whose sandwich engines are not built yet returns
// false: the caller parks it for the builder thread.
static bool srv_resolve(pq_server *S, SrvReq &q) {
    pq_sim *s = S->sims[q.r.sim];
    if (q.r.kind != PQ_REQ_MARGINAL) {
        q.tg = &s->main;
        return true;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->marg.find(std::vector<int>{q.r.qubit});
    if (it == s->marg.end()) return false;
    q.tg = &it->second->tg;
    return true;
}

// Builder thread: builds the sandwich engines of parked marginal requests, one measured qubit
// at a time, without holding the server's or the simulator's lock during the build, then
// returns the requests to the head of the queue (or completes them with the build's error).
static void srv_build_loop(pq_server *S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        S->cv_build.wait(lk, [&] { return S->stop_builder || !S->build_q.empty(); });
        if (S->build_q.empty()) break;  // the worker has exited: nothing can be parked any more
        const std::pair<int, int> key = S->build_q.front();
        S->build_q.pop_front();
        lk.unlock();
        pq_sim *s = S->sims[key.first];
        const int32_t qb = key.second;
        int di = 10;
        bool have = false;
        {
            std::lock_guard<std::mutex> l2(s->mu);
            ensure_sandwich(s);
            di = s->di_max;
            have = s->marg.count(std::vector<int>{qb}) != 0;
        }
        pq_status st = PQ_OK;
        std::string why;
        if (!have) {
            std::unique_ptr<pq_sim::Marg> M;
            st = marg_build(s, &qb, 1, di, M);
            if (st != PQ_OK) why = g_err;
            else {
                std::lock_guard<std::mutex> l2(s->mu);
                s->marg.emplace(std::vector<int>{qb}, std::move(M));  // kept if another call built it first
            }
        }
        lk.lock();
        auto it = S->parked.find(key);
        if (it != S->parked.end()) {
            std::vector<SrvReq> rs = std::move(it->second);
            S->parked.erase(it);
            if (st == PQ_OK) {
                for (auto r = rs.rbegin(); r != rs.rend(); ++r) S->pending.push_front(*r);
            } else {
                const double t = srv_now(S);
                for (auto &r : rs) S->finished.push_back(srv_result(r, st, t));
                S->cv_done.notify_all();
            }
        }
        S->cv_work.notify_all();
    }
}

static pq_status srv_launch(pq_server *S, SrvWave &w, const pq_tuning &tu) {
    // group by target (stable), boundaries in that order
    std::stable_sort(w.reqs.begin(), w.reqs.end(), [](const SrvReq &a, const SrvReq &b) { return a.tg < b.tg; });
    std::vector<Segment> segs;
    for (auto &q : w.reqs) {
        const bool same = !segs.empty() && segs.back().tg == q.tg && segs.back().eb == q.eb && segs.back().ee == q.ee &&
                          segs.back().ib == q.ib && segs.back().ie == q.ie;
        if (!same) segs.push_back(Segment(q.tg, 0, q.eb, q.ee, q.ib, q.ie));
        segs.back().count++;
    }
    const int n = (int)w.reqs.size();
    std::vector<uint64_t> xs((size_t)2 * n), ys((size_t)2 * n);
    for (int i = 0; i < n; i++) {
        const pq_request &r = w.reqs[i].r;
        xs[2 * i] = r.x[0];
        xs[2 * i + 1] = r.x[1];
        if (r.kind == PQ_REQ_MARGINAL) {
            ys[2 * i] = ys[2 * i + 1] = 0;
            if (r.outcome) ys[2 * i + (r.qubit >> 6)] |= 1ull << (r.qubit & 63);
        } else {
            ys[2 * i] = r.y[0];
            ys[2 * i + 1] = r.y[1];
        }
    }
    cudaStream_t st = S->streams[w.slot];
    w.plan = std::make_unique<Plan>();
    w.tu = srv_tuning(tu, w.precise);
    pq_status ps = build_plan(segs, 2, st, w.tu, *w.plan, true);
    if (ps != PQ_OK) return ps;
    Plan &P = *w.plan;
    // a background piece runs on one block per SM, leaving room for foreground waves
    if (w.background) P.grid_enum = std::min(P.grid_enum, sm_count());
    CU(cudaMemcpyAsync(P.x.p, xs.data(), xs.size() * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.y.p, ys.data(), ys.size() * 8, cudaMemcpyHostToDevice, st));
    CU(enqueue_core(P, w.precise == 2 ? 1 : 0));
    double *hb = S->hbuf[w.slot];
    CU(cudaMemcpyAsync(hb, P.out.p, (size_t)n * 16, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(hb + 2 * S->max_slots, P.err.p, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    CU(cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming));
    CU(cudaEventRecord(w.done, st));
    return PQ_OK;
}

// Completion of request rq with value (re, im) and bound eb from a launch at tuning tu that did
// (used) or did not use chunk-sum tables.  Probabilities and marginals are promised to 1e-12
// absolute: when the bound cannot show it, the request goes back to the head of the queue at the
// next level that can tighten it -- the chunk-sum tables where some engine has them and this
// launch did not use them, else the FP64 walk where some engine walked in FP32 (engines without a
// joint table already used FP64 weights).  Caller holds S->mu.
static void srv_complete(pq_server *S, const SrvReq &rq, int32_t status, double re, double im, double eb,
                         const pq_tuning &tu, bool used, double t) {
    pq_result r = srv_result(rq, status, t);
    if (status == PQ_OK && rq.r.kind != PQ_REQ_AMPLITUDE && rq.precise < 2) {
        const double pb = rq.r.kind == PQ_REQ_PROBABILITY ? eb * (2.0 * std::sqrt(re * re + im * im) + eb) : eb;
        if (pb > 1e-12) {
            bool any_ctab = false, fp32_any = false, fp32_rest = false;
            eval_cover(*rq.tg, tu, any_ctab, fp32_any, fp32_rest);
            const int next = !used && any_ctab ? 1 : ((used ? fp32_rest : fp32_any) ? 2 : -1);
            if (next > 0) {
                SrvReq again = rq;
                again.precise = next;
                again.pieces = 0;
                again.group = -1;
                again.eb = 0;
                again.ee = -1;
                again.ib = 0;
                again.ie = -1;
                S->pending.push_front(again);
                return;
            }
        }
    }
    if (rq.r.kind == PQ_REQ_AMPLITUDE) {
        r.re = re;
        r.im = im;
        r.errbound = eb;
    } else if (rq.r.kind == PQ_REQ_PROBABILITY) {
        r.re = re * re + im * im;
        r.errbound = eb * (2.0 * std::sqrt(r.re) + eb);
    } else {
        r.re = re > 0.0 ? re : 0.0;
        r.errbound = eb;
    }
    S->finished.push_back(r);
}

static void srv_loop(pq_server *S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        // retire finished waves
        bool progressed = false;
        for (size_t i = 0; i < S->inflight.size();) {
            SrvWave *w = S->inflight[i].get();
            cudaError_t q = cudaEventQuery(w->done);
            if (q == cudaErrorNotReady) {
                i++;
                continue;
            }
            const double t = srv_now(S);
            const double *hb = S->hbuf[w->slot];
            const bool used = w->plan && w->plan->args.use_ctab;
            const int32_t status = q == cudaSuccess ? PQ_OK : PQ_ERR_DEVICE;
            for (size_t k = 0; k < w->reqs.size(); k++) {
                const SrvReq &rq = w->reqs[k];
                const double re = hb[2 * k], im = hb[2 * k + 1], eb = hb[2 * S->max_slots + k];
                if (rq.group < 0) {
                    srv_complete(S, rq, status, re, im, eb, w->tu, used, t);
                    continue;
                }
                // a piece: add it to its request's sum (in piece order: one piece at a time)
                auto g = S->groups.find(rq.group);
                if (g == S->groups.end()) continue;
                SrvGroup &G = g->second;
                if (status != PQ_OK) G.status = status;
                G.re += re;
                G.im += im;
                G.eb += eb;
                if (--G.remaining > 0) continue;
                SrvGroup done = G;
                S->groups.erase(g);
                done.base.pieces = done.npieces;
                // FP64 sums of the pieces: a few ulp of the magnitude
                const double eb2 = done.eb + 4.0 * 1.1102230246251565e-16 * std::sqrt(done.re * done.re + done.im * done.im);
                srv_complete(S, done.base, done.status, done.re, done.im, eb2, w->tu, used, t);
            }
            if (w->background) S->bg_inflight = false;
            S->inflight_bytes -= w->bytes;
            S->busy[w->slot] = 0;
            std::unique_ptr<SrvWave> dead = std::move(S->inflight[i]);
            S->inflight.erase(S->inflight.begin() + (long)i);
            lk.unlock();
            if (dead->done) cudaEventDestroy(dead->done);
            dead.reset();  // stream-ordered frees of the wave's buffers
            lk.lock();
            progressed = true;
        }
        if (progressed) S->cv_done.notify_all();
        if (S->stop && S->pending.empty() && S->inflight.empty() && S->parked.empty() && S->bg.empty()) break;
        auto free_slot = [&]() {
            for (int k = 0; k < (int)S->busy.size(); k++)
                if (!S->busy[k]) return k;
            return -1;
        };
        int slot = free_slot();
        pq_tuning tu;
        {
            std::lock_guard<std::mutex> g(g_mu);
            tu = g_tuning;
        }
        tu.max_branch_dim = std::min(tu.max_branch_dim, S->max_d);
        bool launched = false;
        if (slot >= 0 && !S->pending.empty()) {
            // candidates from the head of the queue
            std::vector<SrvReq> cand;
            while (!S->pending.empty() && (int)cand.size() < S->max_slots) {
                cand.push_back(S->pending.front());
                S->pending.pop_front();
            }
            const int64_t room = S->budget - S->inflight_bytes;
            lk.unlock();
            std::vector<pq_result> refused;
            auto w = std::make_unique<SrvWave>();
            std::vector<SrvReq> back, park, split;
            w->precise = cand.empty() ? 0 : cand.front().precise;
            for (auto &q : cand) {
                if (!back.empty() || q.precise != w->precise) {  // one re-evaluation level per wave
                    back.push_back(q);
                    continue;
                }
                if (!srv_resolve(S, q)) {
                    park.push_back(q);
                    continue;
                }
                // work of the request: branches over all of its branch engines
                if (q.tg->branches_per_amp > std::ldexp(1.0, S->max_d)) {
                    refused.push_back(srv_result(q, PQ_ERR_ADMISSION_REFUSED, srv_now(S)));
                    continue;
                }
                if (q.r.kind == PQ_REQ_MARGINAL && q.precise == 0 && q.tg->fp32_floor > 1e-12) {
                    // the FP32 walk cannot certify this marginal: start at the level that can
                    bool any_ctab = false, fp32_any = false, fp32_rest = false;
                    eval_cover(*q.tg, srv_tuning(tu, 1), any_ctab, fp32_any, fp32_rest);
                    const int lv = any_ctab ? 1 : (fp32_any ? 2 : 0);
                    if (lv != w->precise) {
                        q.precise = lv;
                        back.push_back(q);  // evaluated in a wave of its own level
                        continue;
                    }
                    q.precise = lv;
                }
                if (q.tg->branches_per_amp > std::ldexp(1.0, S->split_log2)) {
                    split.push_back(q);
                    continue;
                }
                q.bytes = request_bytes(*q.tg, srv_tuning(tu, q.precise));
                if (q.bytes > S->budget) {
                    refused.push_back(srv_result(q, PQ_ERR_ADMISSION_REFUSED, srv_now(S)));
                    continue;
                }
                if (w->bytes + q.bytes > room) {  // wait for memory: keep FIFO order
                    back.push_back(q);
                    continue;
                }
                w->bytes += q.bytes;
                w->reqs.push_back(q);
            }
            pq_status lst = PQ_OK;
            if (!w->reqs.empty()) {
                w->slot = slot;
                lst = srv_launch(S, *w, tu);
                if (lst != PQ_OK) {
                    for (auto &q : w->reqs) refused.push_back(srv_result(q, lst, srv_now(S)));
                    w->reqs.clear();
                    if (w->done) cudaEventDestroy(w->done);
                    w->plan.reset();
                }
            }
            lk.lock();
            for (auto it = back.rbegin(); it != back.rend(); ++it) S->pending.push_front(*it);
            for (auto &q : park) {
                const std::pair<int, int> key(q.r.sim, q.r.qubit);
                auto &v = S->parked[key];
                if (v.empty()) {
                    S->build_q.push_back(key);
                    S->cv_build.notify_one();
                }
                v.push_back(q);
            }
            for (auto &q : split) {
                std::vector<SrvReq> pieces = srv_split(q, srv_tuning(tu, q.precise), std::ldexp(1.0, S->piece_log2));
                const int64_t gid = S->next_group++;
                SrvGroup G;
                G.base = q;
                G.remaining = G.npieces = (int)pieces.size();
                S->groups[gid] = G;
                for (auto &pc : pieces) {
                    pc.group = gid;
                    pc.bytes = request_bytes(*pc.tg, srv_tuning(tu, pc.precise));
                    S->bg.push_back(pc);
                }
            }
            for (auto &r : refused) S->finished.push_back(r);
            if (!refused.empty()) S->cv_done.notify_all();
            if (!w->reqs.empty()) {
                S->busy[slot] = 1;
                S->inflight_bytes += w->bytes;
                S->inflight.push_back(std::move(w));
            }
            // requests were moved on (launched, parked, split or refused): look at the queue again
            launched = launched || !w || !park.empty() || !split.empty() || !refused.empty();
        }
        // one background piece at a time, on a free stream, when memory allows
        slot = free_slot();
        if (slot >= 0 && !S->bg_inflight && !S->bg.empty() &&
            S->bg.front().bytes <= S->budget - S->inflight_bytes) {
            auto w = std::make_unique<SrvWave>();
            w->reqs.push_back(S->bg.front());
            S->bg.pop_front();
            w->precise = w->reqs[0].precise;
            w->background = true;
            w->bytes = w->reqs[0].bytes;
            w->slot = slot;
            S->busy[slot] = 1;
            S->bg_inflight = true;
            S->inflight_bytes += w->bytes;
            lk.unlock();
            pq_status lst = srv_launch(S, *w, tu);
            lk.lock();
            if (lst != PQ_OK) {
                // the piece's request completes with the launch's error once its other pieces are in
                auto g = S->groups.find(w->reqs[0].group);
                if (g != S->groups.end()) {
                    g->second.status = lst;
                    if (--g->second.remaining == 0) {
                        S->finished.push_back(srv_result(g->second.base, lst, srv_now(S)));
                        S->groups.erase(g);
                        S->cv_done.notify_all();
                    }
                }
                if (w->done) cudaEventDestroy(w->done);
                w->plan.reset();
                S->busy[slot] = 0;
                S->bg_inflight = false;
                S->inflight_bytes -= w->bytes;
            } else {
                S->inflight.push_back(std::move(w));
                launched = true;
            }
        }
        if (launched) continue;
        // nothing launchable now: wait for a submission or poll in-flight waves again
        S->cv_work.wait_for(lk, std::chrono::microseconds(S->inflight.empty() ? 2000 : 50));
    }
}
}  // namespace pq

extern "C" {

PQ_API pq_status pq_server_create(int32_t nsims, pq_sim *const *sims, int32_t max_slots, int64_t mem_budget_bytes,
                                  int32_t max_branch_dim, pq_server **out) {
    if (nsims <= 0 || !sims || !out || max_slots <= 0 || max_slots > 65536 || mem_budget_bytes <= 0)
        return fail(PQ_ERR_INVALID_ARG, "bad server arguments");
    *out = nullptr;
    auto S = std::make_unique<pq_server>();
    for (int i = 0; i < nsims; i++) {
        if (!sims[i] || sims[i]->host_only) return fail(PQ_ERR_INVALID_ARG, "bad simulator");
        if (sims[i]->circ.nq > 128) return fail(PQ_ERR_INVALID_ARG, "served circuits are limited to 128 qubits");
        S->sims.push_back(sims[i]);
    }
    S->max_slots = max_slots;
    S->budget = mem_budget_bytes;
    S->max_d = max_branch_dim > 0 ? std::min(max_branch_dim, kMaxD) : 48;
    S->device = g_device;
    S->t0 = now_s();
    CU(cudaSetDevice(S->device));
    for (int k = 0; k < kSrvStreams; k++) {
        cudaStream_t st;
        CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        S->streams.push_back(st);
        double *hb = nullptr;
        CU(cudaMallocHost(&hb, (size_t)max_slots * 3 * sizeof(double)));
        S->hbuf.push_back(hb);
        S->busy.push_back(0);
    }
    pq_server *raw = S.release();
    raw->worker = std::thread(srv_loop, raw);
    raw->builder = std::thread(srv_build_loop, raw);
    *out = raw;
    return PQ_OK;
}

PQ_API pq_status pq_server_set_pieces(pq_server *s, int32_t split_log2, int32_t piece_log2) {
    if (!s || split_log2 < 10 || split_log2 > 62 || piece_log2 < split_log2 - 8 || piece_log2 > 62)
        return fail(PQ_ERR_INVALID_ARG, "split_log2 in 10..62, piece_log2 in split_log2-8..62");
    std::lock_guard<std::mutex> lk(s->mu);
    s->split_log2 = split_log2;
    s->piece_log2 = piece_log2;
    return PQ_OK;
}

PQ_API void pq_server_destroy(pq_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    // the worker finishes every queued and parked request (the builder keeps building for it),
    // then the builder stops
    if (s->worker.joinable()) s->worker.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop_builder = true;
    }
    s->cv_build.notify_all();
    if (s->builder.joinable()) s->builder.join();
    delete s;
}

PQ_API double pq_server_now(const pq_server *s) { return s ? srv_now(s) : 0.0; }

PQ_API pq_status pq_server_submit(pq_server *s, int64_t n, const pq_request *reqs) {
    if (!s || n < 0 || (n > 0 && !reqs)) return fail(PQ_ERR_INVALID_ARG, "bad submit arguments");
    std::vector<SrvReq> ok;
    std::vector<pq_result> bad;
    const double t = srv_now(s);
    for (int64_t i = 0; i < n; i++) {
        SrvReq q;
        q.r = reqs[i];
        q.t_submit = t;
        const pq_request &r = reqs[i];
        bool valid = r.sim >= 0 && r.sim < (int)s->sims.size() && r.kind >= 0 && r.kind <= 2;
        if (valid) {
            const int nq = s->sims[r.sim]->circ.nq;
            auto fits = [&](const uint64_t *v) {
                for (int b = nq; b < 128; b++)
                    if ((v[b >> 6] >> (b & 63)) & 1ull) return false;
                return true;
            };
            valid = fits(r.x) && (r.kind == PQ_REQ_MARGINAL || fits(r.y));
            if (r.kind == PQ_REQ_MARGINAL) valid = valid && r.qubit >= 0 && r.qubit < nq && (r.outcome == 0 || r.outcome == 1);
        }
        if (valid) ok.push_back(q);
        else bad.push_back(srv_result(q, PQ_ERR_INVALID_ARG, t));
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &q : ok) s->pending.push_back(q);
        for (auto &r : bad) s->finished.push_back(r);
    }
    s->cv_work.notify_all();
    if (!bad.empty()) s->cv_done.notify_all();
    return PQ_OK;
}

PQ_API int64_t pq_server_poll(pq_server *s, pq_result *out, int64_t cap, double timeout_s) {
    if (!s || !out || cap <= 0) return 0;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->finished.empty() && timeout_s > 0)
        s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return !s->finished.empty(); });
    const int64_t k = std::min<int64_t>(cap, (int64_t)s->finished.size());
    for (int64_t i = 0; i < k; i++) out[i] = s->finished[i];
    s->finished.erase(s->finished.begin(), s->finished.begin() + k);
    return k;
}

PQ_API pq_status pq_server_drain(pq_server *s, double timeout_s) {
    if (!s) return fail(PQ_ERR_INVALID_ARG, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                  [&] {
                                      return s->pending.empty() && s->inflight.empty() && s->parked.empty() &&
                                             s->bg.empty() && s->groups.empty();
                                  });
    return ok ? PQ_OK : fail(PQ_ERR_TIMEOUT, "requests still pending after the timeout");
}

}  // extern "C"
