// Host orchestration and the C ABI (include/darcy_gpu.h).
//
// Single large solves go to the grid engine: a per-(n, options) plan owns the
// device buffers and one CUDA graph holding the whole solve -- hierarchy
// setup, CG init, first preconditioning, a device-side while loop over CG
// iterations (conditional graph node), and the honest-residual check -- so a
// solve is H2D copies, one graph launch, D2H copies. Small and batched solves
// go to the block engine (one CTA per problem, one launch per batch).
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <atomic>
#include <thread>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/darcy_gpu.h"
#include "engine.h"

using namespace dgpu;

namespace {

thread_local std::string g_err;

struct Failure {
    int code;
    std::string msg;
};

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, int line) {
    char buf[512];
    std::snprintf(buf, sizeof buf, "CUDA error %s (%s) at solver.cu:%d in %s", cudaGetErrorName(e),
                  cudaGetErrorString(e), line, what);
    throw Failure{e == cudaErrorMemoryAllocation ? DGPU_NO_MEMORY : DGPU_CUDA_ERROR, buf};
}
#define CK(call)                                          \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) throw_cuda(e_, #call, __LINE__); \
    } while (0)

[[noreturn]] void invalid(const std::string& msg) { throw Failure{DGPU_INVALID_INPUT, msg}; }

// Grid-engine cut-off: the levels of side <= kTailSide form the coarse tail,
// applied as one dense matrix (precomputed at setup) per visit. (A 64-side
// tail for the FP32 cycle -- a 64 MB operator that stays in L2 -- measured
// slower at 1024^2: 44.5 against 38.9 ms, its 4096-column setup and 64 MB
// products outweighing the launches it saves.)
constexpr int kTailSide = 32;
// Batch routing between the engines. A problem of side >= kGridEngineMinSide
// goes to the grid engine, several such solves at once on their own streams
// (grid_solve_many), after the block engine has run the rest: on one CTA it
// would outlast the rest of the batch, and beside many smaller problems it
// would also set the block launch's shape (the autotuner keys on the largest
// side: 1024 threads and one problem per SM for sides >= 256), which the
// small problems then run with. Measured on GB300 (FP64 / mixed): 64 x 384^2
// at contrast 1e4, 481 / 553 ms on the block engine against 199 / 177 ms on
// the grid engine; 64 x 512^2, 1097 / 1188 against 373 / 307 ms; 128 x 256^2
// at contrast 4, 71 / 55 against 182 / 140 ms (hence the lower bound);
// 16384 x 128^2 + 64 x 512^2 end to end, 1.64 / 1.29 s with the 512^2
// problems in the block launch against 1.49-1.62 / 1.10 s routed.
constexpr int kGridEngineMinSide = 384;
// Grid-engine levels of at least this side run the unfused kernels (see
// emit_visit_hybrid); smaller ones the fused visits. Measured on GB300
// (mixed / FP64, ms per solve, all-fused -> unfused from this side):
// 1024^2 at contrast 1e6 30.8 / 38.6 -> 30.6 / 36.9 (side 512: 32.1 / 38.1);
// 2048^2 314 / 411 -> 275 / 364; 4096^2 at contrast 4 91.0 / 127 -> 71.4 / 108.
// The fused visits stage a halo tile and run several barrier-separated
// phases per tile, too few loads in flight to stream a large level; the
// unfused kernels stream it at 60-98% of HBM bandwidth.
constexpr int kUnfusedSide = 1024;
// Concurrent grid-engine solves of a batch of large problems.
constexpr int kGridSlots = 4;
constexpr int kChunk = 8;  // iterations per launch when conditional nodes are unavailable

// Two-pass layout of one device allocation: a pass with base == nullptr only
// measures, the second carves 256-byte-aligned pieces from a buffer of the
// measured size. Running the same layout code both times is what keeps the
// size and the carving from drifting apart.
struct Carver {
    char* base = nullptr;
    size_t cap = 0, off = 0;
    template <class T>
    T* take(size_t count) {
        char* p = base ? base + off : nullptr;
        off += align_up(count * sizeof(T));
        if (base && off > cap) throw Failure{DGPU_CUDA_ERROR, "internal layout overflow"};
        return (T*)p;
    }
};

// One owned device allocation.
struct Arena {
    char* base = nullptr;
    size_t size = 0;
    Arena() = default;
    Arena(const Arena&) = delete;
    Arena& operator=(const Arena&) = delete;
    ~Arena() {
        if (base) cudaFree(base);
    }
    void reserve(size_t bytes) {
        if (bytes <= size) return;
        if (base) cudaFree(base);
        base = nullptr;
        size = 0;
        CK(cudaMalloc(&base, bytes));
        size = bytes;
    }
};

template <class T>
struct DVec {
    T* p = nullptr;
    size_t n = 0;
    ~DVec() {
        if (p) cudaFree(p);
    }
    T* ensure(size_t count) {
        if (count <= n && p) return p;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        CK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
        n = std::max<size_t>(count, 1);
        return p;
    }
};

template <class T>
struct HVec {  // pinned host staging
    T* p = nullptr;
    size_t n = 0;
    ~HVec() {
        if (p) cudaFreeHost(p);
    }
    T* ensure(size_t count) {
        if (count <= n && p) return p;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        CK(cudaMallocHost(&p, std::max<size_t>(count, 1) * sizeof(T)));
        n = std::max<size_t>(count, 1);
        return p;
    }
};

std::vector<int> level_sides(int n) {
    std::vector<int> s;
    for (int v = n; (int)s.size() < kMaxLevels;) {
        s.push_back(v);
        if (v <= 1) break;
        v = (v + 1) / 2;
    }
    return s;
}

// ------------------------------------------------------------------ grid plan

struct PlanKey {
    int n, form, pc, pre, post, gamma, has_f, has_u0;
    int slot = 0;  // instance of concurrent solves (grid_solve_many), 0 otherwise
    bool operator<(const PlanKey& o) const {
        return std::tie(n, form, pc, pre, post, gamma, has_f, has_u0, slot) <
               std::tie(o.n, o.form, o.pc, o.pre, o.post, o.gamma, o.has_f, o.has_u0, o.slot);
    }
};

struct GridPlan {
    PlanKey key{};
    int n = 0, nlev = 0, tail_l0 = 0;
    int ntail = 0;                  // cells of the first tail level (dense operator is ntail x ntail)
    int64_t m = 0;
    bool mixed_mg = false;
    int lf = 0;  // first level of the fused visits (the levels above it run the unfused kernels)
    Arena arena;
    double *a = nullptr, *f = nullptr, *u0 = nullptr, *u = nullptr;
    double *b = nullptr, *r = nullptr, *p = nullptr, *ap = nullptr, *z = nullptr;
    float *x0f = nullptr, *b0f = nullptr, *b0lo = nullptr;
    std::vector<float*> elo, nlo, dlo;  // FP32 lo parts of the coefficients (mixed form)
    std::vector<Lvl64> h;
    std::vector<Lvl<double>> lvd;
    std::vector<Lvl<float>> lvf;
    // two iterate buffers per level for the fused visit kernels (ping-pong);
    // as double* for the FP64 cycle, reinterpreted as float* for the FP32 one
    std::vector<double*> X0, X1;
    bool fused = false;
    void* lv_dev = nullptr;
    Lvl64* h_dev = nullptr;
    double* Td = nullptr;           // dense coarse-tail operator, FP64
    float* Tf = nullptr;            // same, rounded to FP32 (mixed form)
    CgState* st = nullptr;
    double* partials = nullptr;
    DVec<double> history;
    HVec<CgState> st_host;
    bool cond = false;
    size_t nodes_pro = 0, nodes_body = 0, nodes_epi = 0;  // kernel nodes per graph part
    cudaGraphConditionalHandle handle = 0;
    cudaGraphExec_t exec = nullptr;     // whole solve (conditional mode)
    cudaGraphExec_t ex_pro = nullptr, ex_chunk = nullptr, ex_epi = nullptr;  // chunked mode
    cudaGraphExec_t ex_pc = nullptr;    // preconditioner only (apply_preconditioner)
    GridPlan() = default;
    GridPlan(const GridPlan&) = delete;
    GridPlan& operator=(const GridPlan&) = delete;
    ~GridPlan() {
        for (cudaGraphExec_t g : {exec, ex_pro, ex_chunk, ex_epi, ex_pc})
            if (g) cudaGraphExecDestroy(g);
    }
};

struct BlockConfigPOD {
    int threads;
    size_t smem;
};

}  // namespace

struct dgpu_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::mutex mu;
    bool cond_ok = false;
    cudaStream_t copy_stream = nullptr;  // host<->device copies of pipelined batches
    cudaStream_t stream2 = nullptr;      // second compute stream of pipelined batches
    std::vector<cudaEvent_t> chunk_events;
    int sms = 0;
    std::string info;
    std::map<PlanKey, std::unique_ptr<GridPlan>> plans;
    // block-engine buffers
    DVec<double> ba, bf, bu0, bu, bres, btrue, bhist;
    DVec<int> border, bside, biter, bconv, blev;
    DVec<int64_t> boff;
    DVec<unsigned long long> bbad;
    DVec<unsigned> bwork;
    DVec<char> bscratch, bscratch2;  // per-CTA arenas of the two compute streams of a pipelined batch
    DVec<char> flush;
    // apply_operator / hierarchy buffers
    DVec<char> misc;
    int64_t last_launches = 0;
    // batched-engine autotuning cache
    std::string device_name;
    bool tune_loaded = false;
    std::map<std::string, BlockConfigPOD> tuned;
    int last_block_threads = 0;
    size_t last_block_smem = 0;
    // concurrent grid-engine solves: one stream, event pair and plan per slot
    std::vector<cudaStream_t> slot_streams;
    std::vector<cudaEvent_t> slot_events;
    std::map<PlanKey, std::unique_ptr<GridPlan>> slot_plans;
    std::vector<PlanKey> slot_families;  // families with slot plans, least recently used first
};

namespace {

// ------------------------------------------------------------ plan building

// Levels of at least this side run the unfused kernels inside the fused
// W-cycle (DARCY_GPU_UNFUSED_SIDE overrides).
int unfused_side() {
    const char* e = std::getenv("DARCY_GPU_UNFUSED_SIDE");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 ? v : kUnfusedSide;
}

void alloc_plan(dgpu_context* C, GridPlan& P) {
    const PlanKey& K = P.key;
    P.n = K.n;
    P.m = (int64_t)K.n * K.n;
    const std::vector<int> sides = level_sides(K.n);
    P.nlev = (int)sides.size();
    P.mixed_mg = K.form == DGPU_FORM_MIXED && K.pc == kPcMultigrid;
    P.tail_l0 = P.nlev - 1;
    for (int l = 0; l < P.nlev; ++l)
        if (sides[l] <= kTailSide) {
            P.tail_l0 = l;
            break;
        }
    P.ntail = sides[P.tail_l0] * sides[P.tail_l0];
    const size_t m = (size_t)P.m;
    P.h.assign(P.nlev, Lvl64{});
    P.lvd.assign(P.nlev, Lvl<double>{});
    P.lvf.assign(P.nlev, Lvl<float>{});
    P.X0.assign(P.nlev, nullptr);
    P.X1.assign(P.nlev, nullptr);
    P.elo.assign(P.nlev, nullptr);
    P.nlo.assign(P.nlev, nullptr);
    P.dlo.assign(P.nlev, nullptr);
    P.fused = K.pre == 1 && K.post == 1;
    P.lf = 0;
    if (P.fused) {
        const int side = unfused_side();
        while (P.lf < P.tail_l0 && sides[P.lf] >= side) ++P.lf;
    }
    auto layout = [&](Carver& A) {
        P.a = A.take<double>(m);
        P.f = A.take<double>(m);
        P.u0 = A.take<double>(m);
        P.u = A.take<double>(m);
        P.b = A.take<double>(m);
        P.r = A.take<double>(m);
        P.p = A.take<double>(m);
        P.ap = A.take<double>(m);
        P.z = A.take<double>(m);
        P.x0f = A.take<float>(m);
        P.b0f = A.take<float>(m);
        P.b0lo = A.take<float>(m);
        for (int l = 0; l < P.nlev; ++l) {
            const size_t ml = (size_t)sides[l] * sides[l];
            Lvl64& H = P.h[l];
            H.n = sides[l];
            H.e = A.take<double>(ml);
            H.nf = A.take<double>(ml);
            H.d = A.take<double>(ml);
            H.id = A.take<double>(ml);
            H.wb = A.take<double>(sides[l]);
            H.sb = A.take<double>(sides[l]);
            Lvl<float>& F = P.lvf[l];
            F.n = sides[l];
            F.e = A.take<float>(ml);
            F.nf = A.take<float>(ml);
            F.d = A.take<float>(ml);
            F.id = A.take<float>(ml);
            P.elo[l] = A.take<float>(ml);
            P.nlo[l] = A.take<float>(ml);
            P.dlo[l] = A.take<float>(ml);
            Lvl<double>& D = P.lvd[l];
            D.n = sides[l];
            D.e = H.e;
            D.nf = H.nf;
            D.d = H.d;
            D.id = H.id;
            double* xv = A.take<double>(ml);
            double* bv = A.take<double>(ml);
            double* xa = A.take<double>(ml);
            if (l == 0) {
                P.X0[0] = xa;
                P.X1[0] = P.mixed_mg ? (double*)P.x0f : P.z;
            } else {
                P.X0[l] = xv;
                P.X1[l] = xa;
            }
            if (l == 0) {
                D.x = P.z;
                D.b = P.r;
                F.x = P.x0f;
                F.b = P.b0f;
            } else {
                D.x = xv;
                D.b = bv;
                F.x = (float*)xv;
                F.b = (float*)bv;
            }
        }
        P.Td = A.take<double>((size_t)P.ntail * P.ntail);
        P.Tf = A.take<float>((size_t)P.ntail * P.ntail);
        P.h_dev = A.take<Lvl64>(kMaxLevels);
        P.lv_dev = A.take<Lvl<double>>(kMaxLevels);
        P.st = A.take<CgState>(1);
        P.partials = A.take<double>(2 * kMaxBlocks);
    };
    Carver probe;
    layout(probe);
    P.arena.reserve(probe.off);
    Carver real{P.arena.base, P.arena.size, 0};
    layout(real);
    CK(cudaMemcpy(P.h_dev, P.h.data(), sizeof(Lvl64) * P.nlev, cudaMemcpyHostToDevice));
    if (P.mixed_mg)
        CK(cudaMemcpy(P.lv_dev, P.lvf.data(), sizeof(Lvl<float>) * P.nlev, cudaMemcpyHostToDevice));
    else
        CK(cudaMemcpy(P.lv_dev, P.lvd.data(), sizeof(Lvl<double>) * P.nlev, cudaMemcpyHostToDevice));
    P.st_host.ensure(1);
    (void)C;
}

template <class T>
const std::vector<Lvl<T>>& levels_of(const GridPlan& P);
template <>
const std::vector<Lvl<double>>& levels_of<double>(const GridPlan& P) {
    return P.lvd;
}
template <>
const std::vector<Lvl<float>>& levels_of<float>(const GridPlan& P) {
    return P.lvf;
}

template <class T>
const T* tail_matrix(const GridPlan& P);
template <>
const double* tail_matrix<double>(const GridPlan& P) {
    return P.Td;
}
template <>
const float* tail_matrix<float>(const GridPlan& P) {
    return P.Tf;
}

// Host mirror of run_cycle (multigrid.hpp:97-127) for the large levels; the
// levels from tail_l0 down are one dense matvec per parent visit.
template <class T>
void emit_visit(GridPlan& P, int l, bool first, cudaStream_t s) {
    const auto& lv = levels_of<T>(P);
    const PlanKey& K = P.key;
    const Lvl<T>& A = lv[l];
    for (int q = 0; q < K.pre; ++q) {
        launch_gs<T>(A, 0, first && q == 0, P.st, s);
        launch_gs<T>(A, 1, false, P.st, s);
    }
    if constexpr (sizeof(T) == 4)  // the FP32 cycle restricts a double-float residual
        launch_residual_restrict_df(A, P.elo[l], P.nlo[l], P.dlo[l], l == 0 ? P.b0lo : nullptr, lv[l + 1].b, P.st,
                                    s);
    else
        launch_residual_restrict<T>(A, lv[l + 1].b, P.st, s);
    if (l + 1 >= P.tail_l0) {
        launch_tail_matvec<T>(tail_matrix<T>(P), P.ntail, lv[l + 1].b, lv[l + 1].x, P.st, s);
    } else {
        for (int g = 0; g < K.gamma; ++g) emit_visit<T>(P, l + 1, g == 0, s);
    }
    launch_prolong_gs1<T>(A, lv[l + 1].x, P.st, s);
    for (int q = 0; q < K.post; ++q) {
        if (q > 0) launch_gs<T>(A, 1, false, P.st, s);
        if (l == 0 && q + 1 == K.post)
            launch_gs0_dot<T>(A, P.r, P.st, P.partials, s);
        else
            launch_gs<T>(A, 0, false, P.st, s);
    }
}

// What the fused visit kernels read for level l: the FP64 hierarchy, or the
// FP32 hi/lo pairs of the mixed form (with r's lo part on level 0).
template <class T>
VisitLevel<T> visit_level(const GridPlan& P, int l);
template <>
VisitLevel<double> visit_level<double>(const GridPlan& P, int l) {
    const Lvl64& H = P.h[l];
    return VisitLevel<double>{H.n, H.e, H.nf, H.d, H.id, nullptr, nullptr, nullptr, P.lvd[l].b, nullptr};
}
template <>
VisitLevel<float> visit_level<float>(const GridPlan& P, int l) {
    const Lvl<float>& F = P.lvf[l];
    return VisitLevel<float>{F.n, F.e, F.nf, F.d, F.id, P.elo[l], P.nlo[l], P.dlo[l], F.b, l == 0 ? P.b0lo : nullptr};
}

// Fused visits (pre_sweeps = post_sweeps = 1). The host walks the
// recursion (multigrid.hpp:97-127) into a list of level operations, merges
// every post-visit that is directly followed by the next call's pre-visit of
// the same level into one kernel, then launches the list; iterates alternate
// between the level's two buffers, `cur` tracking which holds each level's.
enum VisitKind { kOpPre, kOpPost, kOpMid, kOpTail };
struct VisitOp {
    int kind, l;
    bool first;
};

void collect_visits(const GridPlan& P, int l, bool first, std::vector<VisitOp>& ops) {
    ops.push_back({kOpPre, l, first});
    if (l + 1 >= P.tail_l0)
        ops.push_back({kOpTail, l, false});
    else
        for (int g = 0; g < P.key.gamma; ++g) collect_visits(P, l + 1, g == 0, ops);
    ops.push_back({kOpPost, l, false});
}

// The fused ops of `calls` consecutive calls of level l_top (the first from a
// zero iterate), a post-visit followed by the next pre-visit of the same
// level merged into one mid-visit.
std::vector<VisitOp> visit_program(const GridPlan& P, int l_top = 0, int calls = 1) {
    std::vector<VisitOp> raw, ops;
    for (int c = 0; c < calls; ++c) collect_visits(P, l_top, c == 0, raw);
    for (size_t i = 0; i < raw.size(); ++i) {
        if (raw[i].kind == kOpPost && i + 1 < raw.size() && raw[i + 1].kind == kOpPre && raw[i + 1].l == raw[i].l &&
            !raw[i + 1].first) {
            ops.push_back({kOpMid, raw[i].l, false});
            ++i;
        } else {
            ops.push_back(raw[i]);
        }
    }
    return ops;
}

template <class T>
void emit_visit_fused(GridPlan& P, std::vector<int>& cur, cudaStream_t s, int l_top = 0, int calls = 1) {
    const auto& lv = levels_of<T>(P);
    const PlanKey& K = P.key;
    auto X = [&](int lvl, int q) { return (T*)(q == 0 ? P.X0[lvl] : P.X1[lvl]); };
    for (const VisitOp& op : visit_program(P, l_top, calls)) {
        const int l = op.l;
        const VisitLevel<T> V = visit_level<T>(P, l);
        switch (op.kind) {
            case kOpPre:
                if (op.first) {
                    launch_visit_pre<T>(V, nullptr, X(l, 0), lv[l + 1].b, s);
                    cur[l] = 0;
                } else {
                    launch_visit_pre<T>(V, X(l, cur[l]), X(l, cur[l] ^ 1), lv[l + 1].b, s);
                    cur[l] ^= 1;
                }
                break;
            case kOpTail:
                launch_tail_matvec<T>(tail_matrix<T>(P), P.ntail, lv[l + 1].b, X(l + 1, 0), P.st, s);
                cur[l + 1] = 0;
                break;
            case kOpPost:
                launch_visit_post<T>(V, X(l, cur[l]), X(l + 1, cur[l + 1]), X(l, cur[l] ^ 1),
                                     l == 0 ? P.r : nullptr, P.st, P.partials, s);
                cur[l] ^= 1;
                break;
            case kOpMid:
                launch_visit_mid<T>(V, X(l, cur[l]), X(l + 1, cur[l + 1]), X(l, cur[l] ^ 1), lv[l + 1].b, s);
                cur[l] ^= 1;
                break;
        }
    }
}

// Hybrid cycle: levels above P.lf (side >= kUnfusedSide) run the unfused
// kernels (one per phase, streaming at a high fraction of HBM bandwidth),
// the levels from P.lf down the fused visits (one launch per visit; the
// small levels are latency-bound). Level l < P.lf works in place on lv[l].x;
// the fused subtree below it leaves its result in X(P.lf, cur[P.lf]), which
// the prolongation of level P.lf - 1 reads. Same arithmetic as the all-fused
// program (the unfused kernels follow the fused ones' operation order).
template <class T>
void emit_visit_hybrid(GridPlan& P, int l, bool first, std::vector<int>& cur, cudaStream_t s) {
    const auto& lv = levels_of<T>(P);
    const PlanKey& K = P.key;
    const Lvl<T>& A = lv[l];
    launch_gs<T>(A, 0, first, P.st, s);
    launch_gs<T>(A, 1, false, P.st, s);
    if constexpr (sizeof(T) == 4)
        launch_residual_restrict_df(A, P.elo[l], P.nlo[l], P.dlo[l], l == 0 ? P.b0lo : nullptr, lv[l + 1].b, P.st,
                                    s);
    else
        launch_residual_restrict<T>(A, lv[l + 1].b, P.st, s);
    const T* xc;
    if (l + 1 >= P.tail_l0) {
        launch_tail_matvec<T>(tail_matrix<T>(P), P.ntail, lv[l + 1].b, lv[l + 1].x, P.st, s);
        xc = lv[l + 1].x;
    } else if (l + 1 < P.lf) {
        for (int g = 0; g < K.gamma; ++g) emit_visit_hybrid<T>(P, l + 1, g == 0, cur, s);
        xc = lv[l + 1].x;
    } else {
        emit_visit_fused<T>(P, cur, s, l + 1, K.gamma);
        xc = (const T*)(cur[l + 1] == 0 ? P.X0[l + 1] : P.X1[l + 1]);
    }
    launch_prolong_gs1<T>(A, xc, P.st, s);
    if (l == 0)
        launch_gs0_dot<T>(A, P.r, P.st, P.partials, s);
    else
        launch_gs<T>(A, 0, false, P.st, s);
}

void emit_setup(GridPlan& P, cudaStream_t s) {
    launch_build_fine(P.a, P.h[0], &P.st->bad, s);
    for (int l = 1; l < P.nlev; ++l) launch_coarsen(P.h[l - 1], P.h[l], s);
    if (P.mixed_mg)
        for (int l = 0; l < P.nlev; ++l)
            launch_to_fp32(P.h[l], (float*)P.lvf[l].e, (float*)P.lvf[l].nf, (float*)P.lvf[l].d,
                           (float*)P.lvf[l].id, P.elo[l], P.nlo[l], P.dlo[l], s);
    if (P.key.pc == kPcMultigrid) {
        // The tail operator is built in FP64 (Galerkin levels and the exact
        // coarsest solve inside it stay FP64) and rounded once for the mixed form.
        const int top_calls = P.tail_l0 == 0 ? 1 : P.key.gamma;
        launch_tail_columns(P.h_dev, P.h.data(), P.tail_l0, P.nlev, P.key.pre, P.key.post, P.key.gamma, top_calls,
                            P.ntail, P.Td, P.mixed_mg ? P.Tf : nullptr, s);
    }
}

void emit_precondition(GridPlan& P, cudaStream_t s) {
    const PlanKey& K = P.key;
    if (K.pc == kPcMultigrid) {
        if (P.tail_l0 == 0) {  // the whole hierarchy is the tail: M is one dense matrix
            if (P.mixed_mg) {
                launch_tail_matvec<float>(P.Tf, P.ntail, P.b0f, P.x0f, P.st, s);
                launch_dot_rz<float>(P.x0f, P.r, P.m, P.st, P.partials, s);
            } else {
                launch_tail_matvec<double>(P.Td, P.ntail, P.r, P.z, P.st, s);
                launch_dot_rz<double>(P.z, P.r, P.m, P.st, P.partials, s);
            }
        } else if (P.fused && P.lf > 0) {
            // unfused large levels; level 0 ends in place in lv[0].x: z / x0f
            std::vector<int> cur(P.nlev, 0);
            if (P.mixed_mg)
                emit_visit_hybrid<float>(P, 0, true, cur, s);
            else
                emit_visit_hybrid<double>(P, 0, true, cur, s);
        } else if (P.fused) {
            // level 0 ends in X1[0] (pre writes X0, post writes X1): z / x0f
            std::vector<int> cur(P.nlev, 0);
            if (P.mixed_mg)
                emit_visit_fused<float>(P, cur, s);
            else
                emit_visit_fused<double>(P, cur, s);
        } else if (P.mixed_mg) {
            emit_visit<float>(P, 0, true, s);
        } else {
            emit_visit<double>(P, 0, true, s);
        }
    } else {
        launch_precond_diag(P.r, K.pc == kPcJacobi ? P.h[0].id : nullptr, P.z, P.m, P.st, P.partials, s);
    }
}

void emit_prologue(GridPlan& P, cudaStream_t s) {
    const double hh = 1.0 / (double)(P.n + 1);
    emit_setup(P, s);
    launch_cg_init(P.key.has_f ? P.f : nullptr, hh * hh, P.m, P.b, P.r, P.u, P.p, P.mixed_mg ? P.b0f : nullptr,
                   P.b0lo, P.key.has_u0 ? P.u0 : nullptr, P.h[0], P.st, P.partials, s);
    emit_precondition(P, s);
}

void emit_body(GridPlan& P, cudaStream_t s) {
    if (P.mixed_mg)
        launch_xpby<float>(P.x0f, P.p, P.m, P.st, s);
    else
        launch_xpby<double>(P.z, P.p, P.m, P.st, s);
    launch_apply_dot(P.h[0], P.p, P.ap, P.st, P.partials, s);
    // Standard beta in both forms: the flexible (Polak-Ribiere) beta that
    // k_cg_update supports measured worse for the FP32 cycle (1024^2 at 1e6
    // contrast: 127 iterations against 114 with the standard beta).
    launch_cg_update(P.p, P.ap, P.u, P.r, P.mixed_mg ? P.b0f : nullptr, P.b0lo, nullptr, P.m, P.st, P.partials, s);
    emit_precondition(P, s);
}

void emit_epilogue(GridPlan& P, cudaStream_t s) {
    launch_true_residual(P.h[0], P.u, P.b, nullptr, P.st, P.partials, s);
}

template <class F>
cudaGraph_t capture(cudaStream_t s, F&& fn) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
        fn();
    } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    CK(cudaStreamEndCapture(s, &g));
    CK(cudaGetLastError());
    return g;
}

void build_graphs(dgpu_context* C, GridPlan& P) {
    cudaStream_t s = C->stream;
    cudaGraph_t gpro = capture(s, [&] { emit_prologue(P, s); });
    cudaGraph_t gbody = capture(s, [&] { emit_body(P, s); });
    cudaGraph_t gepi = capture(s, [&] { emit_epilogue(P, s); });
    CK(cudaGraphGetNodes(gpro, nullptr, &P.nodes_pro));
    CK(cudaGraphGetNodes(gbody, nullptr, &P.nodes_body));
    CK(cudaGraphGetNodes(gepi, nullptr, &P.nodes_epi));
    P.cond = false;
    if (C->cond_ok) {
        cudaGraph_t G = nullptr;
        CK(cudaGraphCreate(&G, 0));
        cudaGraphNode_t npro, nwhile, nepi;
        CK(cudaGraphAddChildGraphNode(&npro, G, nullptr, 0, gpro));
        CK(cudaGraphConditionalHandleCreate(&P.handle, G, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = P.handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        CK(cudaGraphAddNode(&nwhile, G, &npro, nullptr, 1, &cp));
        // The loop body is captured straight into the conditional node's body
        // graph, so the kernels that end the loop (cudaGraphSetConditional in
        // k_xpby / k_apply_dot / k_cg_update) are direct nodes of that body.
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CK(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        emit_body(P, s);
        CK(cudaStreamEndCapture(s, &body));
        CK(cudaGetLastError());
        CK(cudaGraphAddChildGraphNode(&nepi, G, &nwhile, 1, gepi));
        CK(cudaGraphInstantiate(&P.exec, G, 0));
        cudaGraphDestroy(G);
        P.cond = true;
    } else {
        cudaGraph_t chunk = nullptr;
        CK(cudaGraphCreate(&chunk, 0));
        cudaGraphNode_t prev = nullptr;
        for (int q = 0; q < kChunk; ++q) {
            cudaGraphNode_t nd;
            CK(cudaGraphAddChildGraphNode(&nd, chunk, prev ? &prev : nullptr, prev ? 1 : 0, gbody));
            prev = nd;
        }
        CK(cudaGraphInstantiate(&P.ex_pro, gpro, 0));
        CK(cudaGraphInstantiate(&P.ex_chunk, chunk, 0));
        CK(cudaGraphInstantiate(&P.ex_epi, gepi, 0));
        cudaGraphDestroy(chunk);
    }
    cudaGraphDestroy(gpro);
    cudaGraphDestroy(gbody);
    cudaGraphDestroy(gepi);
}

GridPlan& get_plan(dgpu_context* C, const PlanKey& K) {
    auto it = C->plans.find(K);
    if (it != C->plans.end()) return *it->second;
    // keep the cache bounded: plans hold O(n^2) device memory
    if (C->plans.size() >= 8) C->plans.clear();
    auto P = std::make_unique<GridPlan>();
    P->key = K;
    alloc_plan(C, *P);
    build_graphs(C, *P);
    GridPlan& ref = *P;
    C->plans.emplace(K, std::move(P));
    return ref;
}

// --------------------------------------------------------------- validation

void check_options(int64_t n, const dgpu_options* o) {
    if (!o) invalid("options must not be NULL");
    if (n < 1) invalid("grid size must be at least 1");                  // solver.hpp:85
    if (!(o->tol > 0.0)) invalid("tol must be positive");                  // solver.hpp:86
    if (o->max_iter < 1) invalid("max_iter must be at least 1");           // solver.hpp:87
    if (o->preconditioner < 0 || o->preconditioner > 2)
        invalid("unknown preconditioner; expected one of: multigrid, jacobi, none");
    if (o->pre_sweeps < 1 || o->post_sweeps < 1)                           // bindings.cpp:43-44
        invalid("pre_sweeps and post_sweeps must be at least 1");
    if (o->cycle_index < 1 || o->cycle_index > 2)                          // bindings.cpp:45-46
        invalid("cycle_index must be 1 (V-cycle) or 2 (W-cycle)");
    if (o->form != DGPU_FORM_FP64 && o->form != DGPU_FORM_MIXED) invalid("unknown form; expected fp64 or mixed");
    if (n > 46340) invalid("grid size too large for 32-bit cell rows");
}

[[noreturn]] void bad_permeability(unsigned long long k) {
    invalid("permeability must be finite and strictly positive everywhere; offending value at flat index " +
            std::to_string(k));
}

// Fault in the pages of a host output range before its copy out is issued. A
// pageable device-to-host copy into pages never written (a fresh result
// array) faults them in on the copy's own path, after the kernels that
// produce the data: ~1.5 ms for the last 33 MB chunk of a pipelined batch.
// Touching one element per page while the GPU still computes takes that off
// the critical path; on pages already mapped the loop costs a few
// microseconds. The range is output only (the copy overwrites it). A device
// pointer passed where host memory belongs is left to the copy to report.
void prefault_output(double* p, int64_t count) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess)
        (void)cudaGetLastError();  // not known to CUDA: plain host memory
    else if (at.type == cudaMemoryTypeDevice)
        return;
    static const int64_t step = std::max<int64_t>(1, (int64_t)sysconf(_SC_PAGESIZE) / (int64_t)sizeof(double));
    volatile double* v = p;
    for (int64_t k = 0; k < count; k += step) v[k] = 0.0;
    if (count > 0) v[count - 1] = 0.0;
}

// ----------------------------------------------------------------- grid solve

// One solve through plan P on stream s (events e0/e1 bracket it for
// device_ms): H2D copies, one graph launch, D2H copies, synchronise.
void grid_run(GridPlan& P, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, const double* a, const double* f,
              double fscalar, const dgpu_options* o, const double* u0, double* u_out, double* hist,
              dgpu_stats* stats, bool device_ptrs) {
    const size_t bytes = sizeof(double) * (size_t)P.m;
    const cudaMemcpyKind in = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind out = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    CgState& hs = *P.st_host.p;
    std::memset(&hs, 0, sizeof hs);
    hs.tol = o->tol;
    hs.fscalar = fscalar;
    hs.max_iter = o->max_iter;
    hs.record_history = hist ? 1 : 0;
    hs.history = hist;
    hs.use_cond = P.cond ? 1 : 0;
    hs.cond = P.handle;
    hs.bad = ~0ull;
    CK(cudaEventRecord(e0, s));
    CK(cudaMemcpyAsync(P.a, a, bytes, in, s));
    if (f) CK(cudaMemcpyAsync(P.f, f, bytes, in, s));
    if (u0) CK(cudaMemcpyAsync(P.u0, u0, bytes, in, s));
    CK(cudaMemcpyAsync(P.st, &hs, sizeof hs, cudaMemcpyHostToDevice, s));
    if (P.cond) {
        CK(cudaGraphLaunch(P.exec, s));
    } else {
        CK(cudaGraphLaunch(P.ex_pro, s));
        for (int done = 0; !done;) {
            CK(cudaGraphLaunch(P.ex_chunk, s));
            CK(cudaMemcpyAsync(&hs, P.st, sizeof hs, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            done = hs.done;
        }
        CK(cudaGraphLaunch(P.ex_epi, s));
    }
    if (!device_ptrs) prefault_output(u_out, P.m);
    CK(cudaMemcpyAsync(u_out, P.u, bytes, out, s));
    CK(cudaMemcpyAsync(&hs, P.st, sizeof hs, cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(e1, s));
    CK(cudaStreamSynchronize(s));
    if (hs.bad != ~0ull) bad_permeability(hs.bad);
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    const bool f_zero = hs.bnorm == 0.0;
    if (stats) {
        stats->iterations = hs.it;
        stats->residual = hs.residual;
        stats->converged = hs.converged;
        stats->levels = (o->preconditioner == kPcMultigrid && !f_zero) ? P.nlev : 1;
        stats->history_len = hist ? hs.it + 1 : 0;
        stats->true_residual = hs.true_residual;
        stats->device_ms = ms;
        // the loop body runs once per iteration, and once more (all early
        // exits) when the solve was already finished before the first one
        const int64_t bodies = std::max(hs.it, 1);
        stats->kernel_launches = (int64_t)P.nodes_pro + bodies * (int64_t)P.nodes_body + (int64_t)P.nodes_epi;
    }
}

void grid_solve(dgpu_context* C, const double* a, const double* f, double fscalar, int64_t n,
                const dgpu_options* o, const double* u0, double* u_out, double* history_out, dgpu_stats* stats,
                bool device_ptrs, cudaStream_t user_stream) {
    PlanKey K{(int)n, o->form, o->preconditioner, o->pre_sweeps, o->post_sweeps, o->cycle_index, f != nullptr,
              u0 != nullptr};
    GridPlan& P = get_plan(C, K);
    cudaStream_t s = C->stream;
    if (user_stream) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        CK(cudaEventRecord(e, user_stream));
        CK(cudaStreamWaitEvent(s, e, 0));
        cudaEventDestroy(e);
    }
    double* hist = nullptr;
    if (o->record_history) hist = P.history.ensure((size_t)o->max_iter + 1);
    dgpu_stats st{};
    // (grid_run synchronises s before returning, so the caller's stream is
    // ordered after the solve without a further event)
    grid_run(P, s, C->ev0, C->ev1, a, f, fscalar, o, u0, u_out, hist, &st, device_ptrs);
    if (stats) *stats = st;
    C->last_launches = st.kernel_launches;
    if (history_out && hist)
        CK(cudaMemcpy(history_out, hist, sizeof(double) * ((size_t)st.iterations + 1), cudaMemcpyDeviceToHost));
}

// Whether a batched problem of side n goes to the grid engine, in a batch of
// total_cells cells. DARCY_GPU_GRID_SIDE=s overrides: side >= s, nothing else.
bool route_to_grid(const dgpu_context* C, int64_t n, int64_t total_cells) {
    const char* e = std::getenv("DARCY_GPU_GRID_SIDE");
    const int v = e ? std::atoi(e) : 0;
    if (v >= 1) return n >= v;
    (void)C;
    (void)total_cells;
    return n >= kGridEngineMinSide;
}

// Problem families (side, form, options) whose slot plans stay allocated.
constexpr size_t kSlotFamilies = 4;

// Concurrent slots for grid_solve_many (DARCY_GPU_SLOTS overrides, 1..16).
int grid_slots() {
    const char* e = std::getenv("DARCY_GPU_SLOTS");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 && v <= 16 ? v : kGridSlots;
}

// Many grid-engine solves of one side at once. A single large solve leaves
// most SMs idle in its coarse levels (the W-cycle's many small dependent
// launches); solves on separate streams fill them. Each slot owns a plan
// (buffers + graph), a stream and a host thread that pulls problems from a
// shared counter, so pageable host arrays work and slots never wait on one
// another's copies. Problems are taken in `order`; problem q reads
// a + off[q] (u0 at the same offset when given; f too unless f_shared) and
// writes u_out + off[q].
// Returns the device time from the first to the last slot's work (ms).
float grid_solve_many(dgpu_context* C, int side, const std::vector<int64_t>& order, const std::vector<int64_t>& off,
                      const double* a, const double* f, bool f_shared, double fscalar, const dgpu_options* o,
                      const double* u0,
                      double* u_out, int* iterations, double* residuals, int* converged, int* levels,
                      bool device_ptrs) {
    const int S = (int)std::min<int64_t>((int64_t)order.size(), grid_slots());
    while ((int)C->slot_streams.size() < S) {
        cudaStream_t st;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        C->slot_streams.push_back(st);
        for (int k = 0; k < 2; ++k) {
            cudaEvent_t ev;
            CK(cudaEventCreate(&ev));
            C->slot_events.push_back(ev);
        }
    }
    // slot plans of up to kSlotFamilies problem families (they hold O(n^2)
    // memory each), the least recently used family evicted first: rebuilding a
    // family's plans and graphs costs ~1.5 ms a slot at 1024^2, which a caller
    // alternating between two forms would otherwise pay on every call
    PlanKey K{side, o->form, o->preconditioner, o->pre_sweeps, o->post_sweeps, o->cycle_index, f != nullptr,
              u0 != nullptr};
    {
        auto same = [](const PlanKey& x, const PlanKey& y) { return !(x < y) && !(y < x); };
        auto& lru = C->slot_families;  // most recent last
        for (auto it = lru.begin(); it != lru.end(); ++it)
            if (same(*it, K)) {
                lru.erase(it);
                break;
            }
        lru.push_back(K);
        while (lru.size() > kSlotFamilies) {
            const PlanKey old = lru.front();
            lru.erase(lru.begin());
            for (auto it = C->slot_plans.begin(); it != C->slot_plans.end();) {
                PlanKey k0 = it->first;
                k0.slot = 0;
                it = same(k0, old) ? C->slot_plans.erase(it) : std::next(it);
            }
        }
    }
    std::vector<GridPlan*> plans((size_t)S);
    for (int q = 0; q < S; ++q) {
        K.slot = q;
        auto it = C->slot_plans.find(K);
        if (it == C->slot_plans.end()) {
            auto P = std::make_unique<GridPlan>();
            P->key = K;
            alloc_plan(C, *P);
            build_graphs(C, *P);
            it = C->slot_plans.emplace(K, std::move(P)).first;
        }
        plans[(size_t)q] = it->second.get();
    }
    // every slot starts after the work already on the context stream
    CK(cudaEventRecord(C->ev0, C->stream));
    for (int q = 0; q < S; ++q) CK(cudaStreamWaitEvent(C->slot_streams[(size_t)q], C->ev0, 0));
    std::atomic<int64_t> next{0};
    std::atomic<bool> stop{false};
    std::vector<Failure> fails((size_t)S, Failure{DGPU_OK, ""});
    std::vector<int64_t> launches((size_t)S, 0);
    auto worker = [&](int q) {
        try {
            CK(cudaSetDevice(C->device));
            cudaStream_t s = C->slot_streams[(size_t)q];
            for (;;) {
                const int64_t k = next.fetch_add(1);
                if (k >= (int64_t)order.size() || stop.load()) break;
                const int64_t p = order[(size_t)k];
                const int64_t at = off[(size_t)p];
                dgpu_stats st{};
                grid_run(*plans[(size_t)q], s, C->slot_events[2 * (size_t)q], C->slot_events[2 * (size_t)q + 1],
                         a + at, f ? (f_shared ? f : f + at) : nullptr, fscalar, o, u0 ? u0 + at : nullptr, u_out + at, nullptr, &st,
                         device_ptrs);
                iterations[p] = st.iterations;
                residuals[p] = st.residual;
                converged[p] = st.converged;
                if (levels) levels[p] = st.levels;
                launches[(size_t)q] += st.kernel_launches;
            }
        } catch (const Failure& e) {
            fails[(size_t)q] = e;
            stop = true;
        } catch (const std::exception& e) {
            fails[(size_t)q] = Failure{DGPU_CUDA_ERROR, e.what()};
            stop = true;
        }
    };
    std::vector<std::thread> pool;
    for (int q = 1; q < S; ++q) pool.emplace_back(worker, q);
    worker(0);
    for (std::thread& t : pool) t.join();
    for (const Failure& e : fails)
        if (e.code != DGPU_OK) throw e;
    // the context stream continues after every slot
    for (int q = 0; q < S; ++q) {
        CK(cudaEventRecord(C->slot_events[2 * (size_t)q + 1], C->slot_streams[(size_t)q]));
        CK(cudaStreamWaitEvent(C->stream, C->slot_events[2 * (size_t)q + 1], 0));
    }
    CK(cudaEventRecord(C->ev1, C->stream));
    CK(cudaEventSynchronize(C->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, C->ev0, C->ev1));
    C->last_launches = std::accumulate(launches.begin(), launches.end(), (int64_t)0);
    return ms;
}

// --------------------------------------------------------------- block solves

struct BatchOut {
    int* iterations;
    double* residuals;
    int* converged;
    int* levels;
    double* true_residual;
    double* history;
};

// ---------------------------------------------------------- block autotuner
//
// The batched engine's launch shape -- threads per CTA, how many coarse levels
// live in shared memory, and so how many CTAs share an SM -- is picked per
// (size bucket, form, preconditioner, cycle) by timing the candidates on a
// sample of the actual batch (its largest problems), and cached in the
// context and in a JSON file (DARCY_GPU_TUNE_FILE, default
// _build/autotune.json beside the library).

struct BlockConfig {
    int threads = 256;
    size_t smem = 0;
};

int size_bucket(int side) {
    int b = 8;
    while (b < side) b <<= 1;
    return b;
}

std::string tune_file() {
    if (const char* env = std::getenv("DARCY_GPU_TUNE_FILE")) return env;
    Dl_info info;
    if (dladdr((void*)&dgpu_create, &info) && info.dli_fname) {
        std::string path = info.dli_fname;
        const size_t slash = path.rfind('/');
        return (slash == std::string::npos ? std::string(".") : path.substr(0, slash)) + "/_build/autotune.json";
    }
    return "autotune.json";
}

// The cache file is one JSON object: {"<device>|<key>": [threads, smem], ...}.
void load_tuning(dgpu_context* C) {
    if (C->tune_loaded) return;
    C->tune_loaded = true;
    FILE* fp = std::fopen(tune_file().c_str(), "r");
    if (!fp) return;
    std::string text;
    char buf[4096];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, got);
    std::fclose(fp);
    size_t pos = 0;
    while ((pos = text.find('"', pos)) != std::string::npos) {
        const size_t end = text.find('"', pos + 1);
        if (end == std::string::npos) break;
        const std::string key = text.substr(pos + 1, end - pos - 1);
        int threads = 0;
        unsigned long long smem = 0;
        // (a shape the kernel cannot take -- threads not a multiple of 32 in
        // 32..1024, or more shared memory than a CTA has -- is ignored)
        if (std::sscanf(text.c_str() + end + 1, " : [ %d , %llu ]", &threads, &smem) == 2 && threads >= 32 &&
            threads <= 1024 && threads % 32 == 0 && smem <= 200ull * 1024)
            C->tuned[key] = BlockConfigPOD{threads, (size_t)smem};
        pos = end + 1;
    }
}

void save_tuning(dgpu_context* C) {
    const std::string path = tune_file();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        std::string dir = path.substr(0, slash);
        std::string cmd_dir = dir;  // create the directory if missing (no shell)
        mkdir(cmd_dir.c_str(), 0755);
    }
    FILE* fp = std::fopen(path.c_str(), "w");
    if (!fp) return;
    std::fprintf(fp, "{\n");
    size_t q = 0;
    for (const auto& kv : C->tuned)
        std::fprintf(fp, "  \"%s\": [%d, %zu]%s\n", kv.first.c_str(), kv.second.threads, kv.second.smem,
                     ++q < C->tuned.size() ? "," : "");
    std::fprintf(fp, "}\n");
    std::fclose(fp);
}

// Shared memory for the batched engine's coarse levels and dense tail: sized
// so that a 64^2 problem keeps levels 32^2 and 16^2 and its 64 x 64 tail on
// chip with two CTAs per SM.
size_t smem_budget_for(bool mixed) { return mixed ? 48 * 1024 : 96 * 1024; }
// A budget large enough for the whole FP32 cycle of a 64^2 problem (every
// level and the tail on chip, one CTA per SM): then only the FP64 CG vectors
// and fine-level coefficients live in global memory.
constexpr size_t kSmemBudgetLarge = 180 * 1024;
// Level 0 of a 64^2 FP32 cycle alone (6 x 16 KiB), two CTAs of up to 512
// threads per SM: the cycle's heaviest level on chip, and the FP64 CG vectors
// and coefficients of the two resident problems per SM (~300 KB each) within
// the L2.
constexpr size_t kSmemBudgetLevel0 = 100 * 1024;

// Autotuning key of a batch (loads the tuning file on first use). Batches
// too small to put 4 problems on every SM ("few") tune apart from larger ones
// ("many"): the best shape differs (more threads per problem when problems
// are scarce), and a shape tuned on a first small batch would otherwise be
// reused for every large one.
std::string tune_key(dgpu_context* C, int maxside, bool mixed, const dgpu_options* o, int64_t count) {
    char keybuf[176];
    std::snprintf(keybuf, sizeof keybuf, "%s|side<=%d|%s|pc%d|c%d|s%d%d|%s", C->device_name.c_str(),
                  size_bucket(maxside), mixed ? "mixed" : "fp64", o->preconditioner, o->cycle_index,
                  o->pre_sweeps, o->post_sweeps, count >= 4 * (int64_t)std::max(C->sms, 1) ? "many" : "few");
    load_tuning(C);
    return keybuf;
}

// Packed problems through the block engine. sides/off on the host; a, f, u0
// host (or device when device_ptrs) packed arrays.
void block_solve(dgpu_context* C, int64_t count, const std::vector<int>& sides, const std::vector<int64_t>& off,
                 const double* a, const double* f, int f_shared, double fscalar, const double* u0,
                 const dgpu_options* o, double* u_out, BatchOut out, bool device_ptrs, float* ms_out,
                 const std::function<void(const double*, double*, cudaStream_t)>* warm = nullptr) {
    cudaStream_t s = C->stream;
    const int64_t total = off[count - 1] + (int64_t)sides[count - 1] * sides[count - 1];
    const int maxside = *std::max_element(sides.begin(), sides.end());
    const bool mixed = o->form == DGPU_FORM_MIXED && o->preconditioner == kPcMultigrid;
    const cudaMemcpyKind in = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind outk = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;

    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sides[x] > sides[y]; });

    // host arrays read and written by the kernel itself (no staging copies)
    BatchArgs A{};
    A.count = (int)count;
    A.a = C->ba.ensure(total);
    A.u = C->bu.ensure(total);
    A.f = nullptr;
    if (f) A.f = C->bf.ensure(f_shared ? (size_t)sides[0] * sides[0] : (size_t)total);
    A.f_shared = f_shared;
    A.fscalar = fscalar;
    A.u0 = u0 ? C->bu0.ensure(total) : nullptr;
    A.order = C->border.ensure(count);
    A.side = C->bside.ensure(count);
    A.off = C->boff.ensure(count);
    A.iterations = C->biter.ensure(count);
    A.residual = C->bres.ensure(count);
    A.converged = C->bconv.ensure(count);
    A.levels = C->blev.ensure(count);
    A.true_residual = out.true_residual ? C->btrue.ensure(count) : nullptr;
    A.bad = C->bbad.ensure(count);
    A.work = C->bwork.ensure(2);
    A.history = (o->record_history && count == 1) ? C->bhist.ensure((size_t)o->max_iter + 1) : nullptr;
    A.record_history = o->record_history;
    A.tol = o->tol;
    A.max_iter = o->max_iter;
    A.pc = o->preconditioner;
    A.pre = o->pre_sweeps;
    A.post = o->post_sweeps;
    A.gamma = o->cycle_index;

    // Pipelined host copies for a large batch whose launch shape is already
    // tuned: the problems are split into a few chunks; chunk k + 1 is copied
    // in (copy stream) while chunk k runs, and each chunk's solutions are
    // copied out while the later chunks run. The first and last chunks are
    // half the size of the others: their copy in and out are the two that no
    // compute hides.
    const auto tuned_hit = C->tuned.find(tune_key(C, maxside, mixed, o, count));
    const int64_t resident = 2 * (int64_t)C->sms;
    const bool pipelined = !device_ptrs && !warm && tuned_hit != C->tuned.end() &&
                           count >= 4 * resident && !(o->record_history);
    std::vector<int64_t> cut{0, count};
    if (pipelined) {
        // nchunks - 1 full chunks and two half chunks: cuts at (2k - 1) / (2 nchunks - 2)
        const int64_t nchunks = std::min<int64_t>(4, count / (2 * resident));
        const int64_t halves = 2 * nchunks - 2;
        cut.assign(1, 0);
        for (int64_t k = 1; k < nchunks; ++k) cut.push_back(count * (2 * k - 1) / halves);
        cut.push_back(count);
        // largest first within each chunk
        for (size_t k = 0; k + 1 < cut.size(); ++k) {
            std::iota(order.begin() + cut[k], order.begin() + cut[k + 1], (int)cut[k]);
            std::stable_sort(order.begin() + cut[k], order.begin() + cut[k + 1],
                             [&](int x, int y) { return sides[x] > sides[y]; });
        }
    }
    auto cells_of = [&](int64_t p0, int64_t p1) -> std::pair<int64_t, int64_t> {
        const int64_t lo = off[p0];
        const int64_t hi = off[p1 - 1] + (int64_t)sides[p1 - 1] * sides[p1 - 1];
        return {lo, hi - lo};
    };
    if (!pipelined) {
        CK(cudaMemcpyAsync((void*)A.a, a, sizeof(double) * total, in, s));
        if (f)
            CK(cudaMemcpyAsync((void*)A.f, f,
                               sizeof(double) * (f_shared ? (size_t)sides[0] * sides[0] : (size_t)total), in, s));
        if (u0) CK(cudaMemcpyAsync((void*)A.u0, u0, sizeof(double) * total, in, s));
    }
    if (warm) {  // warm start computed on the device from the resident permeability
        double* d_u0 = C->bu0.ensure(total);
        (*warm)(A.a, d_u0, s);
        A.u0 = d_u0;
        A.u0_fallback = 1;
    }
    CK(cudaMemcpyAsync((void*)A.order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)A.side, sides.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)A.off, off.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, s));

    // launch with a given shape over `n_prob` entries of `order` from `first`
    // (slot 1: the second compute stream, its own arenas and work counter)
    auto launch = [&](const BlockConfig& cfg, int64_t n_prob, int64_t first = 0, int slot = 0) {
        const int per_sm = mixed ? block_solve_occupancy<float>(cfg.threads, cfg.smem)
                                 : block_solve_occupancy<double>(cfg.threads, cfg.smem);
        const int ctas = (int)std::min<int64_t>(n_prob, (int64_t)C->sms * std::max(per_sm, 1));
        const size_t stride = align_up(block_arena_bytes(maxside, mixed, cfg.smem));
        cudaStream_t ls = slot ? C->stream2 : s;
        BatchArgs B = A;
        B.count = (int)n_prob;
        B.order = A.order + first;
        B.scratch = (slot ? C->bscratch2 : C->bscratch).ensure(stride * ctas);
        B.scratch_stride = stride;
        B.smem_budget = cfg.smem;
        B.work = A.work + slot;
        CK(cudaMemsetAsync(B.work, 0, sizeof(unsigned), ls));
        if (mixed)
            launch_block_solve<float>(B, ctas, cfg.threads, ls);
        else
            launch_block_solve<double>(B, ctas, cfg.threads, ls);
        CK(cudaGetLastError());
    };

    const std::string key = tune_key(C, maxside, mixed, o, count);
    // Untuned default, and the autotuner's first candidate: 256 threads for
    // small problems (4 CTAs per SM); 1024 when the batch holds problems of
    // side >= 256, whose single-CTA solves dominate a launch (16384 x 128^2 +
    // 64 x 512^2: 1.34 / 1.67 s mixed / FP64 with 1024 threads, 2.28 / 2.54 s
    // with 256).
    BlockConfig cfg;
    if (maxside >= 256) {
        cfg.threads = 1024;
        cfg.smem = 96 * 1024;
    } else {
        cfg.threads = 256;
        cfg.smem = smem_budget_for(mixed);
    }
    auto hit = C->tuned.find(key);
    if (hit != C->tuned.end()) {
        cfg.threads = hit->second.threads;
        cfg.smem = hit->second.smem;
    } else if (count >= C->sms) {
        // time every candidate on the batch's largest problems, 8 per SM: a
        // sample of 2 per SM hid what 4 CTAs of 256 threads gain on a full
        // batch (4096 x 64^2: 512 threads chosen at 174.5K solves/s mixed,
        // 88.6K FP64, against 180.9K and 96.4K with 256). Which shape wins
        // also depends on how the count divides into waves of resident
        // problems, so no sample is exact (the full-batch check below);
        // timing every candidate on the whole batch chose worse shapes for
        // the uneven sides 32..256 (19.8K against 21.2K solves/s mixed) and
        // cost 8 s.
        const int64_t sample = std::min<int64_t>(count, 8 * (int64_t)C->sms);
        float best = 1e30f;
        // (1024 threads: one problem per SM, half the resident arenas of 2 x 512,
        // for when the arenas of all resident problems outgrow the L2)
        std::vector<BlockConfig> cands{cfg};
        auto add = [&](int threads, size_t smem) {
            for (const BlockConfig& c : cands)
                if (c.threads == threads && c.smem == smem) return;
            cands.push_back(BlockConfig{threads, smem});
        };
        for (int threads : {128, 256, 512, 1024}) {
            add(threads, 0);
            add(threads, smem_budget_for(mixed));
            // 48 KiB for both forms (the FP64 form's own 96 KiB leaves 2 CTAs
            // per SM): 4096 uneven sides 32..256 FP64, 512 threads, 14.2K
            // solves/s against 13.6K with 96 KiB
            if (threads <= 512) add(threads, 48 * 1024);
            if (threads == 1024) add(threads, 96 * 1024);
            if (mixed && threads >= 512) add(threads, kSmemBudgetLarge);
            if (mixed && threads >= 256 && threads <= 512) add(threads, kSmemBudgetLevel0);
        }
        // odd warp counts between the powers of two: 5-6 CTAs of 192 threads or
        // 2-3 of 384 per SM, with a smaller coarse-level budget so that they fit
        for (int threads : {192, 256, 384}) add(threads, 32 * 1024);
        for (int threads : {192, 384}) add(threads, smem_budget_for(mixed));
        // Time budget: each candidate costs three launches over the sample,
        // and a launch lasts as long as its largest problem's single-CTA solve
        // (over a second for 512^2). When the default's launch exceeds
        // kTuneLaunchMs, tuning would cost more than it can save: keep the
        // default.
        constexpr float kTuneLaunchMs = 150.f;
        auto time_on = [&](const BlockConfig& c, int64_t n_prob) {
            launch(c, n_prob);  // warm (allocations, clocks)
            float ms = 1e30f;
            for (int rep = 0; rep < 2; ++rep) {  // best of two: one timing let noise pick the shape
                CK(cudaEventRecord(C->ev0, s));
                launch(c, n_prob);
                CK(cudaEventRecord(C->ev1, s));
                CK(cudaEventSynchronize(C->ev1));
                float t = 0.f;
                CK(cudaEventElapsedTime(&t, C->ev0, C->ev1));
                ms = std::min(ms, t);
            }
            return ms;
        };
        std::vector<std::pair<float, BlockConfig>> timed;
        for (size_t ci = 0; ci < cands.size(); ++ci) {
            const float ms = time_on(cands[ci], sample);
            timed.emplace_back(ms, cands[ci]);
            if (ms < best) {
                best = ms;
                cfg = cands[ci];
            }
            if (ci == 0 && ms > kTuneLaunchMs) break;
        }
        // The three fastest on the sample are timed again on the whole batch
        // when its launch is short (estimated from the sample at under
        // kFullCheckMs): 4096 x 64^2 FP64 then takes 256 threads and 48 KiB
        // (41.1 ms) over the sample's choice of 128 threads without a budget
        // (43.0 ms), which wins only on fewer problems.
        constexpr float kFullCheckMs = 80.f;
        if (count > sample && timed.size() > 1 && best * (float)count / (float)sample < kFullCheckMs) {
            std::sort(timed.begin(), timed.end(),
                      [](const auto& x, const auto& y) { return x.first < y.first; });
            float best_full = 1e30f;
            for (size_t k = 0; k < std::min<size_t>(3, timed.size()); ++k) {
                const float ms = time_on(timed[k].second, count);
                if (ms < best_full) {
                    best_full = ms;
                    cfg = timed[k].second;
                }
            }
        }
        C->tuned[key] = BlockConfigPOD{cfg.threads, cfg.smem};
        save_tuning(C);
    }
    C->last_block_threads = cfg.threads;
    C->last_block_smem = cfg.smem;

    CK(cudaEventRecord(C->ev0, s));
    if (pipelined) {
        const size_t nch = cut.size() - 1;
        while (C->chunk_events.size() < 2 * nch) {
            cudaEvent_t ev;
            CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            C->chunk_events.push_back(ev);
        }
        cudaStream_t cs = C->copy_stream;
        if (f && f_shared)
            CK(cudaMemcpyAsync((void*)A.f, f, sizeof(double) * (size_t)sides[0] * sides[0], in, cs));
        // chunks alternate between the two compute streams so that the next
        // chunk's CTAs fill the SMs the previous chunk's last wave leaves idle
        CK(cudaEventRecord(C->chunk_events[0], s));  // order after the uploads above
        CK(cudaStreamWaitEvent(C->stream2, C->chunk_events[0], 0));
        for (size_t k = 0; k < nch; ++k) {
            const auto [lo, len] = cells_of(cut[k], cut[k + 1]);
            const int slot = (int)(k & 1);
            cudaStream_t ks = slot ? C->stream2 : s;
            CK(cudaMemcpyAsync((void*)(A.a + lo), a + lo, sizeof(double) * len, in, cs));
            if (f && !f_shared) CK(cudaMemcpyAsync((void*)(A.f + lo), f + lo, sizeof(double) * len, in, cs));
            if (u0) CK(cudaMemcpyAsync((void*)(A.u0 + lo), u0 + lo, sizeof(double) * len, in, cs));
            CK(cudaEventRecord(C->chunk_events[2 * k], cs));
            CK(cudaStreamWaitEvent(ks, C->chunk_events[2 * k], 0));
            launch(cfg, cut[k + 1] - cut[k], cut[k], slot);
            CK(cudaEventRecord(C->chunk_events[2 * k + 1], ks));
        }
        for (size_t k = 0; k < nch; ++k) {
            const auto [lo, len] = cells_of(cut[k], cut[k + 1]);
            prefault_output(u_out + lo, len);  // while chunk k (or an earlier one) runs
            CK(cudaStreamWaitEvent(cs, C->chunk_events[2 * k + 1], 0));
            CK(cudaMemcpyAsync(u_out + lo, A.u + lo, sizeof(double) * len, outk, cs));
        }
        // the results below are read on the main stream after every chunk and copy
        CK(cudaEventRecord(C->chunk_events[2 * nch - 1], cs));
        CK(cudaStreamWaitEvent(s, C->chunk_events[2 * nch - 1], 0));
    } else {
        launch(cfg, count);
        if (!device_ptrs) prefault_output(u_out, total);
        CK(cudaMemcpyAsync(u_out, A.u, sizeof(double) * total, outk, s));
    }
    std::vector<unsigned long long> bad(count);
    CK(cudaMemcpyAsync(bad.data(), A.bad, sizeof(unsigned long long) * count, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(out.iterations, A.iterations, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(out.residuals, A.residual, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(out.converged, A.converged, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
    if (out.levels) CK(cudaMemcpyAsync(out.levels, A.levels, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
    if (out.true_residual)
        CK(cudaMemcpyAsync(out.true_residual, A.true_residual, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(C->ev1, s));
    CK(cudaStreamSynchronize(s));
    for (int64_t q = 0; q < count; ++q)
        if (bad[q] != ~0ull) bad_permeability(bad[q]);
    if (out.history && A.history && o->record_history) {
        const int len = out.iterations[0] + 1;
        CK(cudaMemcpy(out.history, A.history, sizeof(double) * len, cudaMemcpyDeviceToHost));
    }
    if (ms_out) CK(cudaEventElapsedTime(ms_out, C->ev0, C->ev1));
    C->last_launches = (int64_t)cut.size() - 1;
}

}  // namespace

// ======================================================================= C ABI

namespace {
__global__ void k_set_cond(cudaGraphConditionalHandle h, unsigned v) { cudaGraphSetConditional(h, v); }
__global__ void k_write(int* p, int v) { *p = v; }

// Self-test of device-set graph conditionals with an IF node (no loop, so a
// runtime that ignored the device call could not hang): the body must run
// exactly when the device set the condition to 1.
bool conditional_nodes_work(cudaStream_t s) {
    int* flag = nullptr;
    if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) return false;
    bool ok = true;
    for (unsigned v : {0u, 1u}) {
        cudaGraph_t G = nullptr;
        cudaGraphExec_t X = nullptr;
        int host = -1;
        bool step_ok = false;
        do {
            if (cudaGraphCreate(&G, 0) != cudaSuccess) break;
            cudaGraphConditionalHandle h;
            if (cudaGraphConditionalHandleCreate(&h, G, 0, cudaGraphCondAssignDefault) != cudaSuccess) break;
            cudaGraphNode_t nset, nif, nw;
            cudaKernelNodeParams kp{};
            void* args1[] = {&h, &v};
            kp.func = (void*)k_set_cond;
            kp.gridDim = dim3(1);
            kp.blockDim = dim3(1);
            kp.kernelParams = args1;
            if (cudaGraphAddKernelNode(&nset, G, nullptr, 0, &kp) != cudaSuccess) break;
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            if (cudaGraphAddNode(&nif, G, &nset, nullptr, 1, &cp) != cudaSuccess) break;
            int val = 7;
            void* args2[] = {&flag, &val};
            cudaKernelNodeParams kw{};
            kw.func = (void*)k_write;
            kw.gridDim = dim3(1);
            kw.blockDim = dim3(1);
            kw.kernelParams = args2;
            if (cudaGraphAddKernelNode(&nw, cp.conditional.phGraph_out[0], nullptr, 0, &kw) != cudaSuccess) break;
            if (cudaGraphInstantiate(&X, G, 0) != cudaSuccess) break;
            if (cudaMemsetAsync(flag, 0, sizeof(int), s) != cudaSuccess) break;
            if (cudaGraphLaunch(X, s) != cudaSuccess) break;
            if (cudaMemcpyAsync(&host, flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) break;
            if (cudaStreamSynchronize(s) != cudaSuccess) break;
            step_ok = (v == 1) ? host == 7 : host == 0;
        } while (0);
        if (X) cudaGraphExecDestroy(X);
        if (G) cudaGraphDestroy(G);
        ok = ok && step_ok;
    }
    cudaFree(flag);
    cudaGetLastError();
    return ok;
}

int run(const std::function<void()>& fn) {
    try {
        fn();
        g_err.clear();
        return DGPU_OK;
    } catch (const Failure& e) {
        g_err = e.msg;
        return e.code;
    } catch (const std::exception& e) {
        g_err = e.what();
        return DGPU_CUDA_ERROR;
    }
}

std::vector<int64_t> offsets_of(const std::vector<int>& sides) {
    std::vector<int64_t> off(sides.size());
    int64_t acc = 0;
    for (size_t q = 0; q < sides.size(); ++q) {
        off[q] = acc;
        acc += (int64_t)sides[q] * sides[q];
    }
    return off;
}

void solve_any(dgpu_context* C, const double* a, const double* f, double fscalar, int64_t n, const dgpu_options* o,
               const double* u0, double* u_out, double* history_out, dgpu_stats* stats, bool device_ptrs,
               cudaStream_t user_stream) {
    check_options(n, o);
    if (!a || !u_out) invalid("a and u must not be NULL");
    std::lock_guard<std::mutex> lock(C->mu);
    CK(cudaSetDevice(C->device));
    grid_solve(C, a, f, fscalar, n, o, u0, u_out, history_out, stats, device_ptrs, user_stream);
}

// z = M r through the grid engine's own preconditioner graph (setup, the
// large-level kernels and the dense tail): the apply_preconditioner hook
// therefore checks the exact code path the solves use.
void grid_precondition(dgpu_context* C, const double* a, const double* r, int64_t n, int pre, int post, int cycle,
                       int form, double* z) {
    PlanKey K{(int)n, form, kPcMultigrid, pre, post, cycle, 0, 0};
    GridPlan& P = get_plan(C, K);
    cudaStream_t s = C->stream;
    if (!P.ex_pc) {
        cudaGraph_t g = capture(s, [&] {
            emit_setup(P, s);
            if (P.mixed_mg) launch_copy_cast<float>(P.r, P.b0f, P.m, s);
            emit_precondition(P, s);
            if (P.mixed_mg) launch_copy_back<float>(P.x0f, P.z, P.m, s);
        });
        CK(cudaGraphInstantiate(&P.ex_pc, g, 0));
        cudaGraphDestroy(g);
    }
    CgState& hs = *P.st_host.p;
    std::memset(&hs, 0, sizeof hs);
    hs.bad = ~0ull;
    hs.max_iter = 1;
    const size_t bytes = sizeof(double) * (size_t)P.m;
    CK(cudaMemcpyAsync(P.a, a, bytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(P.r, r, bytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(P.st, &hs, sizeof hs, cudaMemcpyHostToDevice, s));
    CK(cudaGraphLaunch(P.ex_pc, s));
    CK(cudaMemcpyAsync(z, P.z, bytes, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&hs, P.st, sizeof hs, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (hs.bad != ~0ull) bad_permeability(hs.bad);
}

}  // namespace

void dgpu::set_last_error(const char* msg) { g_err = msg ? msg : ""; }

extern "C" {

const char* dgpu_last_error(void) { return g_err.c_str(); }

int dgpu_create(int device, dgpu_context** out) {
    return run([&] {
        if (!out) invalid("out must not be NULL");
        auto C = std::make_unique<dgpu_context>();
        if (device < 0) CK(cudaGetDevice(&device));
        C->device = device;
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&C->stream, cudaStreamNonBlocking));
        CK(cudaEventCreate(&C->ev0));
        CK(cudaEventCreate(&C->ev1));
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, device));
        C->sms = prop.multiProcessorCount;
        C->device_name = prop.name;
        // DARCY_GPU_LOOP=host selects the host-chunked CG loop (graphs
        // without conditional nodes, e.g. for per-kernel profiling).
        const char* loop = std::getenv("DARCY_GPU_LOOP");
        C->cond_ok = !(loop && std::strcmp(loop, "host") == 0) && conditional_nodes_work(C->stream);
        const char* pdl = std::getenv("DARCY_GPU_PDL");
        set_programmatic_launch(!(pdl && std::strcmp(pdl, "0") == 0));
        CK(cudaStreamCreateWithFlags(&C->copy_stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&C->stream2, cudaStreamNonBlocking));
        char buf[512];
        std::snprintf(buf, sizeof buf,
                      "%s | %d SMs | sm_%d%d | %.1f GiB | L2 %.1f MiB | graph while-loop: %s | programmatic launch: %s",
                      prop.name, prop.multiProcessorCount, prop.major, prop.minor,
                      prop.totalGlobalMem / 1073741824.0, prop.l2CacheSize / 1048576.0,
                      C->cond_ok ? "device-side" : "host-chunked", programmatic_launch() ? "on" : "off");
        C->info = buf;
        *out = C.release();
    });
}

void dgpu_destroy(dgpu_context* ctx) {
    if (!ctx) return;
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        cudaSetDevice(ctx->device);
        ctx->plans.clear();
        if (ctx->ev0) cudaEventDestroy(ctx->ev0);
        if (ctx->ev1) cudaEventDestroy(ctx->ev1);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
        if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
        for (cudaEvent_t ev : ctx->chunk_events) cudaEventDestroy(ev);
        ctx->slot_plans.clear();
        for (cudaStream_t st : ctx->slot_streams) cudaStreamDestroy(st);
        for (cudaEvent_t ev : ctx->slot_events) cudaEventDestroy(ev);
    }
    delete ctx;
}

int dgpu_device_info(dgpu_context* ctx, char* out, int capacity) {
    return run([&] {
        if (!ctx || !out || capacity < 1) invalid("bad arguments");
        std::snprintf(out, (size_t)capacity, "%s", ctx->info.c_str());
    });
}

int dgpu_num_levels(int64_t n) { return n < 1 ? 0 : num_levels_for((int)std::min<int64_t>(n, 1 << 30)); }

int dgpu_solve(dgpu_context* ctx, const double* a, const double* f, double f_scalar, int64_t n,
               const dgpu_options* opt, const double* u0, double* u_out, double* history_out, dgpu_stats* stats) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        solve_any(ctx, a, f, f_scalar, n, opt, u0, u_out, history_out, stats, false, nullptr);
    });
}

int dgpu_solve_device(dgpu_context* ctx, const double* d_a, const double* d_f, double f_scalar, int64_t n,
                      const dgpu_options* opt, const double* d_u0, double* d_u, dgpu_stats* stats, void* stream) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        if (opt && opt->record_history) invalid("record_history is not supported on device buffers");
        solve_any(ctx, d_a, d_f, f_scalar, n, opt, d_u0, d_u, nullptr, stats, true, (cudaStream_t)stream);
    });
}

int dgpu_solve_batch(dgpu_context* ctx, const double* a, const double* f, double f_scalar, int f_per_sample,
                     int64_t batch, int64_t n, const dgpu_options* opt, const double* u0, double* u_out,
                     int* iterations, double* residuals, int* converged, int* levels) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        check_options(n, opt);
        if (batch < 1) invalid("a must have shape (batch, n, n)");
        if (!a || !u_out || !iterations || !residuals || !converged) invalid("buffers must not be NULL");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        std::vector<int> sides((size_t)batch, (int)n);
        dgpu_options o = *opt;
        o.record_history = 0;
        if (route_to_grid(ctx, n, batch * n * n)) {  // large problems: concurrent grid-engine solves
            std::vector<int64_t> order((size_t)batch);
            std::iota(order.begin(), order.end(), (int64_t)0);
            grid_solve_many(ctx, (int)n, order, offsets_of(sides), a, f, !f_per_sample, f_scalar, &o, u0, u_out,
                            iterations, residuals, converged, levels, false);
            return;
        }
        BatchOut bo{iterations, residuals, converged, levels, nullptr, nullptr};
        block_solve(ctx, batch, sides, offsets_of(sides), a, f, f_per_sample ? 0 : 1, f_scalar, u0, &o, u_out, bo,
                    false, nullptr);
    });
}

int dgpu_solve_batch_device(dgpu_context* ctx, const double* d_a, const double* d_f, double f_scalar,
                            int f_per_sample, int64_t batch, int64_t n, const dgpu_options* opt, const double* d_u0,
                            double* d_u, int* iterations, double* residuals, int* converged, int* levels,
                            double* device_ms, void* stream) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        check_options(n, opt);
        if (batch < 1) invalid("a must have shape (batch, n, n)");
        if (!d_a || !d_u || !iterations || !residuals || !converged) invalid("buffers must not be NULL");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        cudaStream_t user = (cudaStream_t)stream;
        if (user) {  // order after the caller's stream
            CK(cudaEventRecord(ctx->ev0, user));
            CK(cudaStreamWaitEvent(ctx->stream, ctx->ev0, 0));
        }
        std::vector<int> sides((size_t)batch, (int)n);
        dgpu_options o = *opt;
        o.record_history = 0;
        if (route_to_grid(ctx, n, batch * n * n)) {
            std::vector<int64_t> order((size_t)batch);
            std::iota(order.begin(), order.end(), (int64_t)0);
            const float ms = grid_solve_many(ctx, (int)n, order, offsets_of(sides), d_a, d_f, !f_per_sample, f_scalar,
                                             &o, d_u0, d_u, iterations, residuals, converged, levels, true);
            if (device_ms) *device_ms = ms;
            return;
        }
        BatchOut bo{iterations, residuals, converged, levels, nullptr, nullptr};
        float ms = 0.f;
        block_solve(ctx, batch, sides, offsets_of(sides), d_a, d_f, f_per_sample ? 0 : 1, f_scalar, d_u0, &o, d_u, bo,
                    true, &ms);
        if (device_ms) *device_ms = ms;
        // block_solve synchronised the context stream: the caller's stream may continue
    });
}

int64_t dgpu_last_launches(const dgpu_context* ctx) { return ctx ? ctx->last_launches : 0; }

int dgpu_solve_uneven(dgpu_context* ctx, int64_t count, const int64_t* sides, const double* a, const double* f,
                      double f_scalar, const dgpu_options* opt, const double* u0, double* u_out, int* iterations,
                      double* residuals, int* converged, int* levels) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        if (count < 1 || !sides) invalid("need at least one problem");
        std::vector<int> sv((size_t)count);
        for (int64_t q = 0; q < count; ++q) {
            check_options(sides[q], opt);
            sv[q] = (int)sides[q];
        }
        if (!a || !u_out || !iterations || !residuals || !converged) invalid("buffers must not be NULL");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        dgpu_options o = *opt;
        o.record_history = 0;
        // Problems that one CTA would take longer on than the whole rest of
        // the batch go to the grid engine (route_to_grid), after the block
        // engine has taken the rest.
        const std::vector<int64_t> off = offsets_of(sv);
        std::vector<int64_t> small, big;
        int64_t total = 0;
        for (int v : sv) total += (int64_t)v * v;
        for (int64_t q = 0; q < count; ++q) (route_to_grid(ctx, sv[q], total) ? big : small).push_back(q);
        if (big.empty()) {
            BatchOut bo{iterations, residuals, converged, levels, nullptr, nullptr};
            block_solve(ctx, count, sv, off, a, f, 0, f_scalar, u0, &o, u_out, bo, false, nullptr);
            return;
        }
        if (!small.empty()) {
            const size_t ns = small.size();
            std::vector<int> ss(ns), it(ns), cv(ns), lv(ns);
            std::vector<int64_t> so(ns);
            std::vector<double> rs(ns);
            for (size_t k = 0; k < ns; ++k) {
                ss[k] = sv[small[k]];
                so[k] = off[small[k]];
            }
            BatchOut bo{it.data(), rs.data(), cv.data(), lv.data(), nullptr, nullptr};
            block_solve(ctx, (int64_t)ns, ss, so, a, f, 0, f_scalar, u0, &o, u_out, bo, false, nullptr);
            for (size_t k = 0; k < ns; ++k) {
                iterations[small[k]] = it[k];
                residuals[small[k]] = rs[k];
                converged[small[k]] = cv[k];
                if (levels) levels[small[k]] = lv[k];
            }
        }
        // (the block engine's copy-out covers the cells up to its last
        // problem; the large problems' cells are written after it) -- large
        // problems of one side at a time, concurrently
        int64_t launched = small.empty() ? 0 : ctx->last_launches;
        std::map<int, std::vector<int64_t>> by_side;
        for (int64_t q : big) by_side[sv[q]].push_back(q);
        for (auto it = by_side.rbegin(); it != by_side.rend(); ++it) {
            grid_solve_many(ctx, it->first, it->second, off, a, f, false, f_scalar, &o, u0, u_out, iterations,
                            residuals, converged, levels, false);
            launched += ctx->last_launches;
        }
        ctx->last_launches = launched;
    });
}

int dgpu_solve_batch_learned(dgpu_context* ctx, dgpu_net* net, const double* a, double f_scalar, int64_t batch,
                             int64_t n, const dgpu_options* opt, double* u_out, int* iterations, double* residuals,
                             int* converged, int* levels) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        if (!net) invalid("network must not be NULL");
        check_options(n, opt);
        if (batch < 1) invalid("a must have shape (batch, n, n)");
        if (!a || !u_out || !iterations || !residuals || !converged) invalid("buffers must not be NULL");
        if (net_side(net) != n) invalid("the network was built for another grid side");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        std::vector<int> sides((size_t)batch, (int)n);
        dgpu_options o = *opt;
        o.record_history = 0;
        BatchOut bo{iterations, residuals, converged, levels, nullptr, nullptr};
        const std::function<void(const double*, double*, cudaStream_t)> warm =
            [&](const double* d_a, double* d_u0, cudaStream_t s) {
                std::string msg;
                const int rc = net_predict_on_stream(net, d_a, f_scalar, batch, d_u0, s, &msg);
                if (rc != DGPU_OK) throw Failure{rc, msg};
            };
        block_solve(ctx, batch, sides, offsets_of(sides), a, nullptr, 1, f_scalar, nullptr, &o, u_out, bo, false,
                    nullptr, &warm);
        ctx->last_launches += net_launches(net);
    });
}

int dgpu_apply_operator(dgpu_context* ctx, const double* a, const double* x, int64_t n, double* y) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        if (n < 1) invalid("a must be a square 2-D array with at least one cell");
        if (n > 46340) invalid("grid size too large for 32-bit cell rows");
        if (!a || !x || !y) invalid("buffers must not be NULL");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        cudaStream_t s = ctx->stream;
        const size_t m = (size_t)n * n;
        double *da, *dx, *dy;
        Lvl64 L{};
        unsigned long long* bad;
        auto layout = [&](Carver& c) {
            da = c.take<double>(m);
            dx = c.take<double>(m);
            dy = c.take<double>(m);
            L = Lvl64{(int)n, c.take<double>(m), c.take<double>(m), c.take<double>(m), c.take<double>(m),
                      c.take<double>((size_t)n), c.take<double>((size_t)n)};
            bad = c.take<unsigned long long>(1);
        };
        Carver probe;
        layout(probe);
        Carver real{ctx->misc.ensure(probe.off), probe.off, 0};
        layout(real);
        const unsigned long long init = ~0ull;
        CK(cudaMemcpyAsync(bad, &init, 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(da, a, 8 * m, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dx, x, 8 * m, cudaMemcpyHostToDevice, s));
        launch_build_fine(da, L, bad, s);
        launch_apply(L, dx, dy, s);
        CK(cudaGetLastError());
        unsigned long long hb = 0;
        CK(cudaMemcpyAsync(&hb, bad, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(y, dy, 8 * m, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (hb != ~0ull) bad_permeability(hb);
    });
}

int dgpu_apply_preconditioner(dgpu_context* ctx, const double* a, const double* r, int64_t n, int pre_sweeps,
                              int post_sweeps, int cycle_index, int form, double* z) {
    return run([&] {
        if (!ctx) invalid("context must not be NULL");
        if (n < 1) invalid("a must be a square 2-D array with at least one cell");
        if (!a || !r || !z) invalid("buffers must not be NULL");
        if (pre_sweeps < 1 || post_sweeps < 1) invalid("sweeps must be at least 1");  // bindings.cpp:235
        if (cycle_index < 1 || cycle_index > 2) invalid("cycle_index must be 1 or 2");  // bindings.cpp:236
        if (form != DGPU_FORM_FP64 && form != DGPU_FORM_MIXED) invalid("unknown form; expected fp64 or mixed");
        if (n > 46340) invalid("grid size too large for 32-bit cell rows");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        grid_precondition(ctx, a, r, n, pre_sweeps, post_sweeps, cycle_index, form, z);
    });
}

int64_t dgpu_hierarchy(dgpu_context* ctx, const double* a, int64_t n, double* out, int64_t capacity) {
    int64_t written = -1;
    int rc = run([&] {
        if (!ctx) invalid("context must not be NULL");
        if (n < 1 || n > 46340 || !a || !out) invalid("bad arguments");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        cudaStream_t s = ctx->stream;
        const std::vector<int> sides = level_sides((int)n);
        double* da;
        unsigned long long* bad;
        std::vector<Lvl64> h(sides.size());
        auto layout = [&](Carver& c) {
            da = c.take<double>((size_t)n * n);
            bad = c.take<unsigned long long>(1);
            for (size_t l = 0; l < sides.size(); ++l) {
                const size_t ml = (size_t)sides[l] * sides[l];
                h[l] = Lvl64{sides[l], c.take<double>(ml), c.take<double>(ml), c.take<double>(ml),
                             c.take<double>(ml), c.take<double>((size_t)sides[l]), c.take<double>((size_t)sides[l])};
            }
        };
        Carver probe;
        layout(probe);
        Carver real{ctx->misc.ensure(probe.off), probe.off, 0};
        layout(real);
        const unsigned long long init = ~0ull;
        CK(cudaMemcpyAsync(bad, &init, 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(da, a, 8 * (size_t)n * n, cudaMemcpyHostToDevice, s));
        launch_build_fine(da, h[0], bad, s);
        for (size_t l = 1; l < sides.size(); ++l) launch_coarsen(h[l - 1], h[l], s);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s));
        int64_t pos = 0;
        for (size_t l = 0; l < sides.size(); ++l) {
            const int sd = sides[l];
            const size_t ml = (size_t)sd * sd;
            if (pos + 6 * (int64_t)ml > capacity) invalid("capacity too small");
            std::vector<double> e(ml), nf(ml), d(ml), id(ml), wb(sd), sb(sd);
            CK(cudaMemcpy(e.data(), h[l].e, 8 * ml, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(nf.data(), h[l].nf, 8 * ml, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(d.data(), h[l].d, 8 * ml, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(id.data(), h[l].id, 8 * ml, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(wb.data(), h[l].wb, 8 * sd, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(sb.data(), h[l].sb, 8 * sd, cudaMemcpyDeviceToHost));
            double* E = out + pos;
            double* W = E + ml;
            double* N = W + ml;
            double* S = N + ml;
            double* D = S + ml;
            double* I = D + ml;
            for (int i = 0; i < sd; ++i)
                for (int j = 0; j < sd; ++j) {
                    const size_t k = (size_t)i * sd + j;
                    E[k] = e[k];
                    N[k] = nf[k];
                    W[k] = j > 0 ? e[k - 1] : wb[i];
                    S[k] = i > 0 ? nf[k - sd] : sb[j];
                    D[k] = d[k];
                    I[k] = id[k];
                }
            pos += 6 * (int64_t)ml;
        }
        unsigned long long hb = 0;
        CK(cudaMemcpy(&hb, bad, 8, cudaMemcpyDeviceToHost));
        if (hb != ~0ull) bad_permeability(hb);
        written = pos;
    });
    return rc == DGPU_OK ? written : -1;
}

int dgpu_profile_kernels(dgpu_context* ctx, const double* a, int64_t n, const dgpu_options* opt, int reps,
                         dgpu_kernel_time* out, int cap, int* count) {
    return run([&] {
        if (!ctx || !a || !out || !count || cap < 1 || reps < 1) invalid("bad arguments");
        check_options(n, opt);
        if (opt->preconditioner != kPcMultigrid) invalid("profiling needs the multigrid preconditioner");
        std::vector<double> u((size_t)(n * n));
        dgpu_stats st{};
        dgpu_options o = *opt;
        o.record_history = 0;
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        grid_solve(ctx, a, nullptr, 1.0, n, &o, nullptr, u.data(), nullptr, &st, false, nullptr);
        PlanKey K{(int)n, o.form, o.preconditioner, o.pre_sweeps, o.post_sweeps, o.cycle_index, 0, 0};
        GridPlan& P = get_plan(ctx, K);
        cudaStream_t s = ctx->stream;
        // A state that never stops: tol 0, no iteration cap, no graph handle.
        CgState& hs = *P.st_host.p;
        CK(cudaMemcpy(&hs, P.st, sizeof hs, cudaMemcpyDeviceToHost));
        hs.done = 0;
        hs.tol = 0.0;
        hs.max_iter = 1 << 30;
        hs.use_cond = 0;
        hs.record_history = 0;
        hs.it = 1;
        for (unsigned& t : hs.ticket) t = 0;
        const double m = (double)P.m;
        const bool f32 = P.mixed_mg;
        const double w = f32 ? 4.0 : 8.0;
        const int nc = (P.n + 1) / 2;
        const double mc = (double)nc * nc;
        int visits_tail = 1;  // tail products per iteration: parent visits = gamma^(tail_l0 - 1)
        for (int l = 1; l < P.tail_l0; ++l) visits_tail *= K.gamma;
        struct Item {
            std::string name;
            double bytes, per_it;
            std::function<void()> launch;
        };
        std::vector<Item> items;
        // Lambdas below capture plain pointers and level views only.
        CgState* const stp = P.st;
        double* const partials = P.partials;
        const double* const rvec = P.r;
        const int ntail = P.ntail;
        const int64_t mm = P.m;
        const int tail_l0 = P.tail_l0;
        auto add_level0 = [&](auto tag) {
            using T = decltype(tag);
            const Lvl<T> L0 = levels_of<T>(P)[0];
            if (tail_l0 == 0) return;
            const Lvl<T> L1 = levels_of<T>(P)[1];
            const T* Tm = tail_matrix<T>(P);
            // algorithmic bytes: every array the kernel must touch, once;
            // launches per iteration 1 for the kernels level 0 runs (fused
            // visits, or the unfused kernels from kUnfusedSide up), else 0
            const bool l0_unfused = !P.fused || P.lf > 0;
            const double on_f = l0_unfused ? 0.0 : 1.0, on_u = l0_unfused ? 1.0 : 0.0;
            if (P.fused) {
                const VisitLevel<T> V0 = visit_level<T>(P, 0);
                T* xa = (T*)P.X0[0];
                T* xb = (T*)P.X1[0];
                T* x1 = (T*)P.X0[1];
                const double cb = sizeof(T) == 4 ? 7 * 4.0 : 4 * 8.0;  // staged coefficient bytes per cell
                items.push_back({"visit_pre(l0)", cb * m + w * (2 * m + mc) + (sizeof(T) == 4 ? 4 * m : 0), on_f,
                                 [=] { launch_visit_pre<T>(V0, nullptr, xa, L1.b, s); }});
                items.push_back({"visit_post(l0)", 3 * w * m + w * (3 * m + mc) + 8 * m, on_f, [=] {
                                     launch_visit_post<T>(V0, xa, x1, xb, rvec, stp, partials, s);
                                 }});
            }
            items.push_back({"gs_colour0_zero(l0)", w * m * 1.5, on_u, [=] { launch_gs<T>(L0, 0, true, stp, s); }});
            items.push_back({"gs_colour1(l0)", w * (m * 0.5 * 3 + m * 2 + m), on_u,
                             [=] { launch_gs<T>(L0, 1, false, stp, s); }});
            if constexpr (sizeof(T) == 4) {  // double-float: e, nf, d and their lo parts, x, b, b_lo
                const float *elo = P.elo[0], *nlo = P.nlo[0], *dlo = P.dlo[0], *blo = P.b0lo;
                items.push_back({"residual_restrict(l0)", w * (8 * m + mc) + 4 * m, on_u, [=] {
                                     launch_residual_restrict_df(L0, elo, nlo, dlo, blo, L1.b, stp, s);
                                 }});
            } else {
                items.push_back({"residual_restrict(l0)", w * (5 * m + mc), on_u,
                                 [=] { launch_residual_restrict<T>(L0, L1.b, stp, s); }});
            }
            items.push_back({"prolong_gs1(l0)", w * (m * 0.5 * 3 + m * 2 + m + mc), on_u,
                             [=] { launch_prolong_gs1<T>(L0, L1.x, stp, s); }});
            items.push_back({"gs0_dot(l0)", w * (m * 0.5 * 3 + m * 2 + m) + 8 * m, on_u,
                             [=] { launch_gs0_dot<T>(L0, rvec, stp, partials, s); }});
            const double nt = (double)ntail;
            items.push_back({"tail_matvec", w * (nt * nt + 2 * nt), (double)visits_tail,
                             [=] { launch_tail_matvec<T>(Tm, ntail, L1.b, L1.x, stp, s); }});
        };
        // The fused visits of the coarse levels (side < the unfused-kernel
        // side, above the dense tail), by kind and level, with their launches
        // per preconditioner application: the fused program from level lf runs
        // once per visit of level lf - 1, i.e. gamma^(lf - 1) times per cycle.
        auto add_coarse = [&](auto tag) {
            using T = decltype(tag);
            if (!P.fused || P.tail_l0 <= 1) return;
            const auto& lv = levels_of<T>(P);
            const int lf = P.lf;
            int reps_top = 1;
            for (int l = 1; l < lf; ++l) reps_top *= K.gamma;
            const std::vector<VisitOp> prog = lf == 0 ? visit_program(P, 0, 1) : visit_program(P, lf, K.gamma);
            // (kind, level, first) -> launches per cycle
            std::map<std::tuple<int, int, bool>, int> counts;
            for (const VisitOp& op : prog)
                if (op.kind != kOpTail && op.l >= 1) counts[{op.kind, op.l, op.kind == kOpPre && op.first}] += reps_top;
            const double cb = sizeof(T) == 4 ? 7 * 4.0 : 4 * 8.0;  // staged coefficient bytes per cell
            for (const auto& kv : counts) {
                const int kind = std::get<0>(kv.first), l = std::get<1>(kv.first);
                const bool first = std::get<2>(kv.first);
                const VisitLevel<T> V = visit_level<T>(P, l);
                T* x0 = (T*)P.X0[l];
                T* x1 = (T*)P.X1[l];
                T* xc = (T*)P.X0[l + 1];
                T* bc = lv[l + 1].b;
                const double ml = (double)V.n * V.n;
                const int ncl = (V.n + 1) / 2;
                const double mcl = (double)ncl * ncl;
                char nm[48];
                if (kind == kOpPre) {
                    std::snprintf(nm, sizeof nm, "visit_pre%s(l%d)", first ? "_zero" : "", l);
                    items.push_back({nm, cb * ml + w * ((first ? 2 : 3) * ml + mcl),
                                     (double)kv.second, [=] { launch_visit_pre<T>(V, first ? nullptr : x0, x1, bc, s); }});
                } else if (kind == kOpMid) {
                    std::snprintf(nm, sizeof nm, "visit_mid(l%d)", l);
                    items.push_back({nm, cb * ml + w * (3 * ml + 2 * mcl), (double)kv.second,
                                     [=] { launch_visit_mid<T>(V, x0, xc, x1, bc, s); }});
                } else {
                    std::snprintf(nm, sizeof nm, "visit_post(l%d)", l);
                    items.push_back({nm, 3 * w * ml + w * (3 * ml + mcl), (double)kv.second,
                                     [=] { launch_visit_post<T>(V, x0, xc, x1, nullptr, stp, partials, s); }});
                }
            }
        };
        if (f32) {
            add_level0(float{});
            add_coarse(float{});
        } else {
            add_level0(double{});
            add_coarse(double{});
        }
        const Lvl64 H0 = P.h[0];
        double* const pv = P.p;
        double* const apv = P.ap;
        double* const uv = P.u;
        double* const rw = P.r;
        float* const x0f = P.x0f;
        float* const b0f = P.b0f;
        float* const b0lo = P.b0lo;
        const double* const zv = P.z;
        if (f32)
            items.push_back({"xpby", (4 + 16) * m, 1.0, [=] { launch_xpby<float>(x0f, pv, mm, stp, s); }});
        else
            items.push_back({"xpby", 24 * m, 1.0, [=] { launch_xpby<double>(zv, pv, mm, stp, s); }});
        items.push_back({"apply_dot", 40 * m, 1.0, [=] { launch_apply_dot(H0, pv, apv, stp, partials, s); }});
        items.push_back({"cg_update", (48 + (f32 ? 8 : 0)) * m, 1.0, [=] {
                             launch_cg_update(pv, apv, uv, rw, f32 ? b0f : nullptr, b0lo, nullptr, mm, stp, partials,
                                              s);
                         }});
        // DARCY_GPU_PROFILE_DIRECT=1 launches each kernel straight on the
        // stream instead of from a graph, for a kernel profiler (which does
        // not replay graph nodes of kernels that can end the CG loop).
        const char* de = std::getenv("DARCY_GPU_PROFILE_DIRECT");
        const bool direct = de && std::strcmp(de, "1") == 0;
        int q = 0;
        for (const Item& it : items) {
            if (q >= cap) break;
            CK(cudaMemcpyAsync(P.st, &hs, sizeof hs, cudaMemcpyHostToDevice, s));
            cudaGraphExec_t x = nullptr;
            if (!direct) {
                cudaGraph_t g = capture(s, [&] {
                    for (int r = 0; r < reps; ++r) it.launch();
                });
                CK(cudaGraphInstantiate(&x, g, 0));
                cudaGraphDestroy(g);
            }
            auto run_all = [&] {
                if (x)
                    CK(cudaGraphLaunch(x, s));
                else
                    for (int r = 0; r < reps; ++r) it.launch();
            };
            run_all();  // warm
            CK(cudaMemcpyAsync(P.st, &hs, sizeof hs, cudaMemcpyHostToDevice, s));
            CK(cudaEventRecord(ctx->ev0, s));
            run_all();
            CK(cudaEventRecord(ctx->ev1, s));
            CK(cudaStreamSynchronize(s));
            if (x) cudaGraphExecDestroy(x);
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
            std::snprintf(out[q].name, sizeof out[q].name, "%s", it.name.c_str());
            out[q].avg_ms = ms / reps;
            out[q].bytes = it.bytes;
            out[q].launches_per_iteration = it.per_it;
            ++q;
        }
        *count = q;
    });
}

int dgpu_flush_l2(dgpu_context* ctx, int64_t bytes) {
    return run([&] {
        if (!ctx || bytes < 1) invalid("bad arguments");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        char* p = ctx->flush.ensure((size_t)bytes);
        CK(cudaMemsetAsync(p, 1, (size_t)bytes, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    });
}

int64_t dgpu_check_conversions(dgpu_context* ctx, const double* x, int64_t count, float* hi, float* lo,
                               float* rounded, double* widened) {
    int64_t mism = -1;
    const int rc = run([&] {
        if (!ctx || !x || count < 1 || !hi || !lo || !rounded || !widened) invalid("bad arguments");
        std::lock_guard<std::mutex> lock(ctx->mu);
        CK(cudaSetDevice(ctx->device));
        const size_t m = (size_t)count;
        // x, widened (8 B each), the mismatch counter, then hi, lo, rounded (4 B each)
        char* base = ctx->misc.ensure(m * (8 + 8 + 4 + 4 + 4) + 8);
        double* dx = (double*)base;
        double* dw = dx + m;
        unsigned long long* dm = (unsigned long long*)(dw + m);
        float* dh = (float*)(dm + 1);
        float* dl = dh + m;
        float* dr = dl + m;
        cudaStream_t s = ctx->stream;
        CK(cudaMemcpyAsync(dx, x, m * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(dm, 0, sizeof(unsigned long long), s));
        launch_check_conversions(dx, (int64_t)m, dh, dl, dr, dw, dm, s);
        CK(cudaGetLastError());
        unsigned long long hm = 0;
        CK(cudaMemcpyAsync(hi, dh, m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(lo, dl, m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(rounded, dr, m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(widened, dw, m * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(&hm, dm, sizeof hm, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        mism = (int64_t)hm;
    });
    return rc == DGPU_OK ? mism : -1;
}

}  // extern "C"
