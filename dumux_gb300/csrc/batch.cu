// batch.cu -- batched and served forms: many independent problems advanced together.
//
// The single-problem path (api.cu) leaves most of the GPU idle on small and medium
// grids: the ILU(0) sweeps are a wavefront whose critical path is one dependent block
// update per level, so one problem occupies one cluster of at most 16 SMs and spends
// its time waiting on latency.  The engine here advances all active problems by one
// tick per call: problems that begin a Newton iteration are assembled and factorised,
// every problem runs a chunk of BiCGSTAB iterations, and problems whose solve ended
// take their update.  Each kernel (volume variables, Jacobian rows, FP64->FP32 copy,
// ILU(0) factor and sweeps, SpMV, BiCGSTAB vector updates, Newton update) is launched
// once for all problems of a kind, each problem reading its own argument block
// (blockIdx.y, or the cluster index in the sweeps).  Every problem keeps its own
// reduction scratch and Krylov scalars, and a problem reduces over the same block
// count as when it runs alone, so its arithmetic -- and its result -- is the same
// alone and in any mix.  Problems whose solve has ended skip inside the chunk, so a
// slow problem costs the others nothing but its own sweeps.
//
// Control stays per problem on the host: after each chunk one gathered status record
// per problem (Krylov status, shift, flags) is read back, and each problem follows
// the reference's Newton / time-loop logic (NewtonSolver::solve_ and solveImpl_,
// dumux/nonlinear/newtonsolver.hh:309-382, 917-1072; newtonProceed / newtonConverged
// :428-446, 657-701; suggestTimeStepSize :784-798; TimeLoop::setTimeStepSize capped by
// the maximum, common/timeloop.hh:323).
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "context.h"

using namespace dxg;

namespace {

// ---------------------------------------------------------------- small batched kernels
struct SlotReport {
    double def0, def, shift, norm;
    int status, halfsteps, singular, timeout;
};
struct GatherArgs {
    const KrylovState* ks;
    const double* scal;   // [0] shift, [1] norm
    int* flags;           // [0] singular pivot, [1] sweep wait timeout
};

__global__ void gatherKernel(const GatherArgs* __restrict__ g, SlotReport* __restrict__ out, int count)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    const GatherArgs a = g[p];
    SlotReport r;
    r.def0 = a.ks->def0;
    r.def = a.ks->def;
    r.status = a.ks->status;
    r.halfsteps = a.ks->halfsteps;
    r.shift = a.scal[0];
    r.norm = a.scal[1];
    r.singular = a.flags[0];
    r.timeout = a.flags[1];
    out[p] = r;
}
__global__ void clearFlagsKernel(const GatherArgs* __restrict__ g, int count)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    g[p].flags[0] = 0;
    g[p].flags[1] = 0;
}

// y = x (x != nullptr) or y = 0, one problem per blockIdx.y
struct CopyArgs {
    double* y;
    const double* x;
    int64_t n;
};
__global__ void copyKernel(const CopyArgs* __restrict__ batch)
{
    const CopyArgs a = batch[blockIdx.y];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x)
        a.y[k] = a.x ? a.x[k] : 0.0;
}

// ---------------------------------------------------------------- argument arena
// Argument blocks are staged in pinned host memory and copied to device memory in
// the stream order of the launches that read them.  Space is handed out append-only
// during one iteration and recycled at the start of the next (after its final sync).
struct Arena {
    struct Block {
        unsigned char* host = nullptr;
        unsigned char* dev = nullptr;
        size_t cap = 0, used = 0;
    };
    std::vector<Block> blocks;
    size_t cur = 0;

    void reset()
    {
        for (auto& b : blocks) b.used = 0;
        cur = 0;
    }
    template <class T>
    T* put(const std::vector<T>& v, cudaStream_t st)
    {
        const size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
        const size_t need = (bytes + 255) & ~(size_t)255;
        while (cur < blocks.size() && blocks[cur].used + need > blocks[cur].cap) ++cur;
        if (cur == blocks.size()) {
            Block b;
            b.cap = std::max<size_t>(need, 4u << 20);
            DXG_CUDA(cudaMallocHost(&b.host, b.cap));
            if (cudaMalloc(&b.dev, b.cap) != cudaSuccess) {
                cudaGetLastError();
                cudaFreeHost(b.host);
                throw Error(DXG_ERR_OOM, "argument arena allocation failed");
            }
            blocks.push_back(b);
        }
        Block& b = blocks[cur];
        unsigned char* h = b.host + b.used;
        unsigned char* d = b.dev + b.used;
        if (!v.empty()) std::memcpy(h, v.data(), v.size() * sizeof(T));
        DXG_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st));
        b.used += need;
        return reinterpret_cast<T*>(d);
    }
    ~Arena()
    {
        for (auto& b : blocks) {
            cudaFreeHost(b.host);
            cudaFree(b.dev);
        }
    }
};

enum { SLOT_ACTIVE = 0, SLOT_DONE = 1, SLOT_FAILED = 2 };

// problems sharing kernels: num_eq, dim, difference method, gravity, transient, upwind
using GroupKey = std::tuple<int, int, int, int, int, int>;
struct GroupState;

struct Slot {
    int64_t id = 0;
    dxg_ctx* c = nullptr;
    dxg_newton_params p{};
    int64_t bytes = 0;
    // time loop
    bool transient = false;
    double t = 0.0, tEnd = 0.0, dtMax = 0.0, dt = 0.0;
    int steps = 0;
    // Newton state of the current attempt
    int numSteps = 0, divisions = 0;
    double shift = 0.0, lastShift = 0.0;
    double reduction = 0.0, lastReduction = 1.0, initialResidual = 0.0;
    // linear solve of the current iteration
    bool solving = false, linConv = false;
    int chunks = 0, linIters = 0;
    int linStatus = DXG_OK;
    // outcome
    int state = SLOT_ACTIVE;
    int status = DXG_OK;
    int totalDivisions = 0;
    int64_t newtonIters = 0, linearIters = 0;
    double tAdmit = 0.0, tFinish = -1.0;

    ~Slot()
    {
        if (c) dxg_ctx_destroy(c);
    }
};

}  // namespace

struct dxg_batch {
    int device = 0;
    int precision = DXG_PRECISION_MIXED;
    cudaStream_t stream = nullptr;
    cudaStream_t aux[3] = {nullptr, nullptr, nullptr};   // forked streams of the sweep classes
    cudaEvent_t forkEv = nullptr;
    cudaEvent_t joinEv[3] = {nullptr, nullptr, nullptr};
    std::string err;
    bool graphs = true, autotune = true;
    bool redBlack = false;            // red-black ordered ILU(0) instead of the natural order
    bool amg = false;                 // AMG-BiCGSTAB instead of ILU(0)-BiCGSTAB
    int64_t budget = 0, bytesInUse = 0;
    int64_t nextId = 1;
    int64_t launches = 0;
    std::map<int64_t, std::unique_ptr<Slot>> slots;
    Arena arena;
    DevBuf<SlotReport> reports;
    DevBuf<int> tuneFlags;
    SlotReport* reportsHost = nullptr;
    size_t reportsCap = 0;
    std::map<GroupKey, std::unique_ptr<GroupState>> groups;              // per kind: chunk arguments, graph
    std::chrono::steady_clock::time_point epoch = std::chrono::steady_clock::now();

    // optional event timing per kernel class (direct launches while it is on)
    struct Timed {
        cudaEvent_t start, stop;
        int kclass;
        double bytes;
    };
    bool timing = false;
    std::vector<Timed> pending;
    std::vector<cudaEvent_t> eventPool;
    int64_t kcLaunches[DXG_KC_COUNT] = {};
    double kcMs[DXG_KC_COUNT] = {};
    double kcBytes[DXG_KC_COUNT] = {};

    double clock() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - epoch).count();
    }
};

namespace {

std::string g_batchCreateError;

template <class F>
int guardedB(dxg_batch* b, F&& f)
{
    try {
        return f();
    } catch (const Error& e) {
        b->err = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        b->err = "host allocation failed";
        return DXG_ERR_OOM;
    } catch (const std::exception& e) {
        b->err = e.what();
        return DXG_ERR_CUDA;
    }
}

using Members = std::vector<Slot*>;

cudaEvent_t takeEventB(dxg_batch* B)
{
    if (!B->eventPool.empty()) {
        cudaEvent_t e = B->eventPool.back();
        B->eventPool.pop_back();
        return e;
    }
    cudaEvent_t e;
    DXG_CUDA(cudaEventCreate(&e));
    return e;
}

void resolveTimingsB(dxg_batch* B)
{
    if (B->pending.empty()) return;
    DXG_CUDA(cudaStreamSynchronize(B->stream));
    for (auto& t : B->pending) {
        float ms = 0.f;
        DXG_CUDA(cudaEventElapsedTime(&ms, t.start, t.stop));
        B->kcLaunches[t.kclass] += 1;
        B->kcMs[t.kclass] += ms;
        B->kcBytes[t.kclass] += t.bytes;
        B->eventPool.push_back(t.start);
        B->eventPool.push_back(t.stop);
    }
    B->pending.clear();
}

// Brackets the launches of one kernel class with events while timing is on.
struct TimedB {
    dxg_batch* B;
    cudaEvent_t e0 = nullptr;
    int kc;
    double bytes;
    TimedB(dxg_batch* b, int kclass, double by) : B(b), kc(kclass), bytes(by)
    {
        if (!B->timing) return;
        e0 = takeEventB(B);
        DXG_CUDA(cudaEventRecord(e0, B->stream));
    }
    ~TimedB()
    {
        if (!e0) return;
        cudaEvent_t e1 = takeEventB(B);
        cudaEventRecord(e1, B->stream);
        B->pending.push_back({e0, e1, kc, bytes});
    }
};

// Algorithmic bytes of one launch over the members (per-problem FP64 figures, scaled
// to the operand size of the launch).
double bytesOf(const std::vector<Slot*>& S, double dxg_ctx::*field, double scale)
{
    double t = 0.0;
    for (Slot* s : S) t += s->c->*field;
    return t * scale;
}

void ensureReports(dxg_batch* B, size_t n)
{
    if (n <= B->reportsCap) return;
    const size_t cap = std::max<size_t>(n, 2 * B->reportsCap);
    DXG_CUDA(cudaStreamSynchronize(B->stream));
    if (B->reportsHost) cudaFreeHost(B->reportsHost);
    B->reportsHost = nullptr;
    DXG_CUDA(cudaMallocHost(&B->reportsHost, cap * sizeof(SlotReport)));
    B->reports.alloc(cap);
    B->reportsCap = cap;
}

// Gathers one status record per member into reportsHost (synchronises the stream).
void gather(dxg_batch* B, const Members& S)
{
    ensureReports(B, S.size());
    std::vector<GatherArgs> g(S.size());
    for (size_t k = 0; k < S.size(); ++k) g[k] = {S[k]->c->ks.get(), S[k]->c->scal.get(), S[k]->c->singular.get()};
    GatherArgs* dg = B->arena.put(g, B->stream);
    gatherKernel<<<(unsigned)((S.size() + 127) / 128), 128, 0, B->stream>>>(dg, B->reports.get(), (int)S.size());
    DXG_CUDA(cudaGetLastError());
    B->launches += 1;
    DXG_CUDA(cudaMemcpyAsync(B->reportsHost, B->reports.get(), S.size() * sizeof(SlotReport), cudaMemcpyDeviceToHost,
                             B->stream));
    DXG_CUDA(cudaStreamSynchronize(B->stream));
}

void batchCopy(dxg_batch* B, const std::vector<CopyArgs>& v)
{
    if (v.empty()) return;
    int64_t mx = 1;
    for (const auto& a : v) mx = std::max(mx, a.n);
    const unsigned gx = (unsigned)std::min<int64_t>((mx + 255) / 256, 1184);
    copyKernel<<<dim3(gx, (unsigned)v.size()), 256, 0, B->stream>>>(B->arena.put(v, B->stream));
    DXG_CUDA(cudaGetLastError());
    B->launches += 1;
}

int64_t maxCells(const Members& S)
{
    int64_t m = 1;
    for (Slot* s : S) m = std::max(m, s->c->N);
    return m;
}
int64_t maxDofs(const Members& S)
{
    int64_t m = 1;
    for (Slot* s : S) m = std::max(m, s->c->M);
    return m;
}

// ---------------------------------------------------------------- sweep shape
std::vector<WaveGeom> geomsFor(const Members& S, int ctas)
{
    std::vector<WaveGeom> g;
    g.reserve(S.size());
    for (Slot* s : S) g.push_back(waveGeom(s->c->dim, s->c->pcHost.nx, s->c->pcHost.ny, s->c->pcHost.nz, ctas));
    return g;
}

// Candidate launch shapes: cluster sizes 1..16, the fewest threads that keep every
// problem at <= 2 lines per thread (and twice that), prefetch depths 1..8 through the
// shared-memory ring or 0 (direct loads behind L1 prefetches).
std::vector<WaveBatchPlan> candidates(const Members& S, int dim, int b, bool fp64)
{
    std::vector<WaveBatchPlan> out;
    for (int ctas : {1, 2, 4, 8, 16}) {
        const std::vector<WaveGeom> g = geomsFor(S, ctas);
        int maxLines = 0;
        for (const auto& x : g) maxLines = std::max(maxLines, x.linesPerCta);
        const int t2 = ((maxLines + 1) / 2 + 31) / 32 * 32;
        for (int threads : {t2, 2 * t2}) {
            if (threads < 32 || threads > 1024) continue;
            for (int pf : {0, 1, 2, 4, 8}) {
                WaveBatchPlan p;
                p.ctas = ctas;
                p.threads = threads;
                p.pf = pf;
                if (completeWaveBatchPlan(p, g, dim, b, fp64) > 0) out.push_back(p);
            }
        }
    }
    return out;
}

template <class T>
WaveArgs<T> waveArgsOf(const dxg_ctx* c, const WaveGeom& g, const T* A, T* L, T* Dinv, const T* rhs, T* v,
                       const KrylovState* ks)
{
    WaveArgs<T> w{};
    w.dim = c->dim;
    w.nx = c->pcHost.nx;
    w.ny = c->pcHost.ny;
    w.nz = c->pcHost.nz;
    w.N = c->N;
    w.ctas = g.ctas;
    w.linesPerCta = g.linesPerCta;
    w.haloLines = g.haloLines;
    w.A = A;
    w.L = L;
    w.Dinv = Dinv;
    w.rhs = rhs;
    w.v = v;
    w.err = c->singular.get() + 1;
    w.singular = c->singular.get();
    w.ks = ks;
    return w;
}

// Per-problem operands of the ILU(0) preconditioner in precision PT: the FP64 Jacobian
// and factors (plain path), or the FP32 Jacobian copy, factors and operand copies
// (mixed precision).  Krylov vectors and SpMV are FP64 in both.
template <class PT>
struct Pre;
template <>
struct Pre<double> {
    static const double* A(dxg_ctx* c) { return c->A.get(); }
    static double* L(dxg_ctx* c) { return c->L.get(); }
    static double* Dinv(dxg_ctx* c) { return c->Dinv.get(); }
    static const double* pIn(dxg_ctx* c) { return c->kp.get(); }
    static const double* rIn(dxg_ctx* c) { return c->kr.get(); }
    static double* yOut(dxg_ctx* c) { return c->ky.get(); }
};
template <>
struct Pre<float> {
    static const float* A(dxg_ctx* c) { return c->Af.get(); }
    static float* L(dxg_ctx* c) { return c->Lf.get(); }
    static float* Dinv(dxg_ctx* c) { return c->Dinvf.get(); }
    static const float* pIn(dxg_ctx* c) { return c->fp.get(); }
    static const float* rIn(dxg_ctx* c) { return c->fr.get(); }
    static float* yOut(dxg_ctx* c) { return c->fy.get(); }
};

template <class T>
RbArgs<T> rbArgsOf(dxg_ctx* c, const KrylovState* ks)
{
    RbArgs<T> r{};
    r.A = Pre<T>::A(c);
    r.Dinv = Pre<T>::Dinv(c);
    r.nbmask = c->nbmask.get();
    r.N = c->N;
    for (int s = 0; s < 7; ++s) r.off[s] = c->off[s];
    r.nx = (int)c->pcHost.nx;
    r.ny = (int)c->pcHost.ny;
    r.nz = (int)c->pcHost.nz;
    r.singular = c->singular.get();
    r.ks = ks;
    return r;
}

BicgArgs<double> krylovArgs(dxg_ctx* c, bool mixed)
{
    BicgArgs<double> a{c->kx.get(), c->kr.get(), c->krt.get(), c->kp.get(), c->kv.get(), c->kt.get(), c->ky.get(),
                       c->M, c->ks.get(), c->scratch(), nullptr, 0.0, 0, nullptr, nullptr, nullptr};
    if (mixed) {
        a.pLow = c->fp.get();
        a.rLow = c->fr.get();
        a.yLow = c->fy.get();
    }
    return a;
}

// Times the forward + backward sweep pair of every candidate shape on the members'
// own factors (Krylov state detached, so nothing is skipped) and keeps the fastest.
// The sweeps read the members' preconditioner inputs and write only their
// preconditioner outputs, which hold no state between BiCGSTAB half steps.
template <class PT>
WaveBatchPlan tunePlan(dxg_batch* B, const Members& S, int dim, int b)
{
    const bool fp64 = sizeof(PT) == 8;
    std::vector<WaveBatchPlan> cand = candidates(S, dim, b, fp64);
    if (cand.empty()) throw Error(DXG_ERR_ARG, "no batched ILU(0) sweep shape fits these grids");
    if (!B->autotune || cand.size() == 1) {
        // fixed rule: the largest cluster with the fewest threads and the deepest prefetch
        WaveBatchPlan best = cand.front();
        for (const auto& p : cand)
            if (p.ctas > best.ctas || (p.ctas == best.ctas && p.threads < best.threads) ||
                (p.ctas == best.ctas && p.threads == best.threads && p.pf > best.pf))
                best = p;
        return best;
    }
    cudaStream_t st = B->stream;
    // the tuning sweeps report expired waits into the batch's own flags, not the members'
    if (!B->tuneFlags.get()) B->tuneFlags.alloc(2);
    DXG_CUDA(cudaMemsetAsync(B->tuneFlags.get(), 0, 2 * sizeof(int), st));
    cudaEvent_t e0, e1;
    DXG_CUDA(cudaEventCreate(&e0));
    DXG_CUDA(cudaEventCreate(&e1));
    float bestMs = 1e30f;
    WaveBatchPlan best = cand.front();
    for (const WaveBatchPlan& p : cand) {
        const std::vector<WaveGeom> g = geomsFor(S, p.ctas);
        std::vector<WaveArgs<PT>> fw(S.size()), bw(S.size());
        for (size_t k = 0; k < S.size(); ++k) {
            dxg_ctx* c = S[k]->c;
            fw[k] = waveArgsOf<PT>(c, g[k], Pre<PT>::A(c), Pre<PT>::L(c), Pre<PT>::Dinv(c), Pre<PT>::rIn(c),
                                   Pre<PT>::yOut(c), nullptr);
            bw[k] = waveArgsOf<PT>(c, g[k], Pre<PT>::A(c), Pre<PT>::L(c), Pre<PT>::Dinv(c), nullptr,
                                   Pre<PT>::yOut(c), nullptr);
            fw[k].singular = bw[k].singular = B->tuneFlags.get();
            fw[k].err = bw[k].err = B->tuneFlags.get() + 1;
        }
        const WaveArgs<PT>* dfw = B->arena.put(fw, st);
        const WaveArgs<PT>* dbw = B->arena.put(bw, st);
        launchWaveApplyBatch<PT>(p, dfw, dbw, (int)S.size(), dim, b, st);   // warm-up
        DXG_CUDA(cudaEventRecord(e0, st));
        for (int rep = 0; rep < 2; ++rep) launchWaveApplyBatch<PT>(p, dfw, dbw, (int)S.size(), dim, b, st);
        DXG_CUDA(cudaEventRecord(e1, st));
        DXG_CUDA(cudaEventSynchronize(e1));
        B->launches += 6;
        float ms = 0.f;
        DXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < bestMs) {
            bestMs = ms;
            best = p;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int flags[2] = {0, 0};
    DXG_CUDA(cudaMemcpy(flags, B->tuneFlags.get(), sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags[1]) throw Error(DXG_ERR_TIMEOUT, "ILU(0) wavefront wait timed out while tuning");
    return best;
}

// Batch shape of a set of problems: kind, member count (next power of two), largest
// extents (in multiples of 16 cells); sweep shapes are cached per batch shape.
std::tuple<int, int, int, int, int> shapeKey(const Members& S, int dim, int b, int typeSize)
{
    int mx[3] = {0, 0, 0};
    for (Slot* s : S) {
        mx[0] = std::max(mx[0], s->c->pcHost.nx);
        mx[1] = std::max(mx[1], s->c->pcHost.ny);
        mx[2] = std::max(mx[2], s->c->pcHost.nz);
    }
    int cnt = 1;
    while (cnt < (int)S.size()) cnt *= 2;
    return std::make_tuple(b * 100 + dim * 10 + typeSize, cnt, (mx[0] + 15) / 16, (mx[1] + 15) / 16,
                           (mx[2] + 15) / 16);
}

// Tuned sweep shapes, shared by every batch of the process on the same device (a shape
// depends on the problems' extents and the GPU, not on the batch object): a new batch of
// known shapes starts without re-timing candidates.
struct TuneCache {
    std::mutex m;
    std::map<std::tuple<int, int, std::tuple<int, int, int, int, int>>, WaveBatchPlan> plans;
    std::map<std::tuple<int, std::vector<int>>, std::vector<WaveBatchPlan>> joint;
};
TuneCache& tuneCache()
{
    static TuneCache c;
    return c;
}

template <class PT>
WaveBatchPlan planFor(dxg_batch* B, const Members& S, int dim, int b)
{
    const auto key = std::make_tuple(B->device, (int)B->autotune, shapeKey(S, dim, b, (int)sizeof(PT)));
    TuneCache& tc = tuneCache();
    {
        std::lock_guard<std::mutex> lock(tc.m);
        auto it = tc.plans.find(key);
        if (it != tc.plans.end()) {
            WaveBatchPlan p = it->second;
            if (completeWaveBatchPlan(p, geomsFor(S, p.ctas), dim, b, sizeof(PT) == 8) > 0) return p;
        }
    }
    WaveBatchPlan p = tunePlan<PT>(B, S, dim, b);
    std::lock_guard<std::mutex> lock(tc.m);
    tc.plans[key] = p;
    return p;
}

// ---------------------------------------------------------------- group state
// The members of one kind and the argument blocks of their BiCGSTAB chunk, kept at
// fixed device addresses while the membership is unchanged, so that the chunk is
// captured once as a CUDA graph and replayed every tick.  Members whose solve has
// ended (Krylov status not running) skip inside every kernel of the chunk.
constexpr int kChunk = 8;    // BiCGSTAB iterations per tick

// Sweep size classes: one block size serves every problem of a sweep launch, so problems
// are split by their number of lines (ny*nz in 3D, ny in 2D) into classes with their own
// autotuned launch shape; the classes' sweeps run concurrently on forked streams.
constexpr int kMaxSweepClasses = 4;
inline int sweepClassOf(const dxg_ctx* c)
{
    const int lines = c->dim == 3 ? c->pcHost.ny * c->pcHost.nz : c->pcHost.ny;
    return lines <= 512 ? 0 : lines <= 1024 ? 1 : lines <= 2048 ? 2 : 3;
}

struct SweepClass {
    std::vector<int> members;       // indices into the group
    WaveBatchPlan plan;
    const void* dFwP = nullptr;
    const void* dFwR = nullptr;
    const void* dBw = nullptr;
};

struct GroupState {
    std::vector<int64_t> ids;
    std::vector<SweepClass> classes;
    std::vector<int> classOf;       // per member: index into classes
    std::vector<WaveGeom> geo;      // per member, from its class's launch shape
    DevBuf<unsigned char> args;
    const BicgArgs<double>* dBicg = nullptr;
    const void* dSv1 = nullptr;      // SpmvArgs<double, double, PT>
    const void* dSv2 = nullptr;
    const ToDoubleArgs* dTd = nullptr;
    const void* dRbP = nullptr;      // red-black order: RbArgs<PT> applied to p / to r
    const void* dRbR = nullptr;
    BlockMap mapM, mapN;     // vector kernels over N*b entries, SpMV over N cells
    BlockMap mapH;           // red-black passes over each problem's colour slots
    struct AmgLaunch {
        int kind;
        const void* passes;      // AmgPass<PT>[] of the problems taking part
        BlockMap map;
    };
    std::vector<AmgLaunch> amgP, amgR;   // V-cycle passes applied to p / to r
    int64_t maxN = 1, maxM = 1;
    double sweepBytes = 0, spmvBytes = 0;
    cudaGraphExec_t exec = nullptr;
    bool graphTried = false;
    ~GroupState()
    {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

template <class T>
size_t pack(std::vector<unsigned char>& buf, const std::vector<T>& v)
{
    const size_t off = (buf.size() + 255) & ~(size_t)255;
    buf.resize(off + v.size() * sizeof(T));
    std::memcpy(buf.data() + off, v.data(), v.size() * sizeof(T));
    return off;
}

// The classes' sweeps run concurrently, so shapes tuned class by class (each alone on
// an idle GPU) are not the best together.  One pass of coordinate descent re-chooses each
// class's shape, the others fixed, by timing the whole concurrent apply on the members'
// own factors (Krylov state detached; expired waits go to the batch's tuning flags).
template <class PT>
void refineClassPlans(dxg_batch* B, std::vector<SweepClass>& classes, const Members& S, int dim, int b)
{
    const int nc = (int)classes.size();
    if (nc < 2 || !B->autotune) return;
    std::vector<int> jkey;
    std::vector<Members> subs(nc);
    for (int q = 0; q < nc; ++q) {
        for (int k : classes[q].members) subs[q].push_back(S[k]);
        const auto k = shapeKey(subs[q], dim, b, (int)sizeof(PT));
        jkey.insert(jkey.end(), {std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k), std::get<4>(k)});
    }
    TuneCache& tc = tuneCache();
    const auto ckey = std::make_tuple(B->device, jkey);
    std::vector<WaveBatchPlan> known;
    {
        std::lock_guard<std::mutex> lock(tc.m);
        auto cached = tc.joint.find(ckey);
        if (cached != tc.joint.end()) known = cached->second;
    }
    if (!known.empty()) {
        bool ok = true;
        std::vector<WaveBatchPlan> plans = known;
        for (int q = 0; q < nc && ok; ++q)
            ok = completeWaveBatchPlan(plans[q], geomsFor(subs[q], plans[q].ctas), dim, b, sizeof(PT) == 8) > 0;
        if (ok) {
            for (int q = 0; q < nc; ++q) classes[q].plan = plans[q];
            return;
        }
    }
    cudaStream_t st = B->stream;
    if (!B->tuneFlags.get()) B->tuneFlags.alloc(2);
    DXG_CUDA(cudaMemsetAsync(B->tuneFlags.get(), 0, 2 * sizeof(int), st));
    cudaEvent_t e0, e1;
    DXG_CUDA(cudaEventCreate(&e0));
    DXG_CUDA(cudaEventCreate(&e1));
    auto timeAll = [&](const std::vector<WaveBatchPlan>& plans) {
        std::vector<const WaveArgs<PT>*> dfw(nc), dbw(nc);
        for (int q = 0; q < nc; ++q) {
            const std::vector<WaveGeom> g = geomsFor(subs[q], plans[q].ctas);
            std::vector<WaveArgs<PT>> fw, bw;
            for (size_t j = 0; j < subs[q].size(); ++j) {
                dxg_ctx* c = subs[q][j]->c;
                WaveArgs<PT> f = waveArgsOf<PT>(c, g[j], Pre<PT>::A(c), Pre<PT>::L(c), Pre<PT>::Dinv(c),
                                                Pre<PT>::rIn(c), Pre<PT>::yOut(c), nullptr);
                f.singular = B->tuneFlags.get();
                f.err = B->tuneFlags.get() + 1;
                WaveArgs<PT> w = f;
                w.rhs = nullptr;
                fw.push_back(f);
                bw.push_back(w);
            }
            dfw[q] = B->arena.put(fw, st);
            dbw[q] = B->arena.put(bw, st);
        }
        auto apply = [&] {
            DXG_CUDA(cudaEventRecord(B->forkEv, st));
            for (int q = 0; q < nc; ++q) {
                cudaStream_t sq = q == 0 ? st : B->aux[q - 1];
                if (q > 0) DXG_CUDA(cudaStreamWaitEvent(sq, B->forkEv, 0));
                launchWaveApplyBatch<PT>(plans[q], dfw[q], dbw[q], (int)subs[q].size(), dim, b, sq);
                if (q > 0) DXG_CUDA(cudaEventRecord(B->joinEv[q - 1], sq));
            }
            for (int q = 1; q < nc; ++q) DXG_CUDA(cudaStreamWaitEvent(st, B->joinEv[q - 1], 0));
            B->launches += 2 * nc;
        };
        apply();   // warm-up
        DXG_CUDA(cudaEventRecord(e0, st));
        apply();
        apply();
        DXG_CUDA(cudaEventRecord(e1, st));
        DXG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        DXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return ms;
    };
    std::vector<WaveBatchPlan> plans(nc);
    for (int q = 0; q < nc; ++q) plans[q] = classes[q].plan;
    float best = timeAll(plans);
    for (int q = 0; q < nc; ++q) {
        for (const WaveBatchPlan& c : candidates(subs[q], dim, b, sizeof(PT) == 8)) {
            if (c.ctas == plans[q].ctas && c.threads == plans[q].threads && c.pf == plans[q].pf) continue;
            std::vector<WaveBatchPlan> trial = plans;
            trial[q] = c;
            const float t = timeAll(trial);
            if (t < best) {
                best = t;
                plans = trial;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int flags[2] = {0, 0};
    DXG_CUDA(cudaMemcpy(flags, B->tuneFlags.get(), sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags[1]) throw Error(DXG_ERR_TIMEOUT, "ILU(0) wavefront wait timed out while tuning");
    {
        std::lock_guard<std::mutex> lock(tc.m);
        tc.joint[ckey] = plans;
    }
    for (int q = 0; q < nc; ++q) classes[q].plan = plans[q];
}

// The passes of one V-cycle for every member, aligned by (level, phase, sweep): a problem
// takes part in a pass when it has that level (above its last) and that many sweeps.  The
// per-problem sequence is the single context's (same passes, same buffers, same order).
template <class PT>
struct AmgPassList {
    int kind;
    std::vector<AmgPass<PT>> passes;
    std::vector<uint2> map;
};
template <class PT>
std::vector<AmgPassList<PT>> amgCycleSchedule(const std::vector<std::vector<AmgLevel<PT>>>& lv,
                                              const std::vector<const KrylovState*>& ks, int b)
{
    size_t dmax = 0;
    int smax = 1;
    for (const auto& L : lv) {
        dmax = std::max(dmax, L.size());
        for (const auto& l : L) smax = std::max(smax, l.sweeps);
    }
    std::vector<AmgPassList<PT>> out;
    const PT omega = (PT)kAmgOmega;
    auto emit = [&](int kind, auto&& make) {
        AmgPassList<PT> pl;
        pl.kind = kind;
        for (size_t k = 0; k < lv.size(); ++k) {
            AmgPass<PT> p{};
            if (!make(k, p)) continue;
            p.ks = ks[k];
            p.omega = omega;
            const unsigned nb = amgPassBlocks(kind == AMG_RESTRICT ? p.C.N : (kind == AMG_COARSE ? p.L.N * b : p.L.N));
            for (unsigned j = 0; j < nb; ++j) pl.map.push_back(make_uint2((unsigned)pl.passes.size(), j));
            pl.passes.push_back(p);
        }
        if (!pl.passes.empty()) out.push_back(std::move(pl));
    };
    for (size_t l = 0; l + 1 < dmax; ++l) {
        emit(AMG_FIRST, [&](size_t k, AmgPass<PT>& p) {
            if (l + 1 >= lv[k].size()) return false;
            p.L = lv[k][l];
            p.out = p.L.tmp;
            return true;
        });
        for (int kk = 1; kk < smax; ++kk)
            emit(AMG_JACOBI, [&](size_t k, AmgPass<PT>& p) {
                if (l + 1 >= lv[k].size() || kk >= lv[k][l].sweeps) return false;
                p.L = lv[k][l];
                PT* buf[2] = {p.L.tmp, p.L.x};
                p.in = buf[(kk - 1) & 1];
                p.out = buf[kk & 1];
                return true;
            });
        emit(AMG_RESIDUAL, [&](size_t k, AmgPass<PT>& p) {
            if (l + 1 >= lv[k].size()) return false;
            p.L = lv[k][l];
            PT* buf[2] = {p.L.tmp, p.L.x};
            p.in = buf[(p.L.sweeps - 1) & 1];
            return true;
        });
        emit(AMG_RESTRICT, [&](size_t k, AmgPass<PT>& p) {
            if (l + 1 >= lv[k].size()) return false;
            p.L = lv[k][l];
            p.C = lv[k][l + 1];
            return true;
        });
    }
    emit(AMG_COARSE, [&](size_t k, AmgPass<PT>& p) {
        p.L = lv[k].back();
        return true;
    });
    for (size_t l = dmax - 1; l-- > 0;) {
        emit(AMG_JACOBI, [&](size_t k, AmgPass<PT>& p) {
            if (l + 1 >= lv[k].size()) return false;
            p.L = lv[k][l];
            p.C = lv[k][l + 1];
            PT* buf[2] = {p.L.tmp, p.L.x};
            const int sw = p.L.sweeps;
            p.in = buf[(sw - 1) & 1];
            p.out = buf[sw & 1];
            p.prolong = 1;
            return true;
        });
        for (int kk = 1; kk < smax; ++kk)
            emit(AMG_JACOBI, [&](size_t k, AmgPass<PT>& p) {
                if (l + 1 >= lv[k].size() || kk >= lv[k][l].sweeps) return false;
                p.L = lv[k][l];
                PT* buf[2] = {p.L.tmp, p.L.x};
                const int sw = p.L.sweeps;
                p.in = buf[(sw - 1 + kk) & 1];
                p.out = buf[(sw + kk) & 1];
                return true;
            });
    }
    return out;
}

// (Re)builds the group's chunk arguments when its membership changed.
template <class PT>
GroupState& groupState(dxg_batch* B, const GroupKey& key, const Members& S)
{
    auto& slot = B->groups[key];
    std::vector<int64_t> ids;
    for (Slot* s : S) ids.push_back(s->id);
    if (slot && slot->ids == ids) return *slot;
    constexpr bool mixed = sizeof(PT) == 4;
    cudaStream_t st = B->stream;
    DXG_CUDA(cudaStreamSynchronize(st));     // the previous arguments may still be read
    slot.reset(new GroupState());
    GroupState& G = *slot;
    G.ids = ids;
    const int n = (int)S.size();
    const int dim = S[0]->c->dim, b = S[0]->c->b;
    if (!B->redBlack && !B->amg) {
        int cls[kMaxSweepClasses] = {-1, -1, -1, -1};
        G.classOf.resize(n);
        for (int k = 0; k < n; ++k) {
            const int q = sweepClassOf(S[k]->c);
            if (cls[q] < 0) {
                cls[q] = (int)G.classes.size();
                G.classes.emplace_back();
            }
            G.classOf[k] = cls[q];
            G.classes[cls[q]].members.push_back(k);
        }
        G.geo.resize(n);
        for (SweepClass& sc : G.classes) {
            Members sub;
            for (int k : sc.members) sub.push_back(S[k]);
            sc.plan = planFor<PT>(B, sub, dim, b);
        }
        refineClassPlans<PT>(B, G.classes, S, dim, b);
        for (SweepClass& sc : G.classes) {
            Members sub;
            for (int k : sc.members) sub.push_back(S[k]);
            const std::vector<WaveGeom> g = geomsFor(sub, sc.plan.ctas);
            for (size_t j = 0; j < sc.members.size(); ++j) G.geo[sc.members[j]] = g[j];
        }
    }
    G.maxN = maxCells(S);
    G.maxM = maxDofs(S);
    G.sweepBytes = bytesOf(S, &dxg_ctx::bytesSweep, sizeof(PT) / 8.0);
    // the operator is the FP64 Jacobian in both precisions (mixed: times the FP32 preconditioner
    // output, whose entries are read at half the bytes)
    G.spmvBytes = bytesOf(S, &dxg_ctx::bytesSpmv, 1.0);
    if (mixed)
        for (Slot* q : S) G.spmvBytes -= 0.5 * (double)q->c->N * q->c->b * 8.0;
    std::vector<BicgArgs<double>> ba(n);
    std::vector<SpmvArgs<double, double, PT>> sv1(n), sv2(n);
    std::vector<WaveArgs<PT>> fwP(n), fwR(n), bw(n);   // member order; repacked per class below
    std::vector<RbArgs<PT>> rbP(n), rbR(n);
    std::vector<ToDoubleArgs> td(n);
    for (int k = 0; k < n; ++k) {
        dxg_ctx* c = S[k]->c;
        ba[k] = krylovArgs(c, mixed);
        SpmvArgs<double, double, PT> sv{};
        sv.A = c->A.get();
        sv.nbmask = c->nbmask.get();
        sv.N = c->N;
        for (int q = 0; q < 7; ++q) sv.off[q] = c->off[q];
        sv.ks = c->ks.get();
        sv.scratch = c->scratch();
        sv.x = Pre<PT>::yOut(c);
        sv.y = ba[k].v;
        sv.w = ba[k].rt;
        sv1[k] = sv;
        sv.y = ba[k].t;
        sv.w = ba[k].r;
        sv2[k] = sv;
        const PT* PA = Pre<PT>::A(c);
        if (!B->redBlack && !B->amg) {
            fwP[k] = waveArgsOf<PT>(c, G.geo[k], PA, Pre<PT>::L(c), Pre<PT>::Dinv(c), Pre<PT>::pIn(c),
                                    Pre<PT>::yOut(c), c->ks.get());
            fwR[k] = waveArgsOf<PT>(c, G.geo[k], PA, Pre<PT>::L(c), Pre<PT>::Dinv(c), Pre<PT>::rIn(c),
                                    Pre<PT>::yOut(c), c->ks.get());
            bw[k] = waveArgsOf<PT>(c, G.geo[k], PA, Pre<PT>::L(c), Pre<PT>::Dinv(c), nullptr, Pre<PT>::yOut(c),
                                   c->ks.get());
        }
        RbArgs<PT> rb = rbArgsOf<PT>(c, c->ks.get());
        rb.v = Pre<PT>::yOut(c);
        rb.d = Pre<PT>::pIn(c);
        rbP[k] = rb;
        rb.d = Pre<PT>::rIn(c);
        rbR[k] = rb;
        td[k] = {c->fy.get(), c->ky.get(), c->M};
    }
    std::vector<int64_t> lenM, lenN, lenH;
    for (Slot* s : S) {
        lenM.push_back(s->c->M);
        lenN.push_back(s->c->N);
        lenH.push_back(rbSlots((int)s->c->pcHost.nx, (int)s->c->pcHost.ny, (int)s->c->pcHost.nz));
    }
    std::vector<uint2> mM, mN, mH;
    buildBlockMap(lenM, false, mM);
    buildBlockMap(lenN, true, mN);
    buildBlockMap(lenH, true, mH);
    std::vector<unsigned char> host;
    const size_t oB = pack(host, ba), o1 = pack(host, sv1), o2 = pack(host, sv2), oT = pack(host, td),
                 oM = pack(host, mM), oN = pack(host, mN), oH = pack(host, mH), oRP = pack(host, rbP),
                 oRR = pack(host, rbR);
    // AMG: the V-cycle passes for the preconditioner applied to p and to r
    struct AmgOff {
        int kind;
        size_t passes, map;
        unsigned blocks;
    };
    std::vector<AmgOff> amgOffP, amgOffR;
    if (B->amg) {
        std::vector<std::vector<AmgLevel<PT>>> lp, lr;
        std::vector<const KrylovState*> ks;
        for (Slot* s : S) {
            dxg_ctx* c = s->c;
            lp.push_back(amgLevelsOf<PT>(c, Pre<PT>::A(c), Pre<PT>::Dinv(c), Pre<PT>::pIn(c), Pre<PT>::yOut(c)));
            lr.push_back(amgLevelsOf<PT>(c, Pre<PT>::A(c), Pre<PT>::Dinv(c), Pre<PT>::rIn(c), Pre<PT>::yOut(c)));
            ks.push_back(c->ks.get());
        }
        for (auto& pl : amgCycleSchedule<PT>(lp, ks, b))
            amgOffP.push_back({pl.kind, pack(host, pl.passes), pack(host, pl.map), (unsigned)pl.map.size()});
        for (auto& pl : amgCycleSchedule<PT>(lr, ks, b))
            amgOffR.push_back({pl.kind, pack(host, pl.passes), pack(host, pl.map), (unsigned)pl.map.size()});
    }
    std::vector<std::array<size_t, 3>> oc;
    for (const SweepClass& sc : G.classes) {
        std::vector<WaveArgs<PT>> cP, cR, cW;
        for (int k : sc.members) {
            cP.push_back(fwP[k]);
            cR.push_back(fwR[k]);
            cW.push_back(bw[k]);
        }
        oc.push_back({pack(host, cP), pack(host, cR), pack(host, cW)});
    }
    G.args.alloc(host.size());
    DXG_CUDA(cudaMemcpy(G.args.get(), host.data(), host.size(), cudaMemcpyHostToDevice));
    unsigned char* d = G.args.get();
    G.dBicg = reinterpret_cast<const BicgArgs<double>*>(d + oB);
    G.dSv1 = d + o1;
    G.dSv2 = d + o2;
    for (size_t q = 0; q < G.classes.size(); ++q) {
        G.classes[q].dFwP = d + oc[q][0];
        G.classes[q].dFwR = d + oc[q][1];
        G.classes[q].dBw = d + oc[q][2];
    }
    G.dTd = reinterpret_cast<const ToDoubleArgs*>(d + oT);
    G.mapM = {reinterpret_cast<const uint2*>(d + oM), (unsigned)mM.size()};
    G.mapN = {reinterpret_cast<const uint2*>(d + oN), (unsigned)mN.size()};
    G.mapH = {reinterpret_cast<const uint2*>(d + oH), (unsigned)mH.size()};
    G.dRbP = d + oRP;
    G.dRbR = d + oRR;
    for (const AmgOff& o : amgOffP)
        G.amgP.push_back({o.kind, d + o.passes, BlockMap{reinterpret_cast<const uint2*>(d + o.map), o.blocks}});
    for (const AmgOff& o : amgOffR)
        G.amgR.push_back({o.kind, d + o.passes, BlockMap{reinterpret_cast<const uint2*>(d + o.map), o.blocks}});
    return G;
}

// One chunk of BiCGSTAB iterations for every member of the group.
template <class PT>
void enqueueChunk(dxg_batch* B, const GroupState& G, int n, int dim, int b)
{
    constexpr bool mixed = sizeof(PT) == 4;
    cudaStream_t st = B->stream;
    const int nc = (int)G.classes.size();
    // forward + backward sweep of every class; classes after the first on forked streams
    auto precondition = [&](bool onP) {
        if (B->amg) {
            TimedB tb(B, DXG_KC_ILU_SWEEP, G.sweepBytes);
            for (const auto& a : onP ? G.amgP : G.amgR)
                launchAmgPassBatch<PT>(a.kind, static_cast<const AmgPass<PT>*>(a.passes), a.map.map, a.map.blocks, dim,
                                       b, st);
            return;
        }
        if (B->redBlack) {
            TimedB tb(B, DXG_KC_ILU_SWEEP, G.sweepBytes);
            launchRbApplyBatch<PT>(static_cast<const RbArgs<PT>*>(onP ? G.dRbP : G.dRbR), G.mapH, b, dim, st);
            return;
        }
        {
            TimedB tb(B, DXG_KC_ILU_SWEEP, G.sweepBytes);
            if (nc > 1) DXG_CUDA(cudaEventRecord(B->forkEv, st));
            for (int q = 0; q < nc; ++q) {
                const SweepClass& sc = G.classes[q];
                cudaStream_t sq = q == 0 ? st : B->aux[q - 1];
                if (q > 0) DXG_CUDA(cudaStreamWaitEvent(sq, B->forkEv, 0));
                launchWaveApplyBatch<PT>(sc.plan, static_cast<const WaveArgs<PT>*>(onP ? sc.dFwP : sc.dFwR),
                                         static_cast<const WaveArgs<PT>*>(sc.dBw), (int)sc.members.size(), dim, b,
                                         sq);
                if (q > 0) DXG_CUDA(cudaEventRecord(B->joinEv[q - 1], sq));
            }
            for (int q = 1; q < nc; ++q) DXG_CUDA(cudaStreamWaitEvent(st, B->joinEv[q - 1], 0));
        }
    };
    for (int it = 0; it < kChunk; ++it) {
        // the rho step ran in the kernel that closed the previous iteration
        launchBicgUpdatePBatch<double>(G.dBicg, G.mapM, st);
        precondition(true);
        {
            TimedB tb(B, DXG_KC_SPMV, G.spmvBytes);
            launchSpmvBatch<double, double, PT>(static_cast<const SpmvArgs<double, double, PT>*>(G.dSv1), G.mapN, b, dim, 1,
                                            st);
        }
        launchBicgAxpyNormBatch<double>(G.dBicg, G.mapM, 0, st);
        precondition(false);
        {
            TimedB tb(B, DXG_KC_SPMV, G.spmvBytes);
            launchSpmvBatch<double, double, PT>(static_cast<const SpmvArgs<double, double, PT>*>(G.dSv2), G.mapN, b, dim, 2,
                                            st);
        }
        launchBicgAxpyNormBatch<double>(G.dBicg, G.mapM, 1, st);
    }
}

template <class PT>
void runChunk(dxg_batch* B, GroupState& G, int n, int dim, int b)
{
    const int launchesPerIt =
        5 + (B->amg ? (int)(G.amgP.size() + G.amgR.size()) : (B->redBlack ? 4 : 4 * (int)G.classes.size()));
    cudaStream_t st = B->stream;
    if (B->graphs && !B->timing && !G.exec && !G.graphTried) {
        G.graphTried = true;
        cudaGraph_t graph = nullptr;
        bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess;
        if (ok) {
            try {
                enqueueChunk<PT>(B, G, n, dim, b);
            } catch (const Error&) {
                ok = false;
            }
            ok = (cudaStreamEndCapture(st, &graph) == cudaSuccess) && ok && graph;
        }
        if (ok && cudaGraphInstantiate(&G.exec, graph, 0) != cudaSuccess) {
            G.exec = nullptr;
            ok = false;
        }
        if (graph) cudaGraphDestroy(graph);
        if (!ok) {
            cudaGetLastError();
            G.exec = nullptr;
        }
    }
    if (G.exec && !B->timing) DXG_CUDA(cudaGraphLaunch(G.exec, st));
    else enqueueChunk<PT>(B, G, n, dim, b);
    B->launches += (int64_t)kChunk * launchesPerIt;
}

// Status of a member's finished BiCGSTAB run.
int krylovFailure(const SlotReport& r)
{
    if (r.timeout) return DXG_ERR_TIMEOUT;
    if (r.singular) return DXG_ERR_LINEAR_BREAKDOWN;
    if (r.status == KS_BREAKDOWN) return DXG_ERR_LINEAR_BREAKDOWN;
    if (r.status == KS_NAN) return DXG_ERR_NAN;
    return DXG_OK;
}

// ---------------------------------------------------------------- Newton control
// newtonProceed (newtonsolver.hh:428-446)
bool proceed(const Slot& s, bool conv)
{
    if (s.numSteps < s.p.min_steps) return true;
    if (conv) return false;
    if (s.numSteps >= s.p.max_steps) return s.shift * 4.0 < s.lastShift;
    return true;
}

// suggestTimeStepSize (newtonsolver.hh:784-798)
double suggest(const Slot& s, double dt)
{
    const int target = s.p.target_steps;
    if (s.numSteps > target) return dt / (1.0 + double(s.numSteps - target) / target);
    return dt * (1.0 + double(target - s.numSteps) / target / 1.2);
}

void finish(dxg_batch* B, Slot* s, int state, int status)
{
    s->state = state;
    s->status = status;
    s->tFinish = B->clock();
}

// ---------------------------------------------------------------- residual reduction
// Members that need the residual norm after an update: Newton.UseLineSearch and
// Newton.EnableResidualCriterion.
bool needsResidual(const Slot* s) { return s->p.use_line_search || s->p.enable_residual_criterion; }

// FVAssembler::assembleResidual for members of one group: own-state volume variables and
// residual rows, the launches of the single context's residual assembly.
void assembleResiduals(dxg_batch* B, const Members& S)
{
    cudaStream_t st = B->stream;
    const dxg_ctx* c0 = S[0]->c;
    std::vector<AssemblyArgs> aa;
    for (Slot* s : S) {
        AssemblyArgs a = s->c->asmArgs();
        a.u = s->c->u.get();
        aa.push_back(a);
    }
    const AssemblyArgs* daa = B->arena.put(aa, st);
    const int64_t maxN = maxCells(S);
    launchVolvarsBatch(daa, (int)S.size(), maxN, c0->b, 2, st);
    launchRowBatch(daa, (int)S.size(), maxN, c0->b, c0->dim, c0->method, false, c0->gravity && c0->pcHost.gravAxisMask,
                   S[0]->transient, c0->fullUpwind, st);
    B->launches += 2;
}

// Euclidean norms of the members' residuals (IstlIterativeLinearSolver::norm) through the
// single context's reduction kernel, so a member's norm is the same alone and batched.
std::vector<double> residualNorms(dxg_batch* B, const Members& S)
{
    for (Slot* s : S) {
        launchNorm2(s->c->r.get(), s->c->M, s->c->scratch(), s->c->scal.get() + 1, B->stream);
        B->launches += 1;
    }
    gather(B, S);
    std::vector<double> n(S.size());
    for (size_t k = 0; k < S.size(); ++k) n[k] = B->reportsHost[k].norm;
    return n;
}

// u = uLast - lambda * delta and the relative shift for each member (in place, u == uLast,
// when `fromLast` is false); the shifts come back through a gather.
std::vector<double> newtonUpdates(dxg_batch* B, const Members& S, const std::vector<double>& lambda,
                                  const std::vector<bool>& fromLast)
{
    std::vector<NewtonUpdArgs> ua;
    std::vector<int64_t> lenM;
    for (size_t k = 0; k < S.size(); ++k) {
        dxg_ctx* c = S[k]->c;
        ua.push_back({fromLast[k] ? c->uLast.get() : c->u.get(), c->kx.get(), c->u.get(), lambda[k], c->M,
                      c->scratch(), c->scal.get()});
        lenM.push_back(c->M);
    }
    std::vector<uint2> mM;
    buildBlockMap(lenM, false, mM);
    launchNewtonUpdateBatch(B->arena.put(ua, B->stream), BlockMap{B->arena.put(mM, B->stream), (unsigned)mM.size()},
                            B->stream);
    B->launches += 1;
    gather(B, S);
    std::vector<double> shift(S.size());
    for (size_t k = 0; k < S.size(); ++k) shift[k] = B->reportsHost[k].shift;
    return shift;
}

// Assembly, ILU(0) factorisation and BiCGSTAB start for members that begin a Newton
// iteration (FVAssembler::assembleJacobianAndResidual + the solver's setup).
template <class PT>
void beginIterations(dxg_batch* B, const GroupState& G, const Members& S, const std::vector<int>& idx)
{
    constexpr bool mixed = sizeof(PT) == 4;
    cudaStream_t st = B->stream;
    const int n = (int)idx.size();
    dxg_ctx* c0 = S[idx[0]]->c;
    const int b = c0->b, dim = c0->dim, method = c0->method;
    const bool grav = c0->gravity && c0->pcHost.gravAxisMask;
    const bool transient = S[idx[0]]->transient;
    Members A;
    for (int k : idx) A.push_back(S[k]);
    const int64_t maxN = maxCells(A), maxM = maxDofs(A);

    // storage of the previous time level for members that start a time step
    std::vector<AssemblyArgs> pv;
    for (Slot* s : A) {
        s->c->dt = s->transient ? s->dt : 0.0;
        if (s->transient && !s->c->stPrevValid) {
            AssemblyArgs a = s->c->asmArgs();
            a.uprev = s->c->uprev.get();
            pv.push_back(a);
            s->c->stPrevValid = true;
        }
    }
    if (!pv.empty()) {
        launchPrevStorageBatch(B->arena.put(pv, st), (int)pv.size(), maxN, b, st);
        B->launches += 1;
    }
    std::vector<AssemblyArgs> aa(n);
    std::vector<ToFloatArgs> tf(n);
    std::vector<GatherArgs> fl(n);
    std::vector<WaveArgs<PT>> fa(n);
    std::vector<RbArgs<PT>> rf(n);
    std::vector<BicgArgs<double>> bi(n);
    int64_t maxA = 1;
    for (int k = 0; k < n; ++k) {
        Slot* s = A[k];
        dxg_ctx* c = s->c;
        aa[k] = c->asmArgs();
        aa[k].u = c->u.get();
        const int64_t nA = (int64_t)c->slots * c->N * c->bb;
        maxA = std::max(maxA, nA);
        tf[k] = {c->A.get(), c->Af.get(), nA};
        fl[k] = {c->ks.get(), c->scal.get(), c->singular.get()};
        // the factor must not skip: no Krylov state
        if (B->redBlack) rf[k] = rbArgsOf<PT>(c, nullptr);
        else if (!B->amg)
            fa[k] = waveArgsOf<PT>(c, G.geo[idx[k]], Pre<PT>::A(c), Pre<PT>::L(c), Pre<PT>::Dinv(c), nullptr,
                                   nullptr, nullptr);
        BicgArgs<double> a = krylovArgs(c, mixed);
        a.rhs = c->r.get();
        a.reduction = s->p.linear_reduction;
        a.maxHalf = 2 * s->p.linear_max_iter;
        bi[k] = a;
    }
    const AssemblyArgs* daa = B->arena.put(aa, st);
    {
        TimedB tb(B, DXG_KC_ASSEMBLY, bytesOf(A, &dxg_ctx::bytesAssembly, 1.0));
        launchVolvarsBatch(daa, n, maxN, b, method, st);
        launchRowBatch(daa, n, maxN, b, dim, method, true, grav, transient, c0->fullUpwind, st);
    }
    // the initial residual of an attempt, for the residual reduction (solveImpl_)
    Members R;
    for (Slot* s : A) {
        if (!needsResidual(s)) continue;
        s->lastReduction = s->numSteps == 0 ? 1.0 : s->reduction;
        if (s->numSteps == 0) R.push_back(s);
    }
    if (!R.empty()) {
        const std::vector<double> r0 = residualNorms(B, R);
        for (size_t k = 0; k < R.size(); ++k) R[k]->initialResidual = r0[k];
    }
    if (mixed) {
        launchToFloatBatch(B->arena.put(tf, st), n, maxA, st);
        B->launches += 1;
    }
    clearFlagsKernel<<<(n + 127) / 128, 128, 0, st>>>(B->arena.put(fl, st), n);
    DXG_CUDA(cudaGetLastError());
    if (B->amg) {
        // AMG setup: pivots of level 0, each coarse operator from the one above, the last
        // level's dense inverse
        std::vector<std::vector<AmgLevel<PT>>> lv;
        size_t dmax = 0;
        int64_t maxLast = 1;
        for (Slot* s : A) {
            dxg_ctx* c = s->c;
            lv.push_back(amgLevelsOf<PT>(c, Pre<PT>::A(c), Pre<PT>::Dinv(c), nullptr, nullptr));
            dmax = std::max(dmax, lv.back().size());
            maxLast = std::max(maxLast, lv.back().back().N);
        }
        auto run = [&](int kind, size_t l) {
            std::vector<AmgPass<PT>> ps;
            std::vector<uint2> mp;
            for (size_t k = 0; k < lv.size(); ++k) {
                if (l >= lv[k].size()) continue;
                AmgPass<PT> p{};
                p.L = kind == AMG_DIAGINV ? lv[k][0] : lv[k][l - 1];
                if (kind == AMG_COARSEN) p.C = lv[k][l];
                p.singular = A[k]->c->singular.get();
                const unsigned nb = amgPassBlocks(kind == AMG_COARSEN ? p.C.N : p.L.N);
                for (unsigned j = 0; j < nb; ++j) mp.push_back(make_uint2((unsigned)ps.size(), j));
                ps.push_back(p);
            }
            if (ps.empty()) return;
            launchAmgPassBatch<PT>(kind, B->arena.put(ps, st), B->arena.put(mp, st), (unsigned)mp.size(), dim, b, st);
            B->launches += 1;
        };
        run(AMG_DIAGINV, 0);
        for (size_t l = 1; l < dmax; ++l) run(AMG_COARSEN, l);
        std::vector<AmgPass<PT>> inv;
        for (size_t k = 0; k < lv.size(); ++k) {
            AmgPass<PT> p{};
            p.L = lv[k].back();
            p.singular = A[k]->c->singular.get();
            inv.push_back(p);
        }
        launchAmgInvertBatch<PT>(B->arena.put(inv, st), (int)inv.size(), (int)maxLast, dim, b, st);
        B->launches += 1;
    }
    if (B->redBlack) {
        std::vector<int64_t> lenH;
        for (Slot* s : A) lenH.push_back(rbSlots((int)s->c->pcHost.nx, (int)s->c->pcHost.ny, (int)s->c->pcHost.nz));
        std::vector<uint2> mH;
        buildBlockMap(lenH, true, mH);
        launchRbFactorBatch<PT>(B->arena.put(rf, st), BlockMap{B->arena.put(mH, st), (unsigned)mH.size()}, b, dim,
                                st);
        B->launches += 2;
    }
    for (size_t q = 0; q < G.classes.size(); ++q) {
        std::vector<WaveArgs<PT>> fq;
        for (int k = 0; k < n; ++k)
            if (G.classOf[idx[k]] == (int)q) fq.push_back(fa[k]);
        if (fq.empty()) continue;
        launchWaveFactorBatch<PT>(G.classes[q].plan, B->arena.put(fq, st), (int)fq.size(), dim, b, st);
        B->launches += 1;
    }
    std::vector<int64_t> lenM;
    for (Slot* s : A) lenM.push_back(s->c->M);
    std::vector<uint2> mM;
    buildBlockMap(lenM, false, mM);
    launchBicgInitBatch<double>(B->arena.put(bi, st), BlockMap{B->arena.put(mM, st), (unsigned)mM.size()}, st);
    B->launches += 4;
    for (Slot* s : A) {
        s->solving = true;
        s->chunks = 0;
    }
}

// One tick of a group: start Newton iterations, one BiCGSTAB chunk for every member,
// then the update and the Newton / time-loop decisions of members whose solve ended.
template <class PT>
void tickGroup(dxg_batch* B, const GroupKey& key, const Members& S)
{
    cudaStream_t st = B->stream;
    GroupState& G = groupState<PT>(B, key, S);
    const int n = (int)S.size();
    const int dim = S[0]->c->dim, b = S[0]->c->b;
    std::vector<int> starting;
    for (int k = 0; k < n; ++k)
        if (!S[k]->solving) starting.push_back(k);
    if (!starting.empty()) beginIterations<PT>(B, G, S, starting);

    runChunk<PT>(B, G, n, dim, b);
    gather(B, S);

    Members U;
    std::vector<int> ended;
    for (int k = 0; k < n; ++k) {
        Slot* s = S[k];
        const SlotReport& r = B->reportsHost[k];
        s->chunks += 1;
        const bool stopped = r.status != KS_RUNNING || r.timeout || s->chunks * kChunk > s->p.linear_max_iter + kChunk;
        if (!stopped) continue;
        s->solving = false;
        s->linIters = (r.halfsteps + 1) / 2;
        s->linStatus = krylovFailure(r);
        s->linConv = s->linStatus == DXG_OK && r.status == KS_CONVERGED;
        ended.push_back(k);
        if (s->linConv) U.push_back(s);
    }
    if (ended.empty()) return;
    // u -= delta and the relative shift for members whose solve converged; members with a
    // line search keep the last iterate (uLastIter) for their backtracking
    std::map<Slot*, double> shifts;
    if (!U.empty()) {
        std::vector<CopyArgs> keep;
        std::vector<bool> fromLast;
        for (Slot* s : U) {
            fromLast.push_back(s->p.use_line_search != 0);
            if (s->p.use_line_search) keep.push_back({s->c->uLast.get(), s->c->u.get(), s->c->M});
        }
        batchCopy(B, keep);
        const std::vector<double> sh = newtonUpdates(B, U, std::vector<double>(U.size(), 1.0), fromLast);
        for (size_t k = 0; k < U.size(); ++k) shifts[U[k]] = sh[k];
    }
    // residual reduction (Newton.EnableResidualCriterion) and the backtracking line search
    // (Newton.UseLineSearch, lineSearchUpdate_, newtonsolver.hh:1154-1178): lambda halves
    // from 1 until the reduction falls below the last iteration's or lambda reaches
    // Newton.LineSearchMinRelaxationFactor; the shift is the accepted iterate's
    Members R;
    std::map<Slot*, double> lambda;
    for (Slot* s : U)
        if (needsResidual(s)) {
            R.push_back(s);
            lambda[s] = 1.0;
        }
    while (!R.empty()) {
        assembleResiduals(B, R);
        const std::vector<double> norms = residualNorms(B, R);
        Members again;
        std::vector<double> lam;
        for (size_t k = 0; k < R.size(); ++k) {
            Slot* s = R[k];
            s->reduction = norms[k] / s->initialResidual;
            if (!s->p.use_line_search || s->reduction < s->lastReduction ||
                lambda[s] <= s->p.line_search_min_relaxation)
                continue;
            lambda[s] *= 0.5;
            again.push_back(s);
            lam.push_back(lambda[s]);
        }
        if (again.empty()) break;
        const std::vector<double> sh = newtonUpdates(B, again, lam, std::vector<bool>(again.size(), true));
        for (size_t k = 0; k < again.size(); ++k) shifts[again[k]] = sh[k];
        R = again;
    }

    std::vector<CopyArgs> restore, advance;
    for (int k : ended) {
        Slot* s = S[k];
        // iterations are counted as the reference reports them: those that reached the
        // update (an iteration whose linear solve failed ends the attempt uncounted)
        if (s->linConv) s->newtonIters += 1;
        s->linearIters += s->linIters;
        if (s->linStatus == DXG_ERR_TIMEOUT) {
            finish(B, s, SLOT_FAILED, DXG_ERR_TIMEOUT);
            continue;
        }
        bool failed = false;
        if (!s->linConv) failed = true;   // NumericalProblem: the linear solver did not converge
        else {
            s->lastShift = s->shift;
            s->shift = shifts[s];
            s->numSteps += 1;
            // newtonConverged (newtonsolver.hh:657-701): the shift, or with the residual
            // criterion either of the shift and the residual reduction
            const bool conv = s->shift <= s->p.max_relative_shift ||
                              (s->p.enable_residual_criterion && s->reduction <= s->p.residual_reduction);
            if (!std::isfinite(s->shift)) failed = true;
            else if (!proceed(*s, conv)) {
                if (!conv) failed = true;
                else {
                    // converged time step (or the stationary solve)
                    s->steps += 1;
                    if (!s->transient) {
                        finish(B, s, SLOT_DONE, DXG_OK);
                        continue;
                    }
                    s->t += s->dt;
                    advance.push_back({s->c->uprev.get(), s->c->u.get(), s->c->M});
                    s->c->stPrevValid = false;
                    const double remaining = s->tEnd - s->t;
                    if (remaining <= 1e-9 * std::max(1.0, s->tEnd)) {
                        finish(B, s, SLOT_DONE, DXG_OK);
                        continue;
                    }
                    s->dt = std::min(std::min(suggest(*s, s->dt), s->dtMax), remaining);
                    s->numSteps = 0;
                    s->shift = s->lastShift = 0.0;
                    s->reduction = 0.0;
                    s->divisions = 0;
                }
            }
        }
        if (failed) {
            // NewtonSolver::solve: back to the previous time level, reduced dt, retry
            if (!s->transient || s->divisions >= s->p.max_time_step_divisions) {
                finish(B, s, SLOT_FAILED, s->linStatus != DXG_OK ? s->linStatus : DXG_ERR_NEWTON_NOT_CONVERGED);
                continue;
            }
            s->divisions += 1;
            s->totalDivisions += 1;
            s->dt *= s->p.retry_time_step_reduction;
            s->numSteps = 0;
            s->shift = s->lastShift = 0.0;
            restore.push_back({s->c->u.get(), s->c->uprev.get(), s->c->M});
        }
    }
    batchCopy(B, restore);
    batchCopy(B, advance);
}

std::string graphsNote(const GroupState& G) { return G.exec ? " graph" : ""; }

GroupKey keyOf(const Slot* s)
{
    const dxg_ctx* c = s->c;
    return GroupKey{c->b, c->dim, c->method, (c->gravity && c->pcHost.gravAxisMask) ? 1 : 0, s->transient ? 1 : 0,
                    c->fullUpwind ? 1 : 0};
}

int64_t problemBytes(int64_t N, int64_t nb, int b, int dim, int method, int precision)
{
    const int64_t bb = (int64_t)b * b, slots = 2 * dim + 1, M = N * b;
    const int NS = 1 + statesPerPv(method) * b;
    int64_t by = 0;
    by += (3 + dim) * N * 8 + b * N * 8 + 2 * (2 * b * N * 8) + N * 4 * 2 + N;   // cell tables, mask, level order
    by += nb * (1 + 8 + 4 * 8 * b);                                             // boundary tables
    by += 5 * M * 8 + b * N * 8 + 3 * (int64_t)NS * b * N * 8 + b * N * 8;       // state, volume variables, eps
    by += slots * N * bb * 8;                                                    // Jacobian
    by += 7 * M * 8;                                                             // Krylov vectors
    if (precision == DXG_PRECISION_FP64) by += (dim + 1) * N * bb * 8;           // L, D^-1
    else by += (slots + dim + 1) * N * bb * 4 + 3 * M * 4;                       // FP32 copy, L, D^-1, operands
    by += 3 * kMaxReduceBlocks * 8 + 4096;                                       // scratch and scalars
    return by + 64 * 1024;                                                       // allocation granularity
}

// Device memory of a problem's AMG levels (the layout of amgLevelsOf): two fine-level
// vectors, per coarse level its operator, pivots and four vectors, the last level's dense
// inverse.
int64_t amgBytes(const dxg_problem_desc* d, int precision)
{
    const int64_t val = precision == DXG_PRECISION_FP64 ? 8 : 4;
    const int dim = d->dim, b = d->num_eq, S = 2 * dim + 1;
    const int64_t bb = (int64_t)b * b;
    int64_t N = 1;
    for (int a = 0; a < dim; ++a) N *= d->cells[a];
    auto align = [](int64_t v) { return (v + 255) & ~(int64_t)255; };
    int64_t by = 2 * align(N * b * val);
    const auto dims = amgLevelDims(dim, (int)d->cells[0], (int)d->cells[1], dim == 3 ? (int)d->cells[2] : 1);
    for (const auto& l : dims) {
        const int64_t n = (int64_t)l[0] * l[1] * l[2];
        by += align(S * n * bb * val) + align(n * bb * val) + 4 * align(n * b * val);
    }
    const int64_t nLast = dims.empty() ? N : (int64_t)dims.back()[0] * dims.back()[1] * dims.back()[2];
    return by + align(nLast * b * nLast * b * val);
}

}  // namespace

// ================================================================ C ABI
extern "C" {

int dxg_batch_create(dxg_batch** out, int device, int precision)
{
    if (!out || (precision != DXG_PRECISION_FP64 && precision != DXG_PRECISION_MIXED)) return DXG_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        g_batchCreateError = "no CUDA device";
        return DXG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return DXG_ERR_ARG;
    auto* b = new dxg_batch();
    b->device = device;
    b->precision = precision;
    const int st = guardedB(b, [&] {
        DXG_CUDA(cudaSetDevice(device));
        DXG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        for (auto& a : b->aux) DXG_CUDA(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
        DXG_CUDA(cudaEventCreateWithFlags(&b->forkEv, cudaEventDisableTiming));
        for (auto& e : b->joinEv) DXG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        return DXG_OK;
    });
    if (st != DXG_OK) {
        g_batchCreateError = b->err;
        delete b;
        return st;
    }
    *out = b;
    return DXG_OK;
}

int dxg_batch_destroy(dxg_batch* b)
{
    if (!b) return DXG_ERR_ARG;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto& t : b->pending) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    for (auto e : b->eventPool) cudaEventDestroy(e);
    b->groups.clear();
    b->slots.clear();
    if (b->reportsHost) cudaFreeHost(b->reportsHost);
    b->reports.release();
    for (auto a : b->aux)
        if (a) {
            cudaStreamSynchronize(a);
            cudaStreamDestroy(a);
        }
    if (b->forkEv) cudaEventDestroy(b->forkEv);
    for (auto e : b->joinEv)
        if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return DXG_OK;
}

const char* dxg_batch_last_error(const dxg_batch* b) { return b ? b->err.c_str() : g_batchCreateError.c_str(); }

int dxg_batch_set_option(dxg_batch* b, int option, int value)
{
    if (!b) return DXG_ERR_ARG;
    if (option == DXG_BATCH_OPT_GRAPHS) b->graphs = value != 0;
    else if (option == DXG_BATCH_OPT_AUTOTUNE) {
        b->autotune = value != 0;
    } else if (option == DXG_BATCH_OPT_AMG) {
        if (!b->slots.empty()) {
            b->err = "the linear solver is chosen before problems are added";
            return DXG_ERR_STATE;
        }
        b->amg = value != 0;
        b->groups.clear();
    } else if (option == DXG_BATCH_OPT_ILU_REDBLACK) {
        if (!b->slots.empty()) {
            b->err = "the ILU(0) ordering is chosen before problems are added";
            return DXG_ERR_STATE;
        }
        b->redBlack = value != 0;
        b->groups.clear();
    } else return DXG_ERR_ARG;
    return DXG_OK;
}

int64_t dxg_problem_device_bytes(const dxg_problem_desc* d, int precision)
{
    if (!d || (d->dim != 2 && d->dim != 3) || (d->num_eq != 1 && d->num_eq != 2)) return -1;
    int64_t N = 1;
    for (int a = 0; a < d->dim; ++a) {
        if (d->cells[a] <= 0) return -1;
        N *= d->cells[a];
    }
    const int64_t nb = dxg_num_boundary_faces(d);
    if (d->discretization == DXG_DISC_MPFA_O) {
        // flux rows (F scvfs x (2^dim coefficients + constant) + kind), stencil mask and
        // source, the Jacobian and its factor over 3^dim slots, eleven vectors
        const int64_t S = d->dim == 2 ? 9 : 27, K = 1 << d->dim, F = 2 * d->dim * (K / 2);
        return N * (F * (K + 1) * 8 + F + 4 + 8) + N * S * 8 * 2 + N * 8 * 12;
    }
    return problemBytes(N, nb, d->num_eq, d->dim, d->numeric_difference_method, precision);
}

int dxg_batch_set_memory_budget(dxg_batch* b, int64_t bytes)
{
    if (!b || bytes < 0) return DXG_ERR_ARG;
    b->budget = bytes;
    return DXG_OK;
}

int64_t dxg_batch_device_bytes(const dxg_batch* b) { return b ? b->bytesInUse : -1; }

int dxg_batch_add(dxg_batch* b, const dxg_problem_desc* d, const double* u0, double dt, double max_dt,
                  double t_end, const dxg_newton_params* params, int64_t* id)
{
    if (!b || !d || !u0 || !id) return DXG_ERR_ARG;
    if (d->discretization != DXG_DISC_TPFA) {
        b->err = "batched problems use the TPFA discretization";
        return DXG_ERR_ARG;
    }
    int64_t need = dxg_problem_device_bytes(d, b->precision);
    if (need < 0) {
        b->err = "invalid problem description";
        return DXG_ERR_ARG;
    }
    if (b->amg) need += amgBytes(d, b->precision);
    if (b->budget > 0 && b->bytesInUse + need > b->budget) {
        b->err = "admission would exceed the device-memory budget";
        return DXG_ERR_BUDGET;
    }
    auto s = std::make_unique<Slot>();
    int st = dxg_ctx_create(&s->c, b->device);
    if (st != DXG_OK) {
        b->err = dxg_last_error(nullptr);
        return st;
    }
    auto step = [&](int status) {
        if (status != DXG_OK && b->err.empty()) b->err = dxg_last_error(s->c);
        return status;
    };
    b->err.clear();
    if ((st = step(dxg_set_precision(s->c, b->precision))) != DXG_OK) return st;
    if ((st = step(dxg_problem_upload(s->c, d))) != DXG_OK) return st;
    if ((st = step(dxg_set_solution(s->c, u0))) != DXG_OK) return st;
    if ((st = step(dxg_set_prev_solution(s->c, u0))) != DXG_OK) return st;
    if (params) s->p = *params;
    else dxg_newton_default_params(&s->p);
    if (s->p.enable_partial_reassembly) {
        b->err = "batched problems reassemble the full Jacobian (no partial reassembly)";
        return DXG_ERR_ARG;
    }
    s->transient = t_end > 0.0 && dt > 0.0;
    s->tEnd = s->transient ? t_end : 0.0;
    s->dt = s->transient ? std::min(dt, t_end) : 0.0;
    s->dtMax = max_dt > 0.0 ? max_dt : 1e300;
    s->bytes = need;
    s->tAdmit = b->clock();
    s->id = b->nextId++;
    *id = s->id;
    b->bytesInUse += need;
    b->slots[s->id] = std::move(s);
    return DXG_OK;
}

int dxg_batch_iterate(dxg_batch* b, int32_t* active)
{
    if (!b) return DXG_ERR_ARG;
    return guardedB(b, [&] {
        DXG_CUDA(cudaSetDevice(b->device));
        std::map<GroupKey, Members> groups;
        for (auto& kv : b->slots)
            if (kv.second->state == SLOT_ACTIVE) groups[keyOf(kv.second.get())].push_back(kv.second.get());
        b->arena.reset();
        // release the chunk arguments and graphs of kinds without active members
        for (auto it = b->groups.begin(); it != b->groups.end();) {
            if (groups.count(it->first)) ++it;
            else {
                DXG_CUDA(cudaStreamSynchronize(b->stream));
                it = b->groups.erase(it);
            }
        }
        for (auto& g : groups) {
            if (b->precision == DXG_PRECISION_FP64) tickGroup<double>(b, g.first, g.second);
            else tickGroup<float>(b, g.first, g.second);
        }
        DXG_CUDA(cudaStreamSynchronize(b->stream));
        int n = 0;
        for (auto& kv : b->slots) n += kv.second->state == SLOT_ACTIVE;
        if (active) *active = n;
        return DXG_OK;
    });
}

int dxg_batch_run(dxg_batch* b)
{
    if (!b) return DXG_ERR_ARG;
    while (true) {
        int32_t n = 0;
        const int st = dxg_batch_iterate(b, &n);
        if (st != DXG_OK) return st;
        if (n == 0) return DXG_OK;
    }
}

int dxg_batch_info(const dxg_batch* b, int64_t id, dxg_batch_problem_info* info)
{
    if (!b || !info) return DXG_ERR_ARG;
    auto it = b->slots.find(id);
    if (it == b->slots.end()) return DXG_ERR_ARG;
    const Slot& s = *it->second;
    info->state = s.state;
    info->status = s.status;
    info->time_steps = s.steps;
    info->time_step_divisions = s.totalDivisions;
    info->newton_iterations = s.newtonIters;
    info->linear_iterations = s.linearIters;
    info->cells = s.c->N;
    info->time = s.t;
    info->seconds_admitted = s.tAdmit;
    info->seconds_finished = s.tFinish;
    return DXG_OK;
}

int dxg_batch_get_solution(dxg_batch* b, int64_t id, double* u)
{
    if (!b || !u) return DXG_ERR_ARG;
    auto it = b->slots.find(id);
    if (it == b->slots.end()) return DXG_ERR_ARG;
    const int st = dxg_get_solution(it->second->c, u);
    if (st != DXG_OK) b->err = dxg_last_error(it->second->c);
    return st;
}

int dxg_batch_remove(dxg_batch* b, int64_t id)
{
    if (!b) return DXG_ERR_ARG;
    auto it = b->slots.find(id);
    if (it == b->slots.end()) return DXG_ERR_ARG;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    b->bytesInUse -= it->second->bytes;
    b->slots.erase(it);
    return DXG_OK;
}

int64_t dxg_batch_launch_count(const dxg_batch* b) { return b ? b->launches : -1; }

int dxg_batch_describe(const dxg_batch* b, char* buf, int64_t len)
{
    if (!b || !buf || len <= 0) return DXG_ERR_ARG;
    std::string out;
    for (const auto& kv : b->groups) {
        const GroupKey& k = kv.first;
        const GroupState& G = *kv.second;
        out += "group num_eq=" + std::to_string(std::get<0>(k)) + " dim=" + std::to_string(std::get<1>(k)) +
               " problems=" + std::to_string(G.ids.size()) + ":";
        if (b->redBlack) out += " [red-black ILU(0): two parallel passes per sweep]";
        if (b->amg) out += " [AMG-BiCGSTAB: " + std::to_string(G.amgP.size()) + " batched passes per V-cycle]";
        for (const SweepClass& sc : G.classes)
            out += " [" + std::to_string(sc.members.size()) + " problems: cluster " + std::to_string(sc.plan.ctas) +
                   " x " + std::to_string(sc.plan.threads) + " threads, prefetch " + std::to_string(sc.plan.pf) +
                   "]";
        out += graphsNote(G) + "\n";
    }
    std::strncpy(buf, out.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
    return DXG_OK;
}

int dxg_batch_set_kernel_timing(dxg_batch* b, int enable)
{
    if (!b) return DXG_ERR_ARG;
    return guardedB(b, [&] {
        resolveTimingsB(b);
        b->timing = enable != 0;
        for (int k = 0; k < DXG_KC_COUNT; ++k) {
            b->kcLaunches[k] = 0;
            b->kcMs[k] = 0;
            b->kcBytes[k] = 0;
        }
        return DXG_OK;
    });
}

int dxg_batch_get_kernel_timing(dxg_batch* b, int kc, int64_t* launches, double* ms, double* bytes)
{
    if (!b || kc < 0 || kc >= DXG_KC_COUNT) return DXG_ERR_ARG;
    return guardedB(b, [&] {
        resolveTimingsB(b);
        if (launches) *launches = b->kcLaunches[kc];
        if (ms) *ms = b->kcMs[kc];
        if (bytes) *bytes = b->kcBytes[kc];
        return DXG_OK;
    });
}

void* dxg_batch_stream(const dxg_batch* b) { return b ? (void*)b->stream : nullptr; }

}  // extern "C"
