// msx_pool.cu -- batched / serving pool of independent explicit solves.
//
// Every admitted solve owns one device arena (mesh, set-up data, nodal state,
// corner forces, CSR, Dirichlet tables) and one entry of the pool's control,
// CFL and NaN-flag tables.  All resident solves advance together: one pooled
// node kernel and one pooled element kernel per step, persistent grids that
// stride over a tile list (tile = contiguous element or node range of one
// solve), captured as a CUDA graph of `steps_per_launch` steps.  Admission is
// by HBM footprint; finished solves are copied out, freed and replaced
// between graph replays (continuous batching).  Tile size, CTA size and grid
// size are picked by timing candidates on the resident work.  In serving mode
// (msx_pool_serve) a library thread launches the replays back to back while
// any solve is resident; admissions build their host tables and upload their
// data without holding the pool's lock, so they overlap the replays.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/msx.h"
#include "msx_internal.h"

using namespace msx;

namespace {

msx_status pfail(msx_status st, const std::string &m)
{
    msx_set_error(m.c_str());
    return st;
}

#define PCUDA(call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return pfail(e_ == cudaErrorMemoryAllocation ? MSX_ERR_OOM : MSX_ERR_CUDA,        \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                 \
    } while (0)

__global__ void pool_init_ctrl(Problem p, double t0, long long limit)
{
    double dt0 = __longlong_as_double((long long)p.dtmin[0]) * p.sf;
    Ctrl c;
    c.t = t0;
    c.dt = dt0;
    c.step = 0;
    c.limit = limit;
    c.ran = 0;
    c.stop = 0;
    c.status = 0;
    c.pad = 0;
    c.pending = 0;
    p.ctrl[0] = c;
    p.ctrl[1] = c;
    p.flags[0] = 0;
    p.flags[1] = 0;
}

double now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Slot {
    bool active = false;
    bool reserved = false;   // taken by an admission whose uploads are still being enqueued
    bool launched = false;   // a replay ordered after the solve's admission has run on it
    long long ticket = -1;
    long long nn = 0, ne = 0;
    void *arena = nullptr;
    size_t bytes = 0;
    Problem P{};
    double submit_ms = 0;
};

// A finished solve: its result, and its arena, kept on the device until
// msx_pool_fetch copies u, v, a out (ready: recorded after the last replay
// and, for the pair-state modes, the merge of u, v, a back to FP64).
struct Finished {
    msx_pool_result res;
    void *arena = nullptr;
    size_t bytes = 0;
    long long nn = 0;
    const double *u = nullptr, *v = nullptr, *a = nullptr;
    cudaEvent_t ready = nullptr;
};

struct Sched {
    int threads = 256;
    int tile_elems = 1024;
    int ctas_per_sm = 4;
};

}  // namespace

struct msx_pool {
    std::mutex mu;
    msx_pool_opts opts{};
    int device = 0, sms = 152;
    cudaStream_t stream = nullptr;   // graph replays and result copies
    cudaStream_t upload = nullptr;   // admissions: uploads and set-up kernels, overlapping a replay
    cudaStream_t fetch = nullptr;    // msx_pool_fetch: result copies, overlapping a replay
    cudaEvent_t ev_upload = nullptr, ev_step = nullptr;
    bool uploads_pending = false;    // admissions since the last replay launch
    std::atomic<int> inject_alloc_failures{0};   // msx_pool_inject_alloc_failures
    bool inflight = false;           // a replay launched by msx_pool_step not yet collected
    std::vector<Slot> slots;
    Problem *d_descs = nullptr;
    Ctrl *d_ctrl = nullptr, *h_ctrl = nullptr;
    unsigned long long *d_dtmin = nullptr;
    int *d_flags = nullptr;
    Tile *d_etiles = nullptr, *d_ntiles = nullptr;
    int *d_counts = nullptr;   // element tiles, claim, done, node tiles, claim, done
    size_t tile_cap = 0;
    std::vector<Tile> h_etiles, h_ntiles;
    bool tiles_dirty = true;
    cudaGraphExec_t graph = nullptr;
    Sched sched;
    bool tuned = false;
    int spl = 32;
    long long next_ticket = 1;
    size_t used = 0, budget = 0;
    std::map<long long, Finished> done;
    std::deque<long long> done_order;
    long long elem_steps_finished = 0;   // element-steps of solves already collected
    long long elem_steps_active = 0;     // element-steps of resident solves at the last read
    // serving mode
    std::thread server;
    std::condition_variable cv_work;   // to the serving thread: a solve was admitted, or stop
    std::condition_variable cv_done;   // to msx_pool_wait: a replay was collected, or serving failed
    bool serving = false, serve_stop = false;
    msx_status serve_status = MSX_OK;
    std::string serve_error;
};

// ------------------------------------------------------------------ helpers
static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static int pool_mode(int precision)
{
    return precision == MSX_PREC_MIXED ? MODE_MIXED : (precision == MSX_PREC_DOUBLE_WORD ? MODE_DW : MODE_FP64);
}

// modes whose running state is the (hi, lo) FP32 pairs uhl, vhl, ahl
static bool pair_state(int precision) { return precision == MSX_PREC_MIXED || precision == MSX_PREC_DOUBLE_WORD; }

static size_t footprint(long long nn, long long ne, long long nbc, int precision, bool cnh)
{
    size_t b = 0;
    if (cnh)   // plain FP64, compressible neo-Hookean: Eref, Mg, rdetE
        b += align256(sizeof(double) * 9 * ne) + align256(sizeof(double) * 6 * ne) + align256(sizeof(double) * ne);
    b += align256(sizeof(int4) * ne) + align256(sizeof(double) * 9 * ne);           // conn, G
    b += 2 * align256(sizeof(double) * ne);                                         // wJ, Lref
    b += align256(sizeof(float) * 9 * ne) + 2 * align256(sizeof(float) * ne);        // G32, wJ32, Lref32
    b += 4 * align256(sizeof(double) * 3 * nn) + 2 * align256(sizeof(double) * nn);  // X, u, v, a, mass, minv
    b += align256(sizeof(float2) * 3 * nn);                                          // uhl
    if (pair_state(precision))                                                       // vhl, ahl, minv2
        b += 2 * align256(sizeof(float2) * 3 * nn) + align256(sizeof(float2) * nn);
    if (precision == MSX_PREC_FP64) b += align256(sizeof(double) * 4 * nn);          // u4 (node-major u)
    if (precision == MSX_PREC_DOUBLE_WORD)                                           // G32lo, wJ32lo
        b += align256(sizeof(float) * 9 * ne) + align256(sizeof(float) * ne);
    b += precision == MSX_PREC_MIXED ? align256(sizeof(float) * 16 * ne) : align256(sizeof(double) * 12 * ne);
    b += align256(sizeof(int) * (nn + 1)) + align256(sizeof(int) * 4 * ne) + align256(sizeof(int) * nn);
    b += align256(sizeof(int4) * ne);                                                // corner slots
    const long long nbcn = std::max(1LL, std::min(nn, nbc));   // nodes with Dirichlet entries, at most
    b += align256(sizeof(int2) * 3 * nbcn) + align256(sizeof(int2) * nbcn) + align256(sizeof(BCEntry) * (nbc > 0 ? nbc : 1));
    return b;
}

static msx_status make_mat(const msx_material &m, MatParams &o)
{
    if (m.law < 0 || m.law > 3) return pfail(MSX_ERR_ARG, "unknown constitutive law");
    if (!material_params(m, o)) return pfail(MSX_ERR_ARG, "material needs E > 0, rho > 0, -1 < nu < 0.5");
    return MSX_OK;
}

static void rebuild_tiles(msx_pool *p)
{
    p->h_etiles.clear();
    p->h_ntiles.clear();
    // node tiles of eight passes of a CTA's threads / 4 nodes: a pooled step has
    // many solves and millions of nodes, and tiles of two passes spent ~6 % of
    // the batched step on claims and barriers (256 solves: 1.81e10 -> 1.92e10
    // element-steps/s with eight passes)
    const int te = p->sched.tile_elems, tn = p->sched.threads * 2;
    for (int s = 0; s < (int)p->slots.size(); s++) {
        const Slot &sl = p->slots[s];
        if (!sl.active) continue;
        for (long long b = 0; b < sl.ne; b += te) p->h_etiles.push_back({s, (int)b, (int)std::min<long long>(sl.ne, b + te)});
        for (long long b = 0; b < sl.nn; b += tn) p->h_ntiles.push_back({s, (int)b, (int)std::min<long long>(sl.nn, b + tn)});
    }
    p->tiles_dirty = true;
}

static msx_status upload_tiles(msx_pool *p)
{
    if (!p->tiles_dirty) return MSX_OK;
    size_t need = std::max(p->h_etiles.size(), p->h_ntiles.size());
    if (need > p->tile_cap) {
        size_t cap = std::max<size_t>(need * 2, 4096);
        if (p->d_etiles) cudaFree(p->d_etiles);
        if (p->d_ntiles) cudaFree(p->d_ntiles);
        PCUDA(cudaMalloc(&p->d_etiles, sizeof(Tile) * cap));
        PCUDA(cudaMalloc(&p->d_ntiles, sizeof(Tile) * cap));
        p->tile_cap = cap;
        if (p->graph) {
            cudaGraphExecDestroy(p->graph);   // kernel arguments changed
            p->graph = nullptr;
        }
    }
    int counts[kTileSched] = {(int)p->h_etiles.size(), 0, 0, (int)p->h_ntiles.size(), 0, 0};
    if (counts[0]) PCUDA(cudaMemcpyAsync(p->d_etiles, p->h_etiles.data(), sizeof(Tile) * counts[0], cudaMemcpyHostToDevice, p->stream));
    if (counts[3]) PCUDA(cudaMemcpyAsync(p->d_ntiles, p->h_ntiles.data(), sizeof(Tile) * counts[3], cudaMemcpyHostToDevice, p->stream));
    PCUDA(cudaMemcpyAsync(p->d_counts, counts, sizeof(counts), cudaMemcpyHostToDevice, p->stream));
    PCUDA(cudaStreamSynchronize(p->stream));
    p->tiles_dirty = false;
    return MSX_OK;
}

static msx_status build_pool_graph(msx_pool *p, int steps)
{
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    const int mode = pool_mode(p->opts.precision);
    const int threads = p->sched.threads, grid = p->sms * p->sched.ctas_per_sm;
    const int node_grid = p->sms * tiled_ctas_per_sm(mode, threads, true);
    cudaGraph_t g;
    PCUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < steps; i++) {
        int parity = (i & 1) ? 0 : 1;
        launch_tiled_node(p->d_descs, p->d_ntiles, p->d_counts, mode, parity, node_grid, threads, p->stream);
        launch_tiled_elem(p->d_descs, p->d_etiles, p->d_counts, mode, parity, grid, threads, p->sched.tile_elems,
                          p->stream);
    }
    cudaError_t err = cudaStreamEndCapture(p->stream, &g);
    if (err != cudaSuccess) return pfail(MSX_ERR_CUDA, std::string("pool graph capture: ") + cudaGetErrorString(err));
    err = cudaGraphInstantiate(&p->graph, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) return pfail(MSX_ERR_CUDA, std::string("pool graph instantiate: ") + cudaGetErrorString(err));
    return MSX_OK;
}

// Copies out and frees every solve whose control slot says it stopped.
static msx_status collect(msx_pool *p)
{
    const size_t n = p->slots.size();
    PCUDA(cudaMemcpyAsync(p->h_ctrl, p->d_ctrl, sizeof(Ctrl) * 2 * n, cudaMemcpyDeviceToHost, p->stream));
    PCUDA(cudaStreamSynchronize(p->stream));
    bool changed = false;
    p->elem_steps_active = 0;
    for (size_t s = 0; s < n; s++) {
        Slot &sl = p->slots[s];
        if (!sl.active || !sl.launched) continue;   // admitted since the last launch: nothing to read yet
        const Ctrl &c = p->h_ctrl[2 * s];   // replays end on parity 0
        if (!c.stop) {
            p->elem_steps_active += sl.ne * c.step;
            continue;
        }
        p->elem_steps_finished += sl.ne * c.step;
        Finished f;
        f.res.ticket = sl.ticket;
        f.res.status = c.status;
        f.res.reserved = 0;
        f.res.steps = c.step;
        f.res.t = c.t;
        // no copy here: the result stays in the solve's arena until it is
        // fetched, so the next replay is not held up by device-to-host copies
        if (pair_state(p->opts.precision)) launch_state_merge(sl.P, p->opts.precision == MSX_PREC_MIXED, p->stream);
        PCUDA(cudaEventCreateWithFlags(&f.ready, cudaEventDisableTiming));
        PCUDA(cudaEventRecord(f.ready, p->stream));
        f.arena = sl.arena;
        f.bytes = sl.bytes;   // still counted in p->used until the fetch
        f.nn = sl.nn;
        f.u = sl.P.u;
        f.v = sl.P.v;
        f.a = sl.P.a;
        f.res.submit_to_done_ms = now_ms() - sl.submit_ms;
        sl = Slot();   // the slot and its control entries can take a new solve
        const long long t = f.res.ticket;
        p->done[t] = std::move(f);
        p->done_order.push_back(t);
        changed = true;
    }
    if (changed) {
        rebuild_tiles(p);
        p->cv_done.notify_all();   // msx_pool_wait callers in serving mode
    }
    return MSX_OK;
}

// One armed admission failure, if any is left (msx_pool_inject_alloc_failures).
static bool take_injected_failure(msx_pool *p)
{
    int n = p->inject_alloc_failures.load();
    while (n > 0 && !p->inject_alloc_failures.compare_exchange_weak(n, n - 1)) {
    }
    return n > 0;
}

static bool any_active(const msx_pool *p)
{
    for (const Slot &s : p->slots)
        if (s.active) return true;
    return false;
}

// One graph replay (spl steps) with the current schedule; returns device ms.
// Replays wait for the admissions enqueued on the upload stream.
static msx_status order_after_uploads(msx_pool *p)
{
    if (p->uploads_pending) {
        PCUDA(cudaStreamWaitEvent(p->stream, p->ev_upload, 0));
        p->uploads_pending = false;
    }
    // from here on every resident solve's control slot is initialised in stream
    // order: collect may read it
    for (Slot &s : p->slots)
        if (s.active) s.launched = true;
    return MSX_OK;
}

// One graph replay, launched without waiting (msx_pool_step): collected by the
// next step, poll or stats call.
static msx_status launch_replay(msx_pool *p)
{
    msx_status st;
    if ((st = order_after_uploads(p)) != MSX_OK) return st;
    if ((st = upload_tiles(p)) != MSX_OK) return st;
    if (!p->graph && (st = build_pool_graph(p, p->spl)) != MSX_OK) return st;
    PCUDA(cudaGraphLaunch(p->graph, p->stream));
    PCUDA(cudaEventRecord(p->ev_step, p->stream));
    p->inflight = true;
    return MSX_OK;
}

// Waits for the replay in flight, if any, and collects it.
static msx_status finish_inflight(msx_pool *p)
{
    if (!p->inflight) return MSX_OK;
    p->inflight = false;
    PCUDA(cudaEventSynchronize(p->ev_step));
    return collect(p);
}

static msx_status replay(msx_pool *p, float *ms)
{
    msx_status st;
    if ((st = order_after_uploads(p)) != MSX_OK) return st;
    if ((st = upload_tiles(p)) != MSX_OK) return st;
    if (!p->graph && (st = build_pool_graph(p, p->spl)) != MSX_OK) return st;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, p->stream);
    cudaError_t err = cudaGraphLaunch(p->graph, p->stream);
    cudaEventRecord(b, p->stream);
    cudaError_t err2 = cudaEventSynchronize(b);
    if (ms) cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (err != cudaSuccess || err2 != cudaSuccess)
        return pfail(MSX_ERR_CUDA, std::string("pool replay: ") + cudaGetErrorString(err != cudaSuccess ? err : err2));
    return MSX_OK;
}

// Autotuner: times one replay per candidate schedule on the resident work and
// keeps the fastest.  Candidates differ only in scheduling, so the solves'
// results are the same whichever one runs a step.
static msx_status autotune(msx_pool *p)
{
    const int mode = pool_mode(p->opts.precision);
    const int occ128 = tiled_ctas_per_sm(mode, 128), occ256 = tiled_ctas_per_sm(mode, 256);
    const Sched cands[] = {{128, 512, occ128}, {128, 1024, occ128}, {256, 512, occ256}, {256, 1024, occ256},
                           {256, 2048, occ256}, {256, 4096, occ256}, {256, 1024, std::max(1, occ256 / 2)},
                           {128, 2048, occ128}};
    const int spl = p->spl;
    p->spl = 2;
    double best = 1e300;
    Sched bs = p->sched;
    msx_status st = MSX_OK;
    for (const Sched &c : cands) {
        if (!any_active(p)) break;
        p->sched = c;
        rebuild_tiles(p);
        if (p->graph) {
            cudaGraphExecDestroy(p->graph);
            p->graph = nullptr;
        }
        float ms = 0, tot = 0;
        for (int r = 0; r < 2 && st == MSX_OK; r++) {
            st = replay(p, &ms);
            tot += ms;
        }
        if (st != MSX_OK || (st = collect(p)) != MSX_OK) break;
        if (tot < best) {
            best = tot;
            bs = c;
        }
    }
    p->spl = spl;
    p->sched = bs;
    rebuild_tiles(p);
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    if (st != MSX_OK) return st;
    p->tuned = true;
    if (p->opts.tune_cache) {
        if (FILE *f = fopen(p->opts.tune_cache, "w")) {
            fprintf(f, "%d %d %d\n", bs.threads, bs.tile_elems, bs.ctas_per_sm);
            fclose(f);
        }
    }
    return MSX_OK;
}

// Serving thread: while any solve is resident, launch a replay, wait for it
// without the lock (admissions, polls and fetches go on meanwhile), collect it.
// Sleeps while the pool is empty.  A failure stops the stepping; msx_pool_poll
// and msx_pool_wait report it.
static void serve_loop(msx_pool *p)
{
    cudaSetDevice(p->device);
    std::unique_lock<std::mutex> lk(p->mu);
    while (!p->serve_stop) {
        if (p->serve_status != MSX_OK || !any_active(p)) {
            p->cv_work.wait(lk);
            continue;
        }
        msx_status st = MSX_OK;
        if (!p->tuned) st = autotune(p);
        if (st == MSX_OK && any_active(p)) st = launch_replay(p);
        if (st == MSX_OK && p->inflight) {
            const cudaEvent_t ev = p->ev_step;
            lk.unlock();
            cudaEventSynchronize(ev);   // errors are read again by finish_inflight
            lk.lock();
            st = finish_inflight(p);
        }
        if (st != MSX_OK) {
            p->serve_status = st;
            p->serve_error = msx_last_error();
        }
        p->cv_done.notify_all();
    }
}

static msx_status serve_failure(msx_pool *p) { return pfail(p->serve_status, "pool serving thread: " + p->serve_error); }

// ------------------------------------------------------------------ C ABI
extern "C" msx_status msx_pool_create(const msx_pool_opts *opts, msx_pool **out)
{
    if (!out || !opts) return pfail(MSX_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (opts->precision != MSX_PREC_FP64 && opts->precision != MSX_PREC_MIXED &&
        opts->precision != MSX_PREC_DOUBLE_WORD)
        return pfail(MSX_ERR_ARG, "pool precision must be FP64, MIXED or DOUBLE_WORD");
    if (opts->max_slots < 1 || opts->max_slots > 4096) return pfail(MSX_ERR_ARG, "max_slots must be 1..4096");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return pfail(MSX_ERR_NO_DEVICE, "no CUDA device");
    msx_pool *p = new msx_pool();
    p->opts = *opts;
    cudaGetDevice(&p->device);
    cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device);
    p->spl = opts->steps_per_launch > 0 ? ((opts->steps_per_launch + 1) & ~1) : 32;
    const int pmode = pool_mode(opts->precision);
    p->sched.threads = kStepThreads;
    p->sched.ctas_per_sm = tiled_ctas_per_sm(pmode, kStepThreads);
    if (opts->elems_per_block > 0) {
        p->sched.threads = opts->elems_per_block >= 256 ? 256 : 128;
        p->sched.tile_elems = opts->elems_per_block;
        p->sched.ctas_per_sm = tiled_ctas_per_sm(pmode, p->sched.threads);
        p->tuned = true;
    } else if (opts->tune_cache) {
        if (FILE *f = fopen(opts->tune_cache, "r")) {
            Sched s;
            if (fscanf(f, "%d %d %d", &s.threads, &s.tile_elems, &s.ctas_per_sm) == 3 && s.threads > 0 &&
                s.threads <= kStepThreads && s.tile_elems > 0 && s.ctas_per_sm > 0 &&
                s.ctas_per_sm <= tiled_ctas_per_sm(pmode, s.threads)) {
                p->sched = s;
                p->tuned = true;
            }
            fclose(f);
        }
    }
    p->slots.resize(opts->max_slots);
    auto bail = [&](msx_status st) {
        msx_pool_destroy(p);
        return st;
    };
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->upload, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->fetch, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_upload, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_step, cudaEventDisableTiming) != cudaSuccess)
        return bail(pfail(MSX_ERR_CUDA, "streams"));
    size_t n = opts->max_slots;
    if (cudaMalloc(&p->d_descs, sizeof(Problem) * n) != cudaSuccess || cudaMalloc(&p->d_ctrl, sizeof(Ctrl) * 2 * n) != cudaSuccess ||
        cudaMalloc(&p->d_dtmin, sizeof(unsigned long long) * 4 * n) != cudaSuccess ||
        cudaMalloc(&p->d_flags, sizeof(int) * 2 * n) != cudaSuccess || cudaMalloc(&p->d_counts, sizeof(int) * kTileSched) != cudaSuccess ||
        cudaMallocHost(&p->h_ctrl, sizeof(Ctrl) * 2 * n) != cudaSuccess)
        return bail(pfail(MSX_ERR_OOM, "pool tables"));
    cudaMemset(p->d_ctrl, 0, sizeof(Ctrl) * 2 * n);
    cudaMemset(p->d_counts, 0, sizeof(int) * kTileSched);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    p->budget = opts->hbm_budget_bytes > 0 ? (size_t)opts->hbm_budget_bytes : (size_t)(0.8 * fr);
    *out = p;
    return MSX_OK;
}

extern "C" msx_status msx_pool_destroy(msx_pool *p)
{
    if (!p) return MSX_OK;
    msx_pool_serve(p, 0);
    if (p->upload) cudaStreamSynchronize(p->upload);
    if (p->stream) cudaStreamSynchronize(p->stream);
    if (p->fetch) cudaStreamSynchronize(p->fetch);
    for (Slot &s : p->slots)
        if (s.arena) cudaFree(s.arena);
    for (auto &d : p->done) {   // results never fetched
        if (d.second.arena) cudaFree(d.second.arena);
        if (d.second.ready) cudaEventDestroy(d.second.ready);
    }
    if (p->graph) cudaGraphExecDestroy(p->graph);
    for (void *q : {(void *)p->d_descs, (void *)p->d_ctrl, (void *)p->d_dtmin, (void *)p->d_flags, (void *)p->d_counts,
                    (void *)p->d_etiles, (void *)p->d_ntiles})
        if (q) cudaFree(q);
    if (p->h_ctrl) cudaFreeHost(p->h_ctrl);
    if (p->stream) cudaStreamDestroy(p->stream);
    if (p->upload) cudaStreamDestroy(p->upload);
    if (p->fetch) cudaStreamDestroy(p->fetch);
    for (cudaEvent_t e : {p->ev_upload, p->ev_step})
        if (e) cudaEventDestroy(e);
    delete p;
    return MSX_OK;
}

extern "C" msx_status msx_pool_submit(msx_pool *p, const msx_mesh *mesh, const msx_material *mat, const msx_bc *bcs,
                                      int64_t num_bcs, const msx_solver_opts *o, int64_t *ticket)
{
    if (!p || !mesh || !mat || !o || !ticket) return pfail(MSX_ERR_ARG, "NULL argument");
    const long long nn = mesh->num_nodes, ne = mesh->num_elems;
    if (!mesh->X || !mesh->conn || nn < 4 || ne < 1 || nn >= (1LL << 31) || 4 * ne >= (1LL << 31))
        return pfail(MSX_ERR_ARG, "bad mesh");
    if (num_bcs < 0 || (num_bcs > 0 && !bcs)) return pfail(MSX_ERR_ARG, "bad boundary conditions");
    if (!(o->scale_factor > 0) || !(o->tf >= o->t0) || o->max_steps < 0) return pfail(MSX_ERR_ARG, "bad solver options");
    if (o->max_steps == 0 && !std::isfinite(o->tf)) return pfail(MSX_ERR_ARG, "need max_steps or a finite tf");
    for (long long k = 0; k < 4 * ne; k++)
        if (mesh->conn[k] < 0 || mesh->conn[k] >= nn) return pfail(MSX_ERR_ARG, "connectivity index out of range");
    MatParams mp;
    msx_status st = make_mat(*mat, mp);
    if (st != MSX_OK) return st;
    const int prec = p->opts.precision;
    if (prec == MSX_PREC_DOUBLE_WORD) {   // the range the double-word kernels need (dw_in_range)
        if (!dw_material_ok(mp))
            return pfail(MSX_ERR_ARG, "double-word pool: a material constant lies outside [2^-100, 2^100]");
        for (long long i = 0; i < 3 * nn; i++)
            if (!dw_in_range(mesh->X[i]))
                return pfail(MSX_ERR_ARG, "double-word pool: a nonzero coordinate lies outside [2^-100, 2^100]");
    }
    const bool cnh = prec == MSX_PREC_FP64 && mp.law == 1;   // the FP64 element kernel's F-free path
    const size_t bytes = footprint(nn, ne, num_bcs, prec, cnh);
    {   // cheap early refusal; the slot is taken below, after the host tables
        std::lock_guard<std::mutex> lk(p->mu);
        bool free_slot = false;
        for (const Slot &q : p->slots) free_slot |= !q.active && !q.reserved;
        if (!free_slot || p->used + bytes > p->budget) return pfail(MSX_ERR_BUSY, "pool full (slots or HBM budget)");
    }

    // host tables, without the pool's lock: Dirichlet records (as the
    // single-solve path); the node -> corner lists are built on the device
    BCTables bt;
    {
        std::string err;
        if (build_bc_tables(nn, bcs, num_bcs, o->t0, o->tf, bt, err) != MSX_OK)
            return pfail(MSX_ERR_ARG, "bad boundary condition entry: " + err);
    }

    int slot = -1;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        for (size_t q = 0; q < p->slots.size(); q++)
            if (!p->slots[q].active && !p->slots[q].reserved) {
                slot = (int)q;
                break;
            }
        if (slot < 0 || p->used + bytes > p->budget) return pfail(MSX_ERR_BUSY, "pool full (slots or HBM budget)");
        p->slots[slot].reserved = true;
        p->used += bytes;
    }
    Slot sl;
    sl.nn = nn;
    sl.ne = ne;
    sl.bytes = bytes;
    // Device uploads and set-up kernels, enqueued on the upload stream without
    // the pool's lock: a replay in flight keeps running, and the serving thread
    // can launch the next one meanwhile.  Replays touch only the tiles of
    // active solves, so none reads this slot's arrays or control entries yet.
    auto upload_solve = [&]() -> msx_status {
        if (take_injected_failure(p))
            return pfail(MSX_ERR_OOM, "cudaMallocAsync(solve arena): out of memory (injected failure)");
        PCUDA(cudaMallocAsync(&sl.arena, bytes, p->upload));
        char *q = (char *)sl.arena;
        auto carve = [&](size_t b) {
            char *r = q;
            q += align256(b);
            return (void *)r;
        };
        Problem &P = sl.P;
        memset(&P, 0, sizeof(P));
        P.nn = nn;
        P.ne = ne;
        P.nmat = 1;
        P.mats[0] = mp;
        P.mat = nullptr;
        P.conn = (int4 *)carve(sizeof(int4) * ne);
        P.G = (double *)carve(sizeof(double) * 9 * ne);
        P.wJ = (double *)carve(sizeof(double) * ne);
        P.Lref = (double *)carve(sizeof(double) * ne);
        P.G32 = (float *)carve(sizeof(float) * 9 * ne);
        P.wJ32 = (float *)carve(sizeof(float) * ne);
        P.Lref32 = (float *)carve(sizeof(float) * ne);
        if (prec == MSX_PREC_DOUBLE_WORD) {
            P.G32lo = (float *)carve(sizeof(float) * 9 * ne);
            P.wJ32lo = (float *)carve(sizeof(float) * ne);
        }
        double *X = (double *)carve(sizeof(double) * 3 * nn);
        P.X = X;
        P.u = (double *)carve(sizeof(double) * 3 * nn);
        P.v = (double *)carve(sizeof(double) * 3 * nn);
        P.a = (double *)carve(sizeof(double) * 3 * nn);
        double *mass = (double *)carve(sizeof(double) * nn), *minv = (double *)carve(sizeof(double) * nn);
        P.mass = mass;
        P.minv = minv;
        P.uhl = (float2 *)carve(sizeof(float2) * 3 * nn);
        if (prec == MSX_PREC_FP64) P.u4 = (double *)carve(sizeof(double) * 4 * nn);
        if (cnh) {   // written by the element set-up, as for a single solve
            P.Eref = (double *)carve(sizeof(double) * 9 * ne);
            P.Mg = (double *)carve(sizeof(double) * 6 * ne);
            P.rdetE = (double *)carve(sizeof(double) * ne);
        }
        float2 *minv2 = nullptr;
        if (pair_state(prec)) {
            P.vhl = (float2 *)carve(sizeof(float2) * 3 * nn);
            P.ahl = (float2 *)carve(sizeof(float2) * 3 * nn);
            minv2 = (float2 *)carve(sizeof(float2) * nn);
            P.minv2 = minv2;
        }
        if (prec == MSX_PREC_MIXED) P.fe32 = (float *)carve(sizeof(float) * 16 * ne);
        else P.fe = (double *)carve(sizeof(double) * 12 * ne);
        int *d_ptr = (int *)carve(sizeof(int) * (nn + 1)), *d_inc = (int *)carve(sizeof(int) * 4 * ne);
        int *d_nbc = (int *)carve(sizeof(int) * nn);
        int4 *d_slot = (int4 *)carve(sizeof(int4) * ne);
        const long long nbcn = std::max(1LL, std::min(nn, (long long)num_bcs));
        int2 *d_rec = (int2 *)carve(sizeof(int2) * 3 * nbcn);
        int2 *d_bcn = (int2 *)carve(sizeof(int2) * nbcn);
        BCEntry *d_ent = (BCEntry *)carve(sizeof(BCEntry) * (num_bcs > 0 ? num_bcs : 1));
        if ((size_t)(q - (char *)sl.arena) > bytes)   // the footprint must cover every array carved above
            return pfail(MSX_ERR_CUDA, "internal: solve arena smaller than its arrays");
        P.node_ptr = d_ptr;
        P.node_inc = d_inc;
        P.slot = d_slot;
        P.node_bc = d_nbc;
        P.bc_rec = d_rec;
        P.bcs = d_ent;
        P.ctrl = p->d_ctrl + 2 * slot;
        P.dtmin = p->d_dtmin + 4 * slot;
        P.flags = p->d_flags + 2 * slot;
        P.sf = o->scale_factor;
        P.tf = o->tf;
        // everything on the upload stream: a replay in flight on the main stream
        // keeps running; the next replay waits for ev_upload
        cudaStream_t s = p->upload;
        PCUDA(cudaMemcpyAsync((void *)P.conn, mesh->conn, sizeof(int4) * ne, cudaMemcpyHostToDevice, s));
        PCUDA(cudaMemcpyAsync(X, mesh->X, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
        {
            std::string err;
            const msx_status cst = build_node_csr(P.conn, mesh->conn, ne, nn, d_ptr, d_inc, d_slot, s, err);
            if (cst != MSX_OK) return pfail(cst, err);
        }
        if (!bt.nodes.empty())
            PCUDA(cudaMemcpyAsync(d_bcn, bt.nodes.data(), sizeof(int2) * bt.nodes.size(), cudaMemcpyHostToDevice, s));
        launch_node_bc_scatter(d_nbc, nn, d_bcn, (long long)bt.nodes.size(), s);
        if (!bt.rec.empty())
            PCUDA(cudaMemcpyAsync(d_rec, bt.rec.data(), sizeof(int2) * bt.rec.size(), cudaMemcpyHostToDevice, s));
        if (!bt.ent.empty())
            PCUDA(cudaMemcpyAsync(d_ent, bt.ent.data(), sizeof(BCEntry) * bt.ent.size(), cudaMemcpyHostToDevice, s));
        PCUDA(cudaMemsetAsync(P.u, 0, sizeof(double) * 3 * nn, s));
        PCUDA(cudaMemsetAsync(P.v, 0, sizeof(double) * 3 * nn, s));
        PCUDA(cudaMemsetAsync(P.a, 0, sizeof(double) * 3 * nn, s));
        PCUDA(cudaMemsetAsync(P.uhl, 0, sizeof(float2) * 3 * nn, s));
        if (P.u4) PCUDA(cudaMemsetAsync(P.u4, 0, sizeof(double) * 4 * nn, s));
        if (pair_state(prec)) {
            PCUDA(cudaMemsetAsync(P.vhl, 0, sizeof(float2) * 3 * nn, s));
            PCUDA(cudaMemsetAsync(P.ahl, 0, sizeof(float2) * 3 * nn, s));
        }
        launch_setup_elements(P, X, s);
        launch_setup_mass(P, mass, minv, s);
        if (pair_state(prec)) launch_minv_split(minv, minv2, nn, s);
        // CFL minima (double bits) and the screen's running minima (FP32 bits)
        unsigned long long inf2[4] = {0x7FF0000000000000ULL, 0x7FF0000000000000ULL, 0x7F800000ULL, 0x7F800000ULL};
        PCUDA(cudaMemcpyAsync(P.dtmin, inf2, sizeof(inf2), cudaMemcpyHostToDevice, s));
        launch_initial_cfl(P, nullptr, 0, s);
        launch_initial_cfl(P, nullptr, 1, s);   // u = 0: the deformed CFL equals the undeformed one
        long long limit = o->max_steps > 0 ? o->max_steps : (1LL << 62);
        pool_init_ctrl<<<1, 1, 0, s>>>(P, o->t0, limit);
        PCUDA(cudaGetLastError());
        PCUDA(cudaMemcpyAsync(p->d_descs + slot, &P, sizeof(Problem), cudaMemcpyHostToDevice, s));
        return MSX_OK;
    };
    st = upload_solve();

    std::lock_guard<std::mutex> lk(p->mu);
    if (st == MSX_OK) {
        // recorded under the lock: the next replay launch waits for everything
        // enqueued on the upload stream up to here, this solve's uploads included
        const cudaError_t e = cudaEventRecord(p->ev_upload, p->upload);
        if (e != cudaSuccess) st = pfail(MSX_ERR_CUDA, std::string("admission event: ") + cudaGetErrorString(e));
    }
    if (st != MSX_OK) {
        if (sl.arena) cudaFreeAsync(sl.arena, p->upload);
        p->slots[slot].reserved = false;
        p->used -= bytes;
        return st;
    }
    p->uploads_pending = true;
    sl.active = true;
    sl.ticket = p->next_ticket++;
    sl.submit_ms = now_ms();
    p->slots[slot] = sl;
    rebuild_tiles(p);
    *ticket = sl.ticket;
    if (p->serving) p->cv_work.notify_one();
    return MSX_OK;
}

extern "C" msx_status msx_pool_serve(msx_pool *p, int32_t enabled)
{
    if (!p) return pfail(MSX_ERR_ARG, "NULL pool");
    if (enabled) {
        std::unique_lock<std::mutex> lk(p->mu);
        // a stop in progress on another thread completes first
        p->cv_done.wait(lk, [p] { return !(p->serving && p->serve_stop); });
        if (p->serving) return MSX_OK;
        msx_status st = finish_inflight(p);   // the serving thread starts with no replay in flight
        if (st != MSX_OK) return st;
        p->serve_stop = false;
        p->serve_status = MSX_OK;
        p->serve_error.clear();
        try {
            p->server = std::thread(serve_loop, p);
        } catch (...) {
            return pfail(MSX_ERR_STATE, "cannot start the pool's serving thread");
        }
        p->serving = true;
        return MSX_OK;
    }
    std::thread server;
    {
        std::unique_lock<std::mutex> lk(p->mu);
        if (!p->serving) return MSX_OK;
        if (p->serve_stop) {
            // another thread is stopping it: wait until that thread has joined it
            p->cv_done.wait(lk, [p] { return !p->serving; });
            return p->serve_status == MSX_OK ? MSX_OK : serve_failure(p);
        }
        p->serve_stop = true;
        server = std::move(p->server);   // the one caller that joins the thread
    }
    p->cv_work.notify_all();
    server.join();   // its last replay was collected before it saw the stop
    std::lock_guard<std::mutex> lk(p->mu);
    p->serving = false;
    p->cv_done.notify_all();
    return p->serve_status == MSX_OK ? MSX_OK : serve_failure(p);
}

extern "C" msx_status msx_pool_inject_alloc_failures(msx_pool *p, int32_t count)
{
    if (!p || count < 0) return pfail(MSX_ERR_ARG, "msx_pool_inject_alloc_failures: NULL pool or negative count");
    p->inject_alloc_failures.store(count);
    return MSX_OK;
}

extern "C" msx_status msx_pool_step(msx_pool *p, int64_t steps)
{
    if (!p) return pfail(MSX_ERR_ARG, "NULL pool");
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->serving) return pfail(MSX_ERR_STATE, "the pool's serving thread drives the steps");
    msx_status st;
    if ((st = finish_inflight(p)) != MSX_OK) return st;
    if (!p->tuned && any_active(p) && (st = autotune(p)) != MSX_OK) return st;
    long long reps = steps > 0 ? (steps + p->spl - 1) / p->spl : 1;
    for (long long r = 0; r < reps; r++) {
        if (r > 0 && (st = finish_inflight(p)) != MSX_OK) return st;
        if (!any_active(p)) break;
        if ((st = launch_replay(p)) != MSX_OK) return st;
    }
    return MSX_OK;   // the last replay may still run: collected by the next step, poll or stats
}

extern "C" msx_status msx_pool_stats_get(msx_pool *p, msx_pool_stats *st)
{
    if (!p || !st) return pfail(MSX_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(p->mu);
    msx_status r = finish_inflight(p);
    if (r == MSX_OK) r = collect(p);
    if (r != MSX_OK) return r;
    int act = 0;
    for (const Slot &s : p->slots) act += s.active;
    st->active = act;
    st->finished_unfetched = (int32_t)p->done.size();
    st->threads = p->sched.threads;
    st->tile_elems = p->sched.tile_elems;
    st->ctas_per_sm = p->sched.ctas_per_sm;
    st->steps_per_launch = p->spl;
    st->element_steps = p->elem_steps_finished + p->elem_steps_active;
    st->used_bytes = (int64_t)p->used;
    st->budget_bytes = (int64_t)p->budget;
    return MSX_OK;
}

extern "C" msx_status msx_pool_poll(msx_pool *p, msx_pool_result *results, int32_t max, int32_t *n)
{
    if (!p || !n || (max > 0 && !results)) return pfail(MSX_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(p->mu);
    *n = 0;
    if (p->serving) {
        if (p->serve_status != MSX_OK) return serve_failure(p);
    } else if (p->inflight) {   // never waits: collect only a replay that has finished
        const cudaError_t q = cudaEventQuery(p->ev_step);
        if (q == cudaSuccess) {
            msx_status st = finish_inflight(p);
            if (st != MSX_OK) return st;
        } else if (q == cudaErrorNotReady) {
            cudaGetLastError();   // "not ready" is no error: keep it out of later launch checks
        } else {
            return pfail(MSX_ERR_CUDA, std::string("pool replay: ") + cudaGetErrorString(q));
        }
    }
    int k = 0;
    while (k < max && !p->done_order.empty()) {
        long long t = p->done_order.front();
        p->done_order.pop_front();
        auto it = p->done.find(t);
        if (it == p->done.end()) continue;
        results[k++] = it->second.res;
    }
    *n = k;
    return MSX_OK;
}

extern "C" msx_status msx_pool_wait(msx_pool *p, int64_t ticket, msx_pool_result *result)
{
    if (!p || !result) return pfail(MSX_ERR_ARG, "NULL argument");
    std::unique_lock<std::mutex> lk(p->mu);
    auto resident = [&] {
        for (const Slot &s : p->slots)
            if (s.active && s.ticket == ticket) return true;
        return false;
    };
    msx_status st;
    for (;;) {
        if (!p->serving && (st = finish_inflight(p)) != MSX_OK) return st;
        auto it = p->done.find(ticket);
        if (it != p->done.end()) {
            *result = it->second.res;
            return MSX_OK;
        }
        if (!resident()) return pfail(MSX_ERR_ARG, "unknown or already fetched ticket");
        if (p->serving) {   // the serving thread steps; wake up at each collected replay
            if (p->serve_status != MSX_OK) return serve_failure(p);
            p->cv_done.wait(lk);
            continue;
        }
        if (!p->tuned && (st = autotune(p)) != MSX_OK) return st;
        if ((st = launch_replay(p)) != MSX_OK) return st;
    }
}

extern "C" msx_status msx_pool_fetch(msx_pool *p, int64_t ticket, double *u, double *v, double *a)
{
    if (!p) return pfail(MSX_ERR_ARG, "NULL pool");
    Finished f;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        auto it = p->done.find(ticket);
        if (it == p->done.end()) return pfail(MSX_ERR_STATE, "ticket not finished or already fetched");
        f = it->second;
        p->done.erase(it);
    }
    // copies on the fetch stream without the pool's lock: replays, admissions
    // and polls go on meanwhile
    const size_t bytes = sizeof(double) * 3 * f.nn;
    cudaError_t e = cudaStreamWaitEvent(p->fetch, f.ready, 0);
    if (e == cudaSuccess && u) e = cudaMemcpyAsync(u, f.u, bytes, cudaMemcpyDeviceToHost, p->fetch);
    if (e == cudaSuccess && v) e = cudaMemcpyAsync(v, f.v, bytes, cudaMemcpyDeviceToHost, p->fetch);
    if (e == cudaSuccess && a) e = cudaMemcpyAsync(a, f.a, bytes, cudaMemcpyDeviceToHost, p->fetch);
    const cudaError_t es = cudaStreamSynchronize(p->fetch);
    if (e == cudaSuccess) e = es;
    cudaFreeAsync(f.arena, p->fetch);
    cudaEventDestroy(f.ready);
    {
        std::lock_guard<std::mutex> lk(p->mu);
        p->used -= f.bytes;
    }
    if (e != cudaSuccess) return pfail(MSX_ERR_CUDA, std::string("pool fetch: ") + cudaGetErrorString(e));
    return MSX_OK;
}

