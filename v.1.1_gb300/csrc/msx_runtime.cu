// msx_runtime.cu -- host runtime and C ABI (include/msx.h) of the explicit
// C3D4 step: validation, node->corner CSR, Dirichlet tables, device buffers,
// step-chunk CUDA graphs, state transfer and the cube generator.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/msx.h"
#include "msx_internal.h"

using namespace msx;

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

static msx_status fail(msx_status st, const std::string &msg)
{
    g_last_error = msg;
    return st;
}

#define MSX_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t err_ = (call);                                                              \
        if (err_ != cudaSuccess)                                                                \
            return fail(err_ == cudaErrorMemoryAllocation ? MSX_ERR_OOM : MSX_ERR_CUDA,          \
                        std::string(#call) + ": " + cudaGetErrorString(err_));                   \
    } while (0)

extern "C" const char *msx_last_error(void) { return g_last_error.c_str(); }

void msx::msx_set_error(const char *msg) { g_last_error = msg; }

// ------------------------------------------------------------------ small kernels
namespace {

__global__ void init_block_kernel(Problem p, double t0, long long limit)
{
    // solverExplicit.cpp:165-166: initial dt from the undeformed lengths
    double dt0 = __longlong_as_double((long long)p.dtmin[0]);
    dt0 = dt0 * p.sf;
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

__global__ void split_kernel(const double *u, float2 *uhl, long long n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = u[i];
    float hi = (float)x;
    uhl[i] = make_float2(hi, (float)(x - (double)hi));
}

}  // namespace

// ------------------------------------------------------------------ device buffer helper
template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count)
    {
        n = count;
        return cudaMalloc((void **)&p, sizeof(T) * (count ? count : 1));
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

typedef void (*launch_fn)(const Problem &, int, cudaStream_t);

struct msx_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    Problem P{};
    // owned device storage
    DBuf<int4> conn, slot;
    DBuf<double> G, wJ, Lref, X, u, v, a, mass, minv, fe;
    DBuf<float> G32, wJ32, Lref32, fe32, G32lo, wJ32lo;
    DBuf<float2> uhl, vhl, ahl, minv2;
    DBuf<double> u4;   // plain FP64 mode: node-major copy of u (Problem::u4)
    // plain FP64 mode with a compressible neo-Hookean material: reference
    // edges, gradient metric and 1/det of the reference Jacobian (Problem::Eref, Mg, rdetE)
    DBuf<double> Eref, Mg, rdetE;
    DBuf<unsigned char> mat;
    DBuf<int> node_ptr, node_inc, node_bc;
    DBuf<int2> bc_nodes;   // (node, record) of the nodes with Dirichlet entries
    DBuf<int2> bc_rec;
    DBuf<BCEntry> bcs;
    // Neumann loads: term lists per DOF, nodal-force entries, gravity terms per
    // gravity block, surface faces and their per-step contributions
    DBuf<double> grav_e, grav_n, fcon;
    DBuf<int> ext_ptr;
    DBuf<unsigned> ext_term;
    DBuf<ForceEntry> nfs;
    DBuf<FaceLoad> faces;
    int nfaces = 0;
    bool loads = false;
    DBuf<Ctrl> ctrl;
    DBuf<unsigned long long> dtmin;
    DBuf<int> flags;
    Ctrl *h_ctrl = nullptr;   // pinned [2]
    // solver block
    double t0 = 0, tf = 0, sf = 1;
    long long max_steps = 0;
    int precision = MSX_PREC_FP64;
    int spg = 64;
    bool block_ready = false;
    double last_t = 0;   // time of the last step run (external force of node extraction)
    long long block_steps = 0;
    double dt_init = 0;
    launch_fn node = nullptr, elem = nullptr;   // reference-order kernels (exact mode)
    bool tiled = false;                          // FP64 / mixed: the shared tiled step kernels
    DBuf<Problem> d_desc;
    DBuf<double> act;                    // activation times (element birth), when set
    bool act_enabled = false;
    // artificial viscosity (msx_set_viscosity): kind and parameters; the
    // elements' previous-step F diagonal while bulk viscosity runs
    int visc_kind = MSX_VISC_NONE;
    double visc_c1 = 0, visc_cl = 0, visc_h = 0, visc_c0 = 0;
    DBuf<double> visc_f0;
    DBuf<float> visc_h0;
    DBuf<Tile> d_etiles, d_ntiles;
    int tile_elems = 0;                 // element-tile size of d_etiles
    DBuf<int> d_counts;
    int tgrid = 0, tgrid_node = 0, tthreads = kStepThreads;
    // captured step chunks: `graph` holds spg steps; part[k] (k >= 1) holds 2^k
    // steps and runs a call's remainder, so a call replays at most one idle step
    cudaGraphExec_t graph = nullptr;
    cudaGraphExec_t part[31] = {};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evc[2] = {nullptr, nullptr};
    bool dw_coords_checked = false, dw_coords_ok = false;   // double-word range of the coordinates
    bool u_zero = true;   // u is still the all-zero state msx_create set (no step run, no state set)
};

static void drop_graphs(msx_handle *h);

// ------------------------------------------------------------------ host helpers
// Law parameters of one material (shared by single solves and the pool);
// false for an invalid material.
bool msx::material_params(const msx_material &m, MatParams &o)
{
    if (m.law < 0 || m.law > 3) return false;
    if (!(m.young > 0) || !(m.rho > 0) || !(m.nu > -1.0) || !(m.nu < 0.5)) return false;
    memset(&o, 0, sizeof(o));
    const double E = m.young, nu = m.nu;
    o.law = m.law;
    o.young = E;
    o.nu = nu;
    o.rho = m.rho;
    // hyperElasticNeoHookean.cpp:23-33 / :206-213
    o.lambda = (E * nu) / ((1. + nu) * (1. - 2. * nu));
    o.mu = 0.5 * E / (1. + nu);
    o.K1 = E / (3 * (1 - 2 * nu));
    // hyperElasticStVenantKirchhoff.cpp:68-69
    o.mu2 = E / (1. + nu);
    o.lam_stvk = E * nu / ((1. + nu) * (1. - (2 * nu)));
    // soundSpeed: NH forms :51-54, StVK :50-55, linear elastic linearElastic.cpp:43-48
    o.c = m.law >= 2 ? std::sqrt(E / m.rho) : std::sqrt((o.lambda + 2 * o.mu) / m.rho);
    o.lambda_f = (float)o.lambda;
    o.mu_f = (float)o.mu;
    o.K1_f = (float)o.K1;
    o.mu2_f = (float)o.mu2;
    o.lam_stvk_f = (float)o.lam_stvk;
    o.inv_c_f = (float)(1.0 / o.c);
    o.rho_f = (float)m.rho;
    auto dw = [](double x) { const float hi = (float)x; return make_float2(hi, (float)(x - (double)hi)); };
    o.lambda_w = dw(o.lambda);
    o.mu_w = dw(o.mu);
    o.K1_w = dw(o.K1);
    o.mu2_w = dw(o.mu2);
    o.lam_stvk_w = dw(o.lam_stvk);
    o.mu3_w = dw(o.mu / 3.0);
    return true;
}

bool msx::dw_in_range(double x)
{
    const double a = std::fabs(x);
    return a == 0.0 || (a >= std::ldexp(1.0, -kDwExpLimit) && a <= std::ldexp(1.0, kDwExpLimit));
}

bool msx::dw_material_ok(const MatParams &m)
{
    for (double x : {m.young, m.rho, m.lambda, m.mu, m.K1, m.mu2, m.lam_stvk})
        if (!dw_in_range(x)) return false;
    return true;
}

static msx_status make_material(const msx_material &m, MatParams &o)
{
    if (m.law < 0 || m.law > 3) return fail(MSX_ERR_ARG, "unknown constitutive law");
    if (!material_params(m, o)) return fail(MSX_ERR_ARG, "material needs E > 0, rho > 0, -1 < nu < 0.5");
    return MSX_OK;
}

// Dirichlet tables: entries grouped by DOF in input order, one record per
// constrained node with (first, count) per component.
msx_status msx::build_bc_tables(long long nn, const msx_bc *bcs, long long nbc, double t0, double tf, BCTables &t,
                                std::string &err)
{
    t.nodes.clear();
    t.rec.clear();
    t.ent.clear();
    if (nbc < 0 || (nbc > 0 && !bcs) || nbc >= (1LL << 31)) {
        err = "bad boundary-condition array";
        return MSX_ERR_ARG;
    }
    // key = (3 node + component) << 31 | input index (3 node + component <
    // 3 * 2^31, so the key fits 64 bits): sorting the keys groups the entries
    // by node and component and keeps each DOF's entries in input order
    std::vector<unsigned long long> key(nbc);
    for (long long k = 0; k < nbc; k++) {
        const msx_bc &b = bcs[k];
        if (b.dof < 0 || b.dof >= 3 * nn) err = "BC dof out of range";
        else if (b.mode < 0 || b.mode > 3) err = "unknown BC mode";
        else if (b.mode == MSX_BC_RAMP && !(tf - t0 != 0)) err = "ramp BC needs tf != t0";
        if (!err.empty()) return MSX_ERR_ARG;
        const unsigned long long node = (unsigned long long)(b.dof % nn), comp = (unsigned long long)(b.dof / nn);
        key[k] = ((3 * node + comp) << 31) | (unsigned long long)k;
    }
    std::sort(key.begin(), key.end());
    t.ent.reserve(nbc);
    long long cur = -1;
    for (long long j = 0; j < nbc; j++) {
        const msx_bc &b = bcs[(long long)(key[j] & 0x7FFFFFFFULL)];
        const unsigned long long nc = key[j] >> 31;
        const long long node = (long long)(nc / 3);
        if (node != cur) {
            t.nodes.push_back(make_int2((int)node, (int)(t.rec.size() / 3)));
            t.rec.resize(t.rec.size() + 3, make_int2(0, 0));
            cur = node;
        }
        int2 &r = t.rec[t.rec.size() - 3 + (int)(nc % 3)];
        if (r.y == 0) r.x = (int)t.ent.size();
        r.y++;
        BCEntry e;
        e.mode = b.mode == MSX_BC_RAMP_RATE ? MSX_BC_RAMP : b.mode;
        e.ramp_steps = b.ramp_steps;
        // classNodes.cpp:58-74: a ramp stores U/duration, an instant BC stores U
        e.val = b.mode == MSX_BC_RAMP ? b.value / (tf - t0) : b.value;
        t.ent.push_back(e);
    }
    return MSX_OK;
}

// Bulk viscosity with a nonzero element size changes the forces; the
// deviatoric kind and a zero size add exact zeros, as in the reference.
static bool visc_running(const msx_handle *h) { return h->visc_kind == MSX_VISC_BULK && h->visc_h != 0.0; }

static void bind_problem(msx_handle *h)
{
    Problem &P = h->P;
    P.visc = visc_running(h) ? 1 : 0;
    P.visc_f0 = P.visc ? h->visc_f0.p : nullptr;
    P.visc_h0 = P.visc ? h->visc_h0.p : nullptr;
    P.visc_h = h->visc_h;
    P.visc_c1 = h->visc_c1;
    P.visc_cl = h->visc_cl;
    P.visc_c0 = h->visc_c0;
    P.visc_hf = (float)h->visc_h;
    P.visc_c1sq_hf = (float)(h->visc_c1 * h->visc_c1 * h->visc_h);
    P.visc_clc0f = (float)(h->visc_cl * h->visc_c0);
    P.act_t = h->act_enabled ? h->act.p : nullptr;
    P.conn = h->conn.p;
    P.G = h->G.p;
    P.wJ = h->wJ.p;
    P.Lref = h->Lref.p;
    P.G32 = h->G32.p;
    P.wJ32 = h->wJ32.p;
    P.Lref32 = h->Lref32.p;
    P.G32lo = h->G32lo.p;
    P.wJ32lo = h->wJ32lo.p;
    P.X = h->X.p;
    P.u = h->u.p;
    P.v = h->v.p;
    P.a = h->a.p;
    P.mass = h->mass.p;
    P.minv = h->minv.p;
    P.uhl = h->uhl.p;
    P.u4 = h->precision == MSX_PREC_FP64 ? h->u4.p : nullptr;
    P.Eref = h->precision == MSX_PREC_FP64 ? h->Eref.p : nullptr;
    P.Mg = h->precision == MSX_PREC_FP64 ? h->Mg.p : nullptr;
    P.rdetE = h->precision == MSX_PREC_FP64 ? h->rdetE.p : nullptr;
    P.vhl = h->vhl.p;
    P.ahl = h->ahl.p;
    P.minv2 = h->minv2.p;
    P.fe = h->fe.p;
    P.fe32 = h->fe32.p;
    P.node_ptr = h->node_ptr.p;
    P.node_inc = h->node_inc.p;
    P.slot = h->slot.p;
    P.node_bc = h->node_bc.p;
    P.bc_rec = h->bc_rec.p;
    P.bcs = h->bcs.p;
    P.ext_ptr = h->loads ? h->ext_ptr.p : nullptr;
    P.ext_term = h->ext_term.p;
    P.nfs = h->nfs.p;
    P.grav_e = h->grav_e.p;
    P.grav_n = h->grav_n.p;
    P.fcon = h->fcon.p;
    P.faces = h->faces.p;
    P.nfaces = h->nfaces;
    P.ctrl = h->ctrl.p;
    P.dtmin = h->dtmin.p;
    P.flags = h->flags.p;
    P.sf = h->sf;
    P.tf = h->tf;
}

static msx_status set_mode(msx_handle *h, int precision)
{
    switch (precision) {
    case MSX_PREC_FP64: h->tiled = true; break;
    case MSX_PREC_FP64_EXACT: h->tiled = false; h->node = launch_node_exact; h->elem = launch_elem_exact; break;
    case MSX_PREC_MIXED: h->tiled = true; break;
    case MSX_PREC_DOUBLE_WORD: h->tiled = true; break;
    default: return fail(MSX_ERR_ARG, "unknown precision mode");
    }
    h->precision = precision;
    return MSX_OK;
}

static int tiled_mode(const msx_handle *h)
{
    return h->precision == MSX_PREC_MIXED ? MODE_MIXED : (h->precision == MSX_PREC_DOUBLE_WORD ? MODE_DW : MODE_FP64);
}

// Modes whose running state is the (hi, lo) FP32 pairs uhl, vhl, ahl.
static bool pair_state(const msx_handle *h)
{
    return h->precision == MSX_PREC_MIXED || h->precision == MSX_PREC_DOUBLE_WORD;
}

// One step's kernels: the shared tiled pair for FP64 / mixed (the same
// machine code the pool runs), the reference-order pair for exact mode.
static void launch_step(msx_handle *h, int parity)
{
    if (h->tiled)
        launch_tiled_node(h->d_desc.p, h->d_ntiles.p, h->d_counts.p, tiled_mode(h), parity, h->tgrid_node,
                          h->tthreads, h->stream);
    else
        h->node(h->P, parity, h->stream);
    if (h->nfaces) launch_face_loads(h->P, parity, pair_state(h), h->stream);
    if (h->tiled)
        launch_tiled_elem(h->d_desc.p, h->d_etiles.p, h->d_counts.p, tiled_mode(h), parity, h->tgrid, h->tthreads,
                          h->tile_elems, h->stream, h->P.act_t != nullptr, h->P.visc != 0);
    else
        h->elem(h->P, parity, h->stream);
}

// Descriptor and one-solve tile list of the tiled kernels.
static msx_status upload_tiled(msx_handle *h)
{
    if (!h->tiled) return MSX_OK;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    h->tgrid = sms * tiled_ctas_per_sm(tiled_mode(h), h->tthreads);
    h->tgrid_node = sms * tiled_ctas_per_sm(tiled_mode(h), h->tthreads, true);
    // Element tiles of P whole CTA passes (P * threads elements).  Spread over
    // the grid, the busiest CTA runs ceil(tiles / grid) tiles; P minimises that
    // count times (P + 1/2), the half pass standing for a tile's close (the
    // FP64 and double-word kernels end each tile with block-wide CFL
    // reductions), so the last wave of tiles fills the grid instead of
    // leaving most CTAs idle.  P is capped at 4096 elements for those two
    // kernels and at 1024 for the mixed one, whose tiles balance best small.
    const int thr = h->tthreads;
    const int pmax = (h->precision == MSX_PREC_MIXED ? 1024 : kMaxTileElems) / thr;
    const long long passes = (h->P.ne + thr - 1) / thr;
    int bestp = pmax;
    double best = 1e300;
    for (int P = pmax; P >= 1; P--) {
        const long long rounds = ((passes + P - 1) / P + h->tgrid - 1) / h->tgrid;
        const double cost = (double)rounds * (P + 0.5);
        if (cost < best) {
            best = cost;
            bestp = P;
        }
    }
    const int te = bestp * thr;
    const int tn = 128;
    if (!h->d_desc.p || te != h->tile_elems) {
        std::vector<Tile> et, nt;
        for (long long b = 0; b < h->P.ne; b += te) et.push_back({0, (int)b, (int)std::min<long long>(h->P.ne, b + te)});
        for (long long b = 0; b < h->P.nn; b += tn) nt.push_back({0, (int)b, (int)std::min<long long>(h->P.nn, b + tn)});
        int counts[kTileSched] = {(int)et.size(), 0, 0, (int)nt.size(), 0, 0};
        h->d_etiles.release();
        h->d_ntiles.release();
        if (!h->d_desc.p) MSX_CUDA(h->d_desc.alloc(1));
        MSX_CUDA(h->d_etiles.alloc(et.size()));
        MSX_CUDA(h->d_ntiles.alloc(nt.size()));
        if (!h->d_counts.p) MSX_CUDA(h->d_counts.alloc(kTileSched));
        MSX_CUDA(cudaMemcpyAsync(h->d_etiles.p, et.data(), sizeof(Tile) * et.size(), cudaMemcpyHostToDevice, h->stream));
        MSX_CUDA(cudaMemcpyAsync(h->d_ntiles.p, nt.data(), sizeof(Tile) * nt.size(), cudaMemcpyHostToDevice, h->stream));
        MSX_CUDA(cudaMemcpyAsync(h->d_counts.p, counts, sizeof(counts), cudaMemcpyHostToDevice, h->stream));
        h->tile_elems = te;
        drop_graphs(h);   // the captured launches name the old tile lists
    }
    MSX_CUDA(cudaMemcpyAsync(h->d_desc.p, &h->P, sizeof(Problem), cudaMemcpyHostToDevice, h->stream));
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    return MSX_OK;
}

// The Dirichlet tables on the device (enqueued on the handle's stream; the
// host vectors may go once this returns).
// pieces of the connectivity upload that the element set-up follows (meshes of
// 2^20 elements and more)
constexpr int kSetupChunks = 4;

static msx_status upload_bc_tables(msx_handle *h, const BCTables &t, cudaStream_t strm = nullptr)
{
    if (!strm) strm = h->stream;
    h->bc_rec.release();
    h->bcs.release();
    h->bc_nodes.release();
    if (!h->node_bc.p) MSX_CUDA(h->node_bc.alloc(h->P.nn));
    MSX_CUDA(h->bc_rec.alloc(t.rec.size()));
    MSX_CUDA(h->bcs.alloc(t.ent.size()));
    MSX_CUDA(h->bc_nodes.alloc(t.nodes.size()));
    if (!t.nodes.empty())
        MSX_CUDA(cudaMemcpyAsync(h->bc_nodes.p, t.nodes.data(), sizeof(int2) * t.nodes.size(), cudaMemcpyHostToDevice,
                                 strm));
    launch_node_bc_scatter(h->node_bc.p, h->P.nn, h->bc_nodes.p, (long long)t.nodes.size(), strm);
    if (!t.rec.empty())
        MSX_CUDA(cudaMemcpyAsync(h->bc_rec.p, t.rec.data(), sizeof(int2) * t.rec.size(), cudaMemcpyHostToDevice,
                                 strm));
    if (!t.ent.empty())
        MSX_CUDA(cudaMemcpyAsync(h->bcs.p, t.ent.data(), sizeof(BCEntry) * t.ent.size(), cudaMemcpyHostToDevice,
                                 strm));
    MSX_CUDA(cudaGetLastError());
    return MSX_OK;
}

static msx_status upload_bcs(msx_handle *h, const msx_bc *bcs, long long nbc)
{
    BCTables t;
    std::string err;
    if (build_bc_tables(h->P.nn, bcs, nbc, h->t0, h->tf, t, err) != MSX_OK) return fail(MSX_ERR_ARG, err);
    msx_status st = upload_bc_tables(h, t);
    if (st != MSX_OK) return st;
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    return MSX_OK;
}

// The arrays only some precision modes read, allocated the first time a block
// runs in such a mode (an FP64 handle of the 6M-tet cube saves ~0.5 GB and its
// allocation time): FP32 G and wJ (mixed, double-word), their low words
// (double-word), the (hi, lo) nodal state and 1/m (mixed, double-word), the
// node-major copy of u (plain FP64), and the corner forces as FP64 (or
// double-word) or FP32 slots.  With `fill`, derived arrays
// are converted from the FP64 set-up data (a later block in a new mode); at
// msx_create the set-up kernels fill them.
// A material of the compressible neo-Hookean law (the plain FP64 mode's
// F-free element path).
static bool has_cnh(const msx_handle *h)
{
    for (int k = 0; k < h->P.nmat; k++)
        if (h->P.mats[k].law == 1) return true;
    return false;
}

static msx_status mode_buffers(msx_handle *h, int precision, bool fill, cudaStream_t strm = nullptr)
{
    if (!strm) strm = h->stream;
    const long long ne = h->P.ne, nn = h->P.nn;
    const bool mixed = precision == MSX_PREC_MIXED, dw = precision == MSX_PREC_DOUBLE_WORD;
    float *G32 = nullptr, *wJ32 = nullptr, *G32lo = nullptr, *wJ32lo = nullptr;
    bool minv2 = false;
    if ((mixed || dw) && !h->G32.p) {
        MSX_CUDA(h->G32.alloc(9 * ne));
        MSX_CUDA(h->wJ32.alloc(ne));
        G32 = h->G32.p;
        wJ32 = h->wJ32.p;
    }
    if (dw && !h->G32lo.p) {
        MSX_CUDA(h->G32lo.alloc(9 * ne));
        MSX_CUDA(h->wJ32lo.alloc(ne));
        G32lo = h->G32lo.p;
        wJ32lo = h->wJ32lo.p;
    }
    if ((mixed || dw) && !h->uhl.p) {
        MSX_CUDA(h->uhl.alloc(3 * nn));
        MSX_CUDA(h->vhl.alloc(3 * nn));
        MSX_CUDA(h->ahl.alloc(3 * nn));
        MSX_CUDA(h->minv2.alloc(nn));
        minv2 = true;
    }
    if (mixed && !h->fe32.p) {
        MSX_CUDA(h->fe32.alloc(16 * ne));
        MSX_CUDA(cudaMemsetAsync(h->fe32.p, 0, sizeof(float) * 16 * ne, strm));
    }
    if (precision == MSX_PREC_FP64 && !h->u4.p) MSX_CUDA(h->u4.alloc(4 * nn));   // filled at each block start
    bool cnh = false;
    if (precision == MSX_PREC_FP64 && has_cnh(h) && !h->Eref.p) {
        MSX_CUDA(h->Eref.alloc(9 * ne));
        MSX_CUDA(h->Mg.alloc(6 * ne));
        MSX_CUDA(h->rdetE.alloc(ne));
        cnh = true;
    }
    if (!mixed && !h->fe.p) {
        MSX_CUDA(h->fe.alloc(12 * ne));
        MSX_CUDA(cudaMemsetAsync(h->fe.p, 0, sizeof(double) * 12 * ne, strm));
    }
    bind_problem(h);
    if (fill) {
        if (G32 || G32lo) launch_mode_arrays(h->P, G32, wJ32, G32lo, wJ32lo, h->stream);
        if (cnh) launch_cnh_arrays(h->P, h->stream);
        if (minv2) launch_minv_split(h->minv.p, h->minv2.p, nn, h->stream);
        MSX_CUDA(cudaGetLastError());
        MSX_CUDA(cudaStreamSynchronize(h->stream));
    }
    return MSX_OK;
}

// Inputs of a double-word block (see dw_in_range): the materials, and the
// coordinates through one device reduction (once per handle).
static msx_status check_double_word(msx_handle *h)
{
    for (int k = 0; k < h->P.nmat; k++)
        if (!dw_material_ok(h->P.mats[k]))
            return fail(MSX_ERR_ARG, "double-word mode: a material constant lies outside [2^-100, 2^100]");
    if (!h->dw_coords_checked) {
        DBuf<unsigned long long> mm;
        MSX_CUDA(mm.alloc(2));
        launch_abs_range(h->X.p, 3 * h->P.nn, mm.p, h->stream);
        unsigned long long r[2] = {0, 0};
        cudaError_t e = cudaMemcpyAsync(r, mm.p, sizeof(r), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        mm.release();
        if (e != cudaSuccess) return fail(MSX_ERR_CUDA, std::string("coordinate range: ") + cudaGetErrorString(e));
        double lo, hi;
        memcpy(&lo, &r[0], sizeof lo);
        memcpy(&hi, &r[1], sizeof hi);
        h->dw_coords_ok = (r[0] == ~0ULL || dw_in_range(lo)) && dw_in_range(hi);
        h->dw_coords_checked = true;
    }
    if (!h->dw_coords_ok)
        return fail(MSX_ERR_ARG, "double-word mode: a nonzero coordinate lies outside [2^-100, 2^100]");
    return MSX_OK;
}

static msx_status set_opts(msx_handle *h, const msx_solver_opts *o)
{
    if (!o) return fail(MSX_ERR_ARG, "solver options required");
    if (!(o->scale_factor > 0)) return fail(MSX_ERR_ARG, "scale factor must be > 0");
    if (!(o->tf >= o->t0)) return fail(MSX_ERR_ARG, "need tf >= t0");
    if (o->max_steps < 0) return fail(MSX_ERR_ARG, "max_steps must be >= 0");
    msx_status st = set_mode(h, o->precision);
    if (st != MSX_OK) return st;
    h->t0 = o->t0;
    h->tf = o->tf;
    h->sf = o->scale_factor;
    h->max_steps = o->max_steps;
    int spg = o->steps_per_graph > 0 ? o->steps_per_graph : 64;
    spg = (spg + 1) & ~1;   // even: every replay starts on the same parity
    if (spg != h->spg && h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->spg = spg;
    h->block_ready = false;
    h->block_steps = 0;
    return MSX_OK;
}

// Set-up of one solver block (solverExplicit.cpp:141-177): initial dt from
// the undeformed lengths and the first step's CFL from uK (u when t0 < 1e-12,
// zero otherwise, which is the undeformed value again).
static msx_status init_block(msx_handle *h)
{
    bind_problem(h);
    msx_status tst = upload_tiled(h);
    if (tst != MSX_OK) return tst;
    const Problem &P = h->P;
    // CFL minima (double bits) and the screen's running minima (FP32 bits)
    unsigned long long inf[4] = {0x7FF0000000000000ULL, 0x7FF0000000000000ULL, 0x7F800000ULL, 0x7F800000ULL};
    MSX_CUDA(cudaMemcpyAsync(h->dtmin.p, inf, sizeof(inf), cudaMemcpyHostToDevice, h->stream));
    launch_initial_cfl(P, nullptr, 0, h->stream);
    if (h->t0 < 1E-12 && !h->u_zero) {
        launch_initial_cfl(P, h->u.p, 1, h->stream);
    } else {
        // the undeformed lengths again (u is zero: X + u reproduces X bit for bit, so the
        // deformed inscribed spheres are the reference ones)
        MSX_CUDA(cudaMemcpyAsync(h->dtmin.p + 1, h->dtmin.p, sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                                 h->stream));
    }
    long long limit = h->max_steps > 0 ? h->max_steps : (1LL << 62);
    init_block_kernel<<<1, 1, 0, h->stream>>>(P, h->t0, limit);
    MSX_CUDA(cudaGetLastError());
    if (P.u4) launch_u4_from_u(P.u, P.u4, P.nn, h->stream);   // the element gathers' copy of u
    if (pair_state(h)) {
        launch_state_split(P, h->precision == MSX_PREC_MIXED, h->stream);   // the running state of a mixed or double-word block
        MSX_CUDA(cudaGetLastError());
    }
    if (P.visc) {
        // the Gauss points' previous F at a block start: that of the handed-over state
        launch_visc_init(P, h->u.p, h->stream);
        MSX_CUDA(cudaGetLastError());
    }
    MSX_CUDA(cudaMemcpyAsync(h->h_ctrl, h->ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    h->dt_init = h->h_ctrl[0].dt;
    h->block_ready = true;
    return MSX_OK;
}

// Destroys the captured step chunks (their launches name the tile lists, the
// kernel instantiation and, in the exact mode, the Problem by value).
static void drop_graphs(msx_handle *h)
{
    if (h->graph) cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
    for (auto &g : h->part) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

// Captures `steps` (even) steps into *out: replays start on parity 1 and keep it.
static msx_status build_graph(msx_handle *h, int steps, cudaGraphExec_t *out)
{
    bind_problem(h);
    cudaGraph_t g;
    MSX_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < steps; i++) launch_step(h, (i & 1) ? 0 : 1);
    cudaError_t err = cudaStreamEndCapture(h->stream, &g);
    if (err != cudaSuccess) return fail(MSX_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(err));
    err = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) {
        *out = nullptr;
        return fail(MSX_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(err));
    }
    return MSX_OK;
}

// Reads the latest control slot, applies this call's step cap and resumes a
// block that an earlier cap stopped (tf and errors stay final).
static msx_status arm_block(msx_handle *h, long long max_steps, long long *start_steps)
{
    MSX_CUDA(cudaMemcpyAsync(h->h_ctrl, h->ctrl.p, 2 * sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    Ctrl latest = h->h_ctrl[0];   // replays start on parity 1 and read slot 0
    *start_steps = latest.step;
    long long limit = h->max_steps > 0 ? h->max_steps : (1LL << 62);
    if (max_steps > 0) limit = std::min(limit, latest.step + max_steps);
    bool resume = latest.stop && latest.status == 0 && latest.t < h->tf - 1E-12 && latest.step < limit;
    if (latest.limit != limit || resume) {
        latest.limit = limit;
        if (resume) {
            // the first resumed step reads the CFL min saved when the block stopped
            latest.stop = 0;
            unsigned long long slot1 = latest.pending;
            int zero = 0;
            MSX_CUDA(cudaMemcpyAsync(h->dtmin.p + 1, &slot1, sizeof(slot1), cudaMemcpyHostToDevice, h->stream));
            MSX_CUDA(cudaMemcpyAsync(h->flags.p + 1, &zero, sizeof(zero), cudaMemcpyHostToDevice, h->stream));
        }
        MSX_CUDA(cudaMemcpyAsync(h->ctrl.p, &latest, sizeof(Ctrl), cudaMemcpyHostToDevice, h->stream));
        MSX_CUDA(cudaStreamSynchronize(h->stream));
        h->h_ctrl[0] = latest;
    }
    return MSX_OK;
}

// ------------------------------------------------------------------ C ABI
extern "C" msx_status msx_create(const msx_mesh *mesh, const msx_material *mats, int32_t num_mats,
                                 const msx_bc *bcs, int64_t num_bcs, const msx_solver_opts *opts,
                                 msx_handle **out)
{
    if (!out) return fail(MSX_ERR_ARG, "out handle pointer is NULL");
    *out = nullptr;
    if (!mesh || !mesh->X || !mesh->conn || mesh->num_nodes < 4 || mesh->num_elems < 1)
        return fail(MSX_ERR_ARG, "mesh needs >= 4 nodes, >= 1 element, X and conn");
    if (mesh->num_nodes >= (1LL << 31) || 4 * mesh->num_elems >= (1LL << 31))
        return fail(MSX_ERR_ARG, "mesh too large for 32-bit node/incidence indices");
    if (!mats || num_mats < 1 || num_mats > kMaxMats) return fail(MSX_ERR_ARG, "need 1..16 materials");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(MSX_ERR_NO_DEVICE, "no CUDA device");
    const long long nn = mesh->num_nodes, ne = mesh->num_elems;
    if (mesh->elem_material)
        for (long long e = 0; e < ne; e++)
            if (mesh->elem_material[e] < 0 || mesh->elem_material[e] >= num_mats)
                return fail(MSX_ERR_ARG, "element material id out of range");

    msx_handle *h = new msx_handle();
    // A second stream uploads the mesh (conn in chunks), builds the node lists
    // (they need only conn) and uploads the Dirichlet tables while the element
    // set-up runs chunk by chunk on the handle's stream; its work is
    // synchronised before any exit.
    struct SideStream {
        cudaStream_t s = nullptr;
        cudaEvent_t chunk[kSetupChunks] = {}, lists = nullptr;
        void finish()
        {
            if (s) cudaStreamSynchronize(s);
        }
        ~SideStream()
        {
            finish();
            if (s) cudaStreamDestroy(s);
            for (cudaEvent_t e : chunk)
                if (e) cudaEventDestroy(e);
            if (lists) cudaEventDestroy(lists);
        }
    } side;
    auto bail = [&](msx_status st) {
        side.finish();
        msx_destroy(h);
        return st;
    };
    msx_status st;
    cudaGetDevice(&h->device);
    int cc_major = 0, cc_minor = 0;
    if (cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, h->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&cc_minor, cudaDevAttrComputeCapabilityMinor, h->device) != cudaSuccess ||
        cc_major * 10 + cc_minor != 103) {
        delete h;
        return fail(MSX_ERR_NO_DEVICE, "the library is built for sm_103 (GB300) only");
    }
    h->P.nn = nn;
    h->P.ne = ne;
    h->P.nmat = num_mats;
    for (int k = 0; k < num_mats; k++)
        if ((st = make_material(mats[k], h->P.mats[k])) != MSX_OK) return bail(st);
    if ((st = set_opts(h, opts)) != MSX_OK) return bail(st);
    // The side stream has the greatest priority: the block scheduler then
    // dispatches the short list-building kernels as soon as set-up blocks retire
    // instead of after the set-up grid's last block.
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&side.s, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
        cudaEventCreateWithFlags(&side.lists, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(MSX_ERR_CUDA, "stream creation failed"));
    for (cudaEvent_t &e : side.chunk)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(MSX_ERR_CUDA, "event creation failed"));
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    cudaEventCreateWithFlags(&h->evc[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&h->evc[1], cudaEventDisableTiming);
#define ALLOC(buf, n) \
    if (cudaError_t e_ = buf.alloc(n)) return bail(fail(MSX_ERR_OOM, std::string("device allocation: ") + cudaGetErrorString(e_)))
    ALLOC(h->conn, ne);
    ALLOC(h->X, 3 * nn);
    cudaStream_t s = h->stream;
#define UP(dst, src, bytes, strm) \
    if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, strm) != cudaSuccess) return bail(fail(MSX_ERR_CUDA, "upload failed"))
    // X, then conn in chunks on the side stream; the element set-up (FP64-bound,
    // the longest set-up kernel) of a chunk runs on the handle's stream while
    // the next chunk uploads, and the arrays it writes are allocated while X
    // and the first chunk upload.  The node-list build after the uploads
    // range-checks conn; the set-up kernel skips an element with an
    // out-of-range node id, and msx_create then fails on the check (every exit
    // waits for both streams).
    UP(h->X.p, mesh->X, sizeof(double) * 3 * nn, side.s);
    {
        const int nchunk = ne >= (1LL << 20) ? kSetupChunks : 1;
        const long long csz = (ne + nchunk - 1) / nchunk;
        for (int c = 0; c < nchunk; c++) {
            const long long e0 = c * csz, e1 = std::min(ne, e0 + csz);
            if (e1 <= e0) break;
            UP(h->conn.p + e0, mesh->conn + 4 * e0, sizeof(int4) * (e1 - e0), side.s);
            if (cudaEventRecord(side.chunk[c], side.s) != cudaSuccess)
                return bail(fail(MSX_ERR_CUDA, "stream ordering failed"));
            if (c == 0) {
                // what the set-up writes (with the FP32 copies of G and wJ of a
                // mixed or double-word handle); the rest is allocated while it runs
                ALLOC(h->G, 9 * ne);
                ALLOC(h->wJ, ne);
                ALLOC(h->Lref, ne);
                ALLOC(h->Lref32, ne);
                if (h->precision == MSX_PREC_MIXED || h->precision == MSX_PREC_DOUBLE_WORD) {
                    ALLOC(h->G32, 9 * ne);
                    ALLOC(h->wJ32, ne);
                }
                if (h->precision == MSX_PREC_DOUBLE_WORD) {
                    ALLOC(h->G32lo, 9 * ne);
                    ALLOC(h->wJ32lo, ne);
                }
                if (h->precision == MSX_PREC_FP64 && has_cnh(h)) {
                    ALLOC(h->Eref, 9 * ne);
                    ALLOC(h->Mg, 6 * ne);
                    ALLOC(h->rdetE, ne);
                }
                bind_problem(h);
            }
            if (cudaStreamWaitEvent(s, side.chunk[c], 0) != cudaSuccess)
                return bail(fail(MSX_ERR_CUDA, "stream ordering failed"));
            launch_setup_elements(h->P, h->X.p, s, e0, e1);
        }
    }
    if (cudaMallocHost((void **)&h->h_ctrl, 2 * sizeof(Ctrl)) != cudaSuccess)
        return bail(fail(MSX_ERR_OOM, "pinned control buffer"));
    ALLOC(h->u, 3 * nn);
    ALLOC(h->v, 3 * nn);
    ALLOC(h->a, 3 * nn);
    ALLOC(h->mass, nn);
    ALLOC(h->minv, nn);
    ALLOC(h->slot, ne);
    ALLOC(h->node_ptr, nn + 1);
    ALLOC(h->node_inc, 4 * ne);
    ALLOC(h->ctrl, 2);
    ALLOC(h->dtmin, 4);
    ALLOC(h->flags, 2);
    if (mesh->elem_material && num_mats > 1) ALLOC(h->mat, ne);
#undef ALLOC
    // the rest of the first block's mode's own arrays (zero fills on the side stream)
    if ((st = mode_buffers(h, h->precision, false, side.s)) != MSX_OK) return bail(st);
    bind_problem(h);
    h->P.mat = h->mat.p;
    // the host builds the Dirichlet tables while the set-up runs
    BCTables bt;
    {
        std::string err;
        if (build_bc_tables(nn, bcs, num_bcs, h->t0, h->tf, bt, err) != MSX_OK) return bail(fail(MSX_ERR_ARG, err));
    }
    cudaMemsetAsync(h->u.p, 0, sizeof(double) * 3 * nn, side.s);
    cudaMemsetAsync(h->v.p, 0, sizeof(double) * 3 * nn, side.s);
    cudaMemsetAsync(h->a.p, 0, sizeof(double) * 3 * nn, side.s);
    {   // node -> (element, corner) lists in element order, built on the device
        // (its range check waits for the side stream only)
        std::string err;
        if ((st = build_node_csr(h->conn.p, mesh->conn, ne, nn, h->node_ptr.p, h->node_inc.p, h->slot.p, side.s,
                                 err)) != MSX_OK)
            return bail(fail(st, err.c_str()));
    }
    if ((st = upload_bc_tables(h, bt, side.s)) != MSX_OK) return bail(st);
    // the material ids (pageable: the copy may wait for the side stream's work)
    std::vector<unsigned char> mids;
    if (h->mat.p) {
        mids.resize(ne);
        for (long long e = 0; e < ne; e++) mids[e] = (unsigned char)mesh->elem_material[e];
        UP(h->mat.p, mids.data(), ne, side.s);
    }
#undef UP
    if (cudaEventRecord(side.lists, side.s) != cudaSuccess || cudaStreamWaitEvent(s, side.lists, 0) != cudaSuccess)
        return bail(fail(MSX_ERR_CUDA, "stream ordering failed"));
    launch_setup_mass(h->P, h->mass.p, h->minv.p, s);
    if (h->minv2.p) launch_minv_split(h->minv.p, h->minv2.p, nn, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return bail(fail(MSX_ERR_CUDA, "set-up kernels failed"));
    if (h->precision == MSX_PREC_DOUBLE_WORD && (st = check_double_word(h)) != MSX_OK) return bail(st);
    bind_problem(h);
    *out = h;
    return MSX_OK;
}

extern "C" msx_status msx_destroy(msx_handle *h)
{
    if (!h) return MSX_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graphs(h);
    DBuf<int4> *b4[] = {&h->conn, &h->slot};
    for (auto *b : b4) b->release();
    for (auto *b : {&h->G, &h->wJ, &h->Lref, &h->X, &h->u, &h->v, &h->a, &h->mass, &h->minv, &h->fe}) b->release();
    for (auto *b : {&h->G32, &h->wJ32, &h->Lref32, &h->fe32, &h->G32lo, &h->wJ32lo}) b->release();
    for (auto *b : {&h->uhl, &h->vhl, &h->ahl, &h->minv2}) b->release();
    h->u4.release();
    for (auto *b : {&h->Eref, &h->Mg, &h->rdetE}) b->release();
    h->mat.release();
    for (auto *b : {&h->node_ptr, &h->node_inc, &h->node_bc, &h->flags}) b->release();
    h->bc_rec.release();
    h->bcs.release();
    h->bc_nodes.release();
    h->act.release();
    h->visc_f0.release();
    h->visc_h0.release();
    h->grav_e.release();
    h->grav_n.release();
    h->fcon.release();
    h->ext_ptr.release();
    h->ext_term.release();
    h->nfs.release();
    h->faces.release();
    h->d_desc.release();
    h->d_etiles.release();
    h->d_ntiles.release();
    h->d_counts.release();
    h->ctrl.release();
    h->dtmin.release();
    if (h->h_ctrl) cudaFreeHost(h->h_ctrl);
    for (cudaEvent_t e : {h->ev0, h->ev1, h->evc[0], h->evc[1]})
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return MSX_OK;
}

// Geometry of a face triangle from its three nodes (node-major xyz), in the
// reference's operation order: the one-point rule's weight * |J| and phi
// (classLinearTriangles::defineGPs, spatialDiscretisation/classLinearTriangles.cpp:194-290,
// order 1 of GPsTriangle2DValues, GPsDistribution.cpp:149-155, with the local
// basis of createOrthogonalBasisOnPlane, mathematics/geometry.cpp:363-390) and
// the unit normal (classLinearTriangles::getn0, :19-45).  Host code built
// without FMA contraction, so both hosts produce the reference's bits.
static double norm3(const double *a)
{
    double s = 0;
    for (int i = 0; i < 3; i++) s += a[i] * a[i];
    return std::sqrt(s);
}

static void cross(const double *A, const double *B, double *C)
{
    C[0] = A[1] * B[2] - A[2] * B[1];
    C[1] = A[2] * B[0] - A[0] * B[2];
    C[2] = A[0] * B[1] - A[1] * B[0];
}

static void face_geometry(const double *xyz, double *wabsJ, double *phi, double *n0)
{
    const double *p1 = xyz;
    double a[3], b[3], nrm[3], xh[3], yh[3];
    for (int i = 0; i < 3; i++) {
        a[i] = xyz[3 + i] + (-1.0) * p1[i];
        b[i] = xyz[6 + i] + (-1.0) * p1[i];
    }
    cross(b, a, nrm);
    cross(a, nrm, xh);
    const double magA = norm3(a), magX = norm3(xh);
    for (int i = 0; i < 3; i++) {
        yh[i] = a[i] / magA;
        xh[i] = xh[i] / magX;
    }
    const double map[6] = {xh[0], xh[1], xh[2], yh[0], yh[1], yh[2]};
    double T[9];   // T[r*3 + k]: coordinate r of face node k relative to the first
    for (int k = 0; k < 3; k++)
        for (int r = 0; r < 3; r++) T[r * 3 + k] = xyz[k * 3 + r] + (-1.0) * p1[r];
    double L[6], Jm[4];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 3; j++) {
            L[i * 3 + j] = 0;
            for (int k = 0; k < 3; k++) L[i * 3 + j] += map[i * 3 + k] * T[k * 3 + j];
        }
    const double dN[6] = {-1.0, -1.0, 1.0, 0.0, 0.0, 1.0};   // d phi_k / d xi_j at [k*2 + j]
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            Jm[i * 2 + j] = 0;
            for (int k = 0; k < 3; k++) Jm[i * 2 + j] += L[i * 3 + k] * dN[k * 2 + j];
        }
    const double J = Jm[0] * Jm[3] - Jm[2] * Jm[1];
    *wabsJ = (0.5 * 1.) * std::fabs(J);
    const double x = 0.33333333333333, y = 0.33333333333333;
    phi[0] = -1.0 * x - 1.0 * y + 1.0;
    phi[1] = 1.0 * x;
    phi[2] = 1.0 * y;
    const double *x1 = xyz, *x2 = xyz + 3, *x3 = xyz + 6;
    for (int i = 0; i < 3; i++) {
        const int c1 = i == 0 ? 1 : (i == 1 ? 2 : 0), c2 = i == 0 ? 2 : (i == 1 ? 0 : 1);
        n0[i] = (x2[c1] - x1[c1]) * (x3[c2] - x1[c2]) - (x3[c1] - x1[c1]) * (x2[c2] - x1[c2]);
    }
    const double no = norm3(n0);
    for (int i = 0; i < 3; i++) n0[i] = n0[i] / no;
}

// Face S (1..4) of a tet: classLinearTetrahedra::getSubElement
// (spatialDiscretisation/classLinearTetrahedra.cpp:30-62).
static void tet_face(const int *c, int S, int *t)
{
    if (S == 1) {
        t[0] = c[0]; t[1] = c[1]; t[2] = c[2];
    } else if (S == 2 || S == 3) {
        t[0] = c[S - 2]; t[1] = c[3]; t[2] = c[S - 1];
    } else {
        t[0] = c[0]; t[1] = c[2]; t[2] = c[S - 1];
    }
}

extern "C" msx_status msx_set_load_blocks(msx_handle *h, const msx_load_block *blocks, int64_t num_blocks)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    if (num_blocks < 0 || (num_blocks > 0 && !blocks)) return fail(MSX_ERR_ARG, "bad load block array");
    const long long nn = h->P.nn, ne = h->P.ne;
    const unsigned kMaxIndex = (1u << kExtIndexBits) - 1;
    long long nforce = 0, ngrav = 0, nface = 0, ncon = 0;
    for (long long b = 0; b < num_blocks; b++) {
        const msx_load_block &B = blocks[b];
        if (B.kind == MSX_LOAD_FORCE) {
            if (B.num_forces < 0 || (B.num_forces > 0 && !B.forces)) return fail(MSX_ERR_ARG, "bad nodal force array");
            for (long long k = 0; k < B.num_forces; k++) {
                if (B.forces[k].dof < 0 || B.forces[k].dof >= 3 * nn)
                    return fail(MSX_ERR_ARG, "nodal force dof out of range");
                if (!(B.forces[k].tf - B.forces[k].t0 != 0)) return fail(MSX_ERR_ARG, "nodal force needs tf != t0");
            }
            nforce += B.num_forces;
        } else if (B.kind == MSX_LOAD_GRAVITY) {
            if (!std::isfinite(B.value[0])) return fail(MSX_ERR_ARG, "gravity must be finite");
            ngrav++;
        } else if (B.kind >= MSX_LOAD_TRACTION_INST && B.kind <= MSX_LOAD_PRESSURE_RAMP) {
            if (B.face < 1 || B.face > 4) return fail(MSX_ERR_ARG, "surface load face must be 1..4");
            if (B.num_elems < 0 || (B.num_elems > 0 && !B.elems)) return fail(MSX_ERR_ARG, "bad surface element list");
            if ((B.kind == MSX_LOAD_TRACTION_RAMP || B.kind == MSX_LOAD_PRESSURE_RAMP) && !(B.tf - B.t0 != 0))
                return fail(MSX_ERR_ARG, "ramped surface load needs tf != t0");
            for (long long k = 0; k < B.num_elems; k++)
                if (B.elems[k] < 0 || B.elems[k] >= ne) return fail(MSX_ERR_ARG, "surface load element out of range");
            nface += B.num_elems;
            ncon += B.num_elems * (B.kind == MSX_LOAD_PRESSURE_RAMP ? 1 : 3);
        } else {
            return fail(MSX_ERR_ARG, "unknown load block kind");
        }
    }
    if (nforce > kMaxIndex || ngrav * std::max(nn, ne) > kMaxIndex || 3 * ncon > kMaxIndex)
        return fail(MSX_ERR_ARG, "too many load terms");

    // host copies of the mesh and the node -> (element, corner) incidences
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    std::vector<double> X(3 * nn);
    std::vector<int4> conn(ne);
    std::vector<int> ptr(nn + 1), inc(4 * ne);
    MSX_CUDA(cudaMemcpy(X.data(), h->X.p, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost));
    MSX_CUDA(cudaMemcpy(conn.data(), h->conn.p, sizeof(int4) * ne, cudaMemcpyDeviceToHost));
    MSX_CUDA(cudaMemcpy(ptr.data(), h->node_ptr.p, sizeof(int) * (nn + 1), cudaMemcpyDeviceToHost));
    MSX_CUDA(cudaMemcpy(inc.data(), h->node_inc.p, sizeof(int) * 4 * ne, cudaMemcpyDeviceToHost));

    // nodal-force entries, faces, and each DOF's terms in deck order (two passes:
    // count, then fill).  A gravity block contributes its per-node sum when it is
    // the first term of the z DOF, else its element terms in element order.
    std::vector<ForceEntry> ents;
    std::vector<FaceLoad> faces;
    std::vector<int> cnt(3 * nn + 1, 0), pos;
    std::vector<unsigned> terms;
    for (int pass = 0; pass < 2; pass++) {
        std::vector<char> touched(3 * nn, 0);
        long long fk = 0, gb = 0, con = 0;
        auto emit = [&](long long dof, unsigned kind, unsigned idx) {
            if (pass == 0) cnt[dof]++;
            else terms[pos[dof]++] = (kind << kExtIndexBits) | idx;
            touched[dof] = 1;
        };
        for (long long b = 0; b < num_blocks; b++) {
            const msx_load_block &B = blocks[b];
            if (B.kind == MSX_LOAD_FORCE) {
                for (long long k = 0; k < B.num_forces; k++, fk++) {
                    const msx_nodal_force &f = B.forces[k];
                    if (pass == 0) ents.push_back({f.value / (f.tf - f.t0), f.t0, f.tf});
                    emit(f.dof, EXT_FORCE, (unsigned)fk);
                }
            } else if (B.kind == MSX_LOAD_GRAVITY) {
                for (long long i = 0; i < nn; i++) {
                    const long long dof = i + 2 * nn;
                    if (!touched[dof]) {
                        emit(dof, EXT_GRAV_NODE, (unsigned)(gb * nn + i));
                    } else {
                        for (int k = ptr[i]; k < ptr[i + 1]; k++)
                            emit(dof, EXT_GRAV_ELEM, (unsigned)(gb * ne + (inc[k] >> 2)));
                    }
                }
                gb++;
            } else {
                const bool pramp = B.kind == MSX_LOAD_PRESSURE_RAMP;
                for (long long k = 0; k < B.num_elems; k++) {
                    const int e = B.elems[k];
                    const int c[4] = {conn[e].x, conn[e].y, conn[e].z, conn[e].w};
                    FaceLoad F{};
                    F.kind = B.kind;
                    F.tet = e;
                    F.con = (int)con;
                    F.t0 = B.t0;
                    F.tf = B.tf;
                    for (int i = 0; i < 3; i++) F.value[i] = B.value[i];
                    int tri[3];
                    tet_face(c, B.face, tri);
                    if (pass == 0) {
                        double xyz[9];
                        for (int a = 0; a < 3; a++)
                            for (int i = 0; i < 3; i++) xyz[a * 3 + i] = X[i * nn + tri[a]];
                        face_geometry(xyz, &F.wabsJ, F.phi, F.n0);
                    }
                    const int nc = pramp ? 1 : 3;
                    for (int a = 0; a < 3; a++) F.node[a] = pramp ? c[0] : tri[a];
                    for (int a = 0; a < nc; a++)
                        for (int i = 0; i < 3; i++) emit(F.node[a] + i * nn, EXT_FACE, (unsigned)((con + a) * 3 + i));
                    if (pass == 0) faces.push_back(F);
                    con += nc;
                }
            }
        }
        if (pass == 0) {
            pos.assign(3 * nn + 1, 0);
            for (long long d = 0; d < 3 * nn; d++) pos[d + 1] = pos[d] + cnt[d];
            cnt.assign(pos.begin(), pos.end());   // cnt now holds the row starts
            terms.resize(pos[3 * nn]);
        }
    }

    for (auto *b : {&h->grav_e, &h->grav_n, &h->fcon}) b->release();
    h->ext_ptr.release();
    h->ext_term.release();
    h->nfs.release();
    h->faces.release();
    h->nfaces = 0;
    h->loads = !terms.empty();
    if (h->loads) {
        MSX_CUDA(h->ext_ptr.alloc(3 * nn + 1));
        MSX_CUDA(h->ext_term.alloc(terms.size()));
        MSX_CUDA(cudaMemcpyAsync(h->ext_ptr.p, cnt.data(), sizeof(int) * (3 * nn + 1), cudaMemcpyHostToDevice, h->stream));
        MSX_CUDA(cudaMemcpyAsync(h->ext_term.p, terms.data(), sizeof(unsigned) * terms.size(), cudaMemcpyHostToDevice,
                                 h->stream));
    }
    if (!ents.empty()) {
        MSX_CUDA(h->nfs.alloc(ents.size()));
        MSX_CUDA(cudaMemcpyAsync(h->nfs.p, ents.data(), sizeof(ForceEntry) * ents.size(), cudaMemcpyHostToDevice,
                                 h->stream));
    }
    if (ngrav > 0) {
        MSX_CUDA(h->grav_e.alloc(ngrav * ne));
        MSX_CUDA(h->grav_n.alloc(ngrav * nn));
        bind_problem(h);
        long long gb = 0;
        for (long long b = 0; b < num_blocks; b++)
            if (blocks[b].kind == MSX_LOAD_GRAVITY) {
                launch_setup_gravity(h->P, blocks[b].value[0], h->grav_e.p + gb * ne, h->grav_n.p + gb * nn, h->stream);
                gb++;
            }
    }
    if (!faces.empty()) {
        MSX_CUDA(h->faces.alloc(faces.size()));
        MSX_CUDA(h->fcon.alloc(3 * ncon));
        MSX_CUDA(cudaMemcpyAsync(h->faces.p, faces.data(), sizeof(FaceLoad) * faces.size(), cudaMemcpyHostToDevice,
                                 h->stream));
        MSX_CUDA(cudaMemsetAsync(h->fcon.p, 0, sizeof(double) * 3 * ncon, h->stream));
        h->nfaces = (int)faces.size();
    }
    bind_problem(h);
    msx_status st = upload_tiled(h);
    if (st != MSX_OK) return st;
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    drop_graphs(h);   // the step's kernel list (face kernel) and the exact mode's Problem changed
    return MSX_OK;
}

extern "C" msx_status msx_set_activation(msx_handle *h, const double *activation_time, int32_t enabled)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    if (activation_time) {
        if (!h->act.p) MSX_CUDA(h->act.alloc(h->P.ne));
        MSX_CUDA(cudaMemcpyAsync(h->act.p, activation_time, sizeof(double) * h->P.ne, cudaMemcpyHostToDevice,
                                 h->stream));
    }
    if (enabled && !h->act.p) return fail(MSX_ERR_STATE, "activation enabled before any activation times were set");
    if (enabled && visc_running(h))
        return fail(MSX_ERR_STATE, "element birth and bulk viscosity together are not supported");
    h->act_enabled = enabled != 0;
    bind_problem(h);
    msx_status st = upload_tiled(h);
    if (st != MSX_OK) return st;
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    drop_graphs(h);   // the exact mode's captured launches hold the Problem by value
    return MSX_OK;
}

extern "C" msx_status msx_set_viscosity(msx_handle *h, int32_t kind, double c1, double cl, double element_size,
                                        double c0)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    if (kind < MSX_VISC_NONE || kind > MSX_VISC_DEV) return fail(MSX_ERR_ARG, "unknown artificial viscosity kind");
    if (!std::isfinite(c1) || !std::isfinite(cl) || !std::isfinite(element_size) || !std::isfinite(c0) ||
        element_size < 0)
        return fail(MSX_ERR_ARG, "viscosity parameters must be finite and the element size >= 0");
    const bool was = visc_running(h);
    const bool on = kind == MSX_VISC_BULK && element_size != 0.0;
    if (on && h->act_enabled) return fail(MSX_ERR_STATE, "element birth and bulk viscosity together are not supported");
    if (on && !h->visc_f0.p) {
        MSX_CUDA(h->visc_f0.alloc(3 * h->P.ne));
        MSX_CUDA(h->visc_h0.alloc(3 * h->P.ne));
    }
    h->visc_kind = kind;
    h->visc_c1 = c1;
    h->visc_cl = cl;
    h->visc_h = element_size;
    h->visc_c0 = c0;
    bind_problem(h);
    if (on && !was) {
        // from here on the previous step's F is that of the current state
        launch_visc_init(h->P, h->u.p, h->stream);
        MSX_CUDA(cudaGetLastError());
    }
    msx_status st = upload_tiled(h);
    if (st != MSX_OK) return st;
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    drop_graphs(h);   // another element-kernel instantiation, and the exact mode's launches hold the Problem
    return MSX_OK;
}

extern "C" msx_status msx_set_loads(msx_handle *h, const msx_nodal_force *forces, int64_t num_forces, double gravity,
                                    int32_t gravity_first)
{
    msx_load_block B[2] = {};
    msx_load_block f{}, g{};
    f.kind = MSX_LOAD_FORCE;
    f.forces = forces;
    f.num_forces = num_forces;
    g.kind = MSX_LOAD_GRAVITY;
    g.value[0] = gravity;
    int n = 0;
    if (gravity_first && gravity != 0) B[n++] = g;
    if (num_forces != 0) B[n++] = f;
    if (!gravity_first && gravity != 0) B[n++] = g;
    if (!std::isfinite(gravity)) return fail(MSX_ERR_ARG, "gravity must be finite");
    return msx_set_load_blocks(h, B, n);
}

extern "C" msx_status msx_run(msx_handle *h, int64_t max_steps, msx_run_report *rep)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    msx_status st;
    if (!h->block_ready && (st = init_block(h)) != MSX_OK) return st;
    long long start_steps = 0;
    if ((st = arm_block(h, max_steps, &start_steps)) != MSX_OK) return st;
    Ctrl latest = h->h_ctrl[0];
    // replays needed to reach the step limit (time may end the block sooner): the
    // limit's last step is post-updated, and the stop raised, by one more node
    // kernel, so room + 1 node kernels in all
    const long long room = latest.limit - latest.step;
    // Full chunks of steps_per_graph steps, then the remainder (rounded up to
    // even) as power-of-two chunks, largest first; an open-ended block
    // replays full chunks until the device raises the stop.
    const bool open = room >= (1LL << 61);
    long long full = open ? (1LL << 62) : (room + 1) / h->spg;
    long long rest = open ? 0 : ((room + 1 - full * h->spg) + 1) & ~1LL;
    if (rest >= h->spg) {
        full++;
        rest = 0;
    }
    int parts[31], nparts = 0;
    for (int b = 30; b >= 1; b--)
        if (rest & (1LL << b)) parts[nparts++] = b;
    if (full == 0 && nparts == 0) parts[nparts++] = 1;   // a stopped block: one short replay reports it
    const long long needed = full + nparts;
    MSX_CUDA(cudaEventRecord(h->ev0, h->stream));
    // two replays in flight: check the older one's control slot
    long long k = 0, replayed = 0;
    for (;; k++) {
        const bool whole = k < full;
        const int n = whole ? h->spg : 1 << parts[k - full];
        cudaGraphExec_t *gx = whole ? &h->graph : &h->part[parts[k - full]];
        // A chunk whose graph is not captured yet is launched step by step, and
        // its graph captured while the device runs it: the first call of a
        // handle does not wait for the captures.
        const bool direct = !*gx;
        if (direct) {
            bind_problem(h);
            for (int i = 0; i < n; i++) launch_step(h, (i & 1) ? 0 : 1);
        } else
            MSX_CUDA(cudaGraphLaunch(*gx, h->stream));
        MSX_CUDA(cudaGetLastError());
        replayed += n;
        MSX_CUDA(cudaMemcpyAsync(h->h_ctrl + (k & 1), h->ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
        MSX_CUDA(cudaEventRecord(h->evc[k & 1], h->stream));
        if (direct && (st = build_graph(h, n, gx)) != MSX_OK) {
            cudaStreamSynchronize(h->stream);
            return st;
        }
        if (latest.stop || k + 1 >= needed) break;
        if (k >= 1) {
            MSX_CUDA(cudaEventSynchronize(h->evc[(k - 1) & 1]));
            if (h->h_ctrl[(k - 1) & 1].stop) break;
        }
    }
    if (pair_state(h)) launch_state_merge(h->P, h->precision == MSX_PREC_MIXED, h->stream);   // u, v, a for the caller
    MSX_CUDA(cudaEventRecord(h->ev1, h->stream));
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    Ctrl fin = h->h_ctrl[k & 1];
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->block_steps = fin.step;
    h->last_t = fin.t;
    if (fin.step > 0) h->u_zero = false;
    if (rep) {
        rep->steps = fin.step - start_steps;
        rep->total_steps = fin.step;
        rep->t = fin.t;
        rep->dt = fin.dt;
        rep->dt_init = h->dt_init;
        rep->status = fin.status;
        rep->device_ms = ms;
        rep->kernel_launches = 2 * replayed;
    }
    if (fin.status == MSX_ERR_NEG_JACOBIAN) return fail(MSX_ERR_NEG_JACOBIAN, "Negative jacobian: dt < 1e-20");
    if (fin.status == MSX_ERR_NAN) return fail(MSX_ERR_NAN, "There are NANs in the displacements");
    return MSX_OK;
}

extern "C" msx_status msx_node_values(msx_handle *h, int32_t field, int32_t comp, const int32_t *nodes, int64_t n,
                                      double *out)
{
    if (!h || n < 0 || (n > 0 && (!nodes || !out))) return fail(MSX_ERR_ARG, "bad node value arguments");
    if (field < MSX_FIELD_DISPLACEMENT || field > MSX_FIELD_INTERNAL_FORCE || comp < 0 || comp > 2)
        return fail(MSX_ERR_ARG, "field must be a msx_node_field, comp 0..2");
    for (int64_t k = 0; k < n; k++)
        if (nodes[k] < 0 || nodes[k] >= h->P.nn) return fail(MSX_ERR_ARG, "node index out of range");
    if (n == 0) return MSX_OK;
    DBuf<int> dn;
    DBuf<double> dv;
    if (dn.alloc(n) != cudaSuccess || dv.alloc(n) != cudaSuccess) {
        dn.release();
        dv.release();
        return fail(MSX_ERR_OOM, "node value scratch");
    }
    bind_problem(h);
    const int mode = h->precision == MSX_PREC_FP64_EXACT ? MODE_EXACT : tiled_mode(h);
    cudaMemcpyAsync(dn.p, nodes, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream);
    launch_node_values(h->P, mode, field, comp, dn.p, n, h->last_t, dv.p, h->stream);
    cudaMemcpyAsync(out, dv.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t err = cudaStreamSynchronize(h->stream);
    dn.release();
    dv.release();
    if (err != cudaSuccess) return fail(MSX_ERR_CUDA, cudaGetErrorString(err));
    return MSX_OK;
}

// Shared checks of the element-extraction calls: the quantity, and the element
// list (NULL = all) copied to the device; n becomes the number of entries.
static msx_status element_list(msx_handle *h, int32_t quantity, const int32_t *elems, int64_t &n, DBuf<int> &de)
{
    if (quantity < MSX_ELEM_FXX || quantity > MSX_ELEM_VOLUME)
        return fail(MSX_ERR_ARG, "quantity must be a msx_element_quantity");
    if (!elems) {
        n = h->P.ne;
        return MSX_OK;
    }
    if (n < 0) return fail(MSX_ERR_ARG, "negative element count");
    for (int64_t k = 0; k < n; k++)
        if (elems[k] < 0 || elems[k] >= h->P.ne) return fail(MSX_ERR_ARG, "element index out of range");
    if (n == 0) return MSX_OK;
    if (de.alloc(n) != cudaSuccess) return fail(MSX_ERR_OOM, "element list scratch");
    cudaMemcpyAsync(de.p, elems, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream);
    return MSX_OK;
}

extern "C" msx_status msx_element_values(msx_handle *h, int32_t quantity, const int32_t *elems, int64_t n, double *out)
{
    if (!h || !out) return fail(MSX_ERR_ARG, "bad element value arguments");
    if (quantity == MSX_ELEM_EXTERNAL_ENERGY) return fail(MSX_ERR_ARG, "EXTERNAL_ENERGY has no per-element value");
    DBuf<int> de;
    DBuf<double> dv;
    msx_status st = element_list(h, quantity, elems, n, de);
    if (st != MSX_OK || n == 0) {
        de.release();
        return st;
    }
    if (dv.alloc(n) != cudaSuccess) {
        de.release();
        return fail(MSX_ERR_OOM, "element value scratch");
    }
    bind_problem(h);
    launch_element_values(h->P, quantity, elems ? de.p : nullptr, n, h->last_t, dv.p, h->stream);
    cudaMemcpyAsync(out, dv.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t err = cudaStreamSynchronize(h->stream);
    de.release();
    dv.release();
    if (err != cudaSuccess) return fail(MSX_ERR_CUDA, cudaGetErrorString(err));
    return MSX_OK;
}

extern "C" msx_status msx_element_reduce(msx_handle *h, int32_t quantity, int32_t op, const int32_t *elems, int64_t n,
                                         double *value)
{
    if (!h || !value) return fail(MSX_ERR_ARG, "bad element reduce arguments");
    if (op < MSX_OP_MEAN || op > MSX_OP_SUM) return fail(MSX_ERR_ARG, "op must be a msx_element_op");
    if (quantity == MSX_ELEM_VOLUME && op == MSX_OP_MEAN)
        return fail(MSX_ERR_ARG, "VOLUME has no Mean (the reference's volume() returns no value for it)");
    if (elems && n == 0) return fail(MSX_ERR_ARG, "empty element list");
    // each listed element once, in element order: the reference's selection
    std::vector<int32_t> set;
    if (elems && n > 0) {
        set.assign(elems, elems + n);
        std::sort(set.begin(), set.end());
        set.erase(std::unique(set.begin(), set.end()), set.end());
        n = (int64_t)set.size();
    }
    DBuf<int> de;
    DBuf<double> scratch;
    msx_status st = element_list(h, quantity, elems ? set.data() : nullptr, n, de);
    if (st != MSX_OK) {
        de.release();
        return st;
    }
    if (quantity == MSX_ELEM_EXTERNAL_ENERGY) {   // u . f_ext over every DOF, whatever the operation
        n = 3 * h->P.nn;
        op = MSX_OP_SUM;
    }
    if (scratch.alloc(element_reduce_scratch()) != cudaSuccess) {
        de.release();
        return fail(MSX_ERR_OOM, "element reduce scratch");
    }
    bind_problem(h);
    double *out = scratch.p + element_reduce_scratch() - 1;
    launch_element_reduce(h->P, quantity, op, elems ? de.p : nullptr, n, h->last_t, scratch.p, out, h->stream);
    cudaMemcpyAsync(value, out, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t err = cudaStreamSynchronize(h->stream);
    de.release();
    scratch.release();
    if (err != cudaSuccess) return fail(MSX_ERR_CUDA, cudaGetErrorString(err));
    return MSX_OK;
}

extern "C" msx_status msx_get_state(msx_handle *h, double *u, double *v, double *a)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    size_t bytes = sizeof(double) * 3 * h->P.nn;
    if (u) MSX_CUDA(cudaMemcpyAsync(u, h->u.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    if (v) MSX_CUDA(cudaMemcpyAsync(v, h->v.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    if (a) MSX_CUDA(cudaMemcpyAsync(a, h->a.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    return MSX_OK;
}

extern "C" msx_status msx_set_state(msx_handle *h, const double *u, const double *v, const double *a)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    if (h->block_steps > 0) return fail(MSX_ERR_STATE, "state can only be set before a block's first step");
    size_t bytes = sizeof(double) * 3 * h->P.nn;
    if (u) {
        MSX_CUDA(cudaMemcpyAsync(h->u.p, u, bytes, cudaMemcpyHostToDevice, h->stream));
        h->u_zero = false;
    }
    if (v) MSX_CUDA(cudaMemcpyAsync(h->v.p, v, bytes, cudaMemcpyHostToDevice, h->stream));
    if (a) MSX_CUDA(cudaMemcpyAsync(h->a.p, a, bytes, cudaMemcpyHostToDevice, h->stream));
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    h->block_ready = false;
    return MSX_OK;
}

extern "C" msx_status msx_next_solver(msx_handle *h, const msx_bc *bcs, int64_t num_bcs, const msx_solver_opts *opts)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    msx_status st;
    if (opts && opts->precision == MSX_PREC_DOUBLE_WORD && (st = check_double_word(h)) != MSX_OK) return st;
    if ((st = set_opts(h, opts)) != MSX_OK) return st;
    if ((st = mode_buffers(h, h->precision, true)) != MSX_OK) return st;
    if ((st = upload_bcs(h, bcs, num_bcs)) != MSX_OK) return st;
    drop_graphs(h);
    return MSX_OK;
}

extern "C" msx_status msx_internal_force(msx_handle *h, const double *u, double *fint)
{
    if (!h || !u || !fint) return fail(MSX_ERR_ARG, "NULL argument");
    size_t bytes = sizeof(double) * 3 * h->P.nn;
    DBuf<double> du, df;
    if (du.alloc(3 * h->P.nn) != cudaSuccess || df.alloc(3 * h->P.nn) != cudaSuccess) {
        du.release();
        df.release();
        return fail(MSX_ERR_OOM, "scratch for internal force");
    }
    bind_problem(h);
    Problem P = h->P;
    P.u = du.p;
    cudaMemcpyAsync(du.p, u, bytes, cudaMemcpyHostToDevice, h->stream);
    DBuf<float2> uh;   // the mixed and double-word kernels read u as (hi, lo) pairs; the block's own stay untouched
    if (pair_state(h)) {
        if (uh.alloc(3 * h->P.nn) != cudaSuccess) {
            du.release();
            df.release();
            return fail(MSX_ERR_OOM, "scratch for internal force");
        }
        long long n = 3 * P.nn;
        P.uhl = uh.p;
        split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(du.p, P.uhl, n);
    }
    if (h->precision == MSX_PREC_FP64_EXACT) launch_internal_force_exact(P, df.p, h->stream);
    else if (h->precision == MSX_PREC_MIXED) launch_internal_force_mixed(P, df.p, h->stream);
    else if (h->precision == MSX_PREC_DOUBLE_WORD) launch_internal_force_dw(P, df.p, h->stream);
    else launch_internal_force_fp64(P, df.p, h->stream);
    cudaMemcpyAsync(fint, df.p, bytes, cudaMemcpyDeviceToHost, h->stream);
    cudaError_t err = cudaStreamSynchronize(h->stream);
    du.release();
    df.release();
    uh.release();
    if (err != cudaSuccess) return fail(MSX_ERR_CUDA, cudaGetErrorString(err));
    return MSX_OK;
}

extern "C" msx_status msx_get_element_data(msx_handle *h, double *G, double *wJ, double *Lref, double *mass)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    const long long ne = h->P.ne, nn = h->P.nn;
    if (G) MSX_CUDA(cudaMemcpyAsync(G, h->G.p, sizeof(double) * 9 * ne, cudaMemcpyDeviceToHost, h->stream));
    if (wJ) MSX_CUDA(cudaMemcpyAsync(wJ, h->wJ.p, sizeof(double) * ne, cudaMemcpyDeviceToHost, h->stream));
    if (Lref) MSX_CUDA(cudaMemcpyAsync(Lref, h->Lref.p, sizeof(double) * ne, cudaMemcpyDeviceToHost, h->stream));
    if (mass) MSX_CUDA(cudaMemcpyAsync(mass, h->mass.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, h->stream));
    MSX_CUDA(cudaStreamSynchronize(h->stream));
    return MSX_OK;
}

extern "C" msx_status msx_profile(msx_handle *h, int64_t steps, msx_profile_report *rep)
{
    if (!h || !rep || steps < 1) return fail(MSX_ERR_ARG, "bad profile arguments");
    msx_status st;
    if (!h->block_ready && (st = init_block(h)) != MSX_OK) return st;
    long long start_steps = 0;
    // replays start on parity 1: launch an even number of steps from parity 1
    long long n = (steps + 1) & ~1LL;
    if ((st = arm_block(h, n, &start_steps)) != MSX_OK) return st;
    bind_problem(h);
    std::vector<cudaEvent_t> ev(3 * n);
    for (auto &e : ev) cudaEventCreate(&e);
    for (long long i = 0; i < n; i++) {
        int parity = (i & 1) ? 0 : 1;
        cudaEventRecord(ev[3 * i], h->stream);
        if (h->tiled)
            launch_tiled_node(h->d_desc.p, h->d_ntiles.p, h->d_counts.p, tiled_mode(h), parity, h->tgrid_node,
                              h->tthreads, h->stream);
        else
            h->node(h->P, parity, h->stream);
        if (h->nfaces) launch_face_loads(h->P, parity, pair_state(h), h->stream);
        cudaEventRecord(ev[3 * i + 1], h->stream);
        if (h->tiled)
            launch_tiled_elem(h->d_desc.p, h->d_etiles.p, h->d_counts.p, tiled_mode(h), parity, h->tgrid, h->tthreads,
                              h->tile_elems, h->stream, h->P.act_t != nullptr, h->P.visc != 0);
        else
            h->elem(h->P, parity, h->stream);
        cudaEventRecord(ev[3 * i + 2], h->stream);
    }
    if (pair_state(h)) launch_state_merge(h->P, h->precision == MSX_PREC_MIXED, h->stream);
    cudaError_t err = cudaStreamSynchronize(h->stream);
    double tn = 0, te = 0;
    for (long long i = 0; i < n; i++) {
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, ev[3 * i], ev[3 * i + 1]);
        cudaEventElapsedTime(&b, ev[3 * i + 1], ev[3 * i + 2]);
        tn += a;
        te += b;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return fail(MSX_ERR_CUDA, cudaGetErrorString(err));
    MSX_CUDA(cudaMemcpy(h->h_ctrl, h->ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost));
    h->block_steps = h->h_ctrl[0].step;
    const double ne = (double)h->P.ne, nn = (double)h->P.nn;
    rep->element_ms = te / n;
    rep->node_ms = tn / n;
    rep->element_launches = n;
    rep->node_launches = n;
    // algorithmic bytes: element data per element (conn 16 + dphi 96 + wJ 8 + Lref 8;
    // the FP32 set 16 + 48 + 4 + 4; the double-word set 16 + 72 + 8 + 4) and
    // nodal state per node (read X, u, v, a 96 + m 8, write u, v, a 72)
    rep->element_alg_bytes =
        ne * (h->precision == MSX_PREC_MIXED ? 72.0 : (h->precision == MSX_PREC_DOUBLE_WORD ? 100.0 : 128.0));
    rep->node_alg_bytes = nn * 176.0;
    return MSX_OK;
}

extern "C" msx_status msx_initial_dt(msx_handle *h, double *dt_init)
{
    if (!h || !dt_init) return fail(MSX_ERR_ARG, "NULL argument");
    msx_status st;
    if (!h->block_ready && (st = init_block(h)) != MSX_OK) return st;
    *dt_init = h->dt_init;
    return MSX_OK;
}

extern "C" msx_status msx_element_fields(msx_handle *h, double *cauchy, double *green_lagrange, double *von_mises)
{
    if (!h) return fail(MSX_ERR_ARG, "NULL handle");
    const long long ne = h->P.ne;
    DBuf<double> dc, dg, dv;
    if ((cauchy && dc.alloc(9 * ne) != cudaSuccess) || (green_lagrange && dg.alloc(9 * ne) != cudaSuccess) ||
        (von_mises && dv.alloc(ne) != cudaSuccess)) {
        dc.release();
        dg.release();
        dv.release();
        return fail(MSX_ERR_OOM, "element field buffers");
    }
    bind_problem(h);
    launch_element_fields(h->P, h->last_t, dc.p, dg.p, dv.p, h->stream);
    if (cauchy) cudaMemcpyAsync(cauchy, dc.p, sizeof(double) * 9 * ne, cudaMemcpyDeviceToHost, h->stream);
    if (green_lagrange) cudaMemcpyAsync(green_lagrange, dg.p, sizeof(double) * 9 * ne, cudaMemcpyDeviceToHost, h->stream);
    if (von_mises) cudaMemcpyAsync(von_mises, dv.p, sizeof(double) * ne, cudaMemcpyDeviceToHost, h->stream);
    cudaError_t err = cudaStreamSynchronize(h->stream);
    dc.release();
    dg.release();
    dv.release();
    if (err != cudaSuccess) return fail(MSX_ERR_CUDA, cudaGetErrorString(err));
    return MSX_OK;
}

extern "C" void *msx_stream(msx_handle *h) { return h ? (void *)h->stream : nullptr; }

extern "C" msx_status msx_set_device(int32_t device)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(MSX_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= n) return fail(MSX_ERR_ARG, "device index out of range");
    MSX_CUDA(cudaSetDevice(device));
    return MSX_OK;
}

// Cube generator (same recipe as the test fixtures): see include/msx.h.
static uint64_t splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

extern "C" msx_status msx_mesh_cube(int32_t n, uint64_t seed, double jitter, double *X, int32_t *conn)
{
    if (n < 1 || n > 1000 || !X || !conn) return fail(MSX_ERR_ARG, "cube needs 1 <= n <= 1000 and buffers");
    const long long m = n + 1, nn = m * m * m;
    const double h = 1.0 / (double)n;
    uint64_t s = seed;
    for (long long k = 0; k < m; k++)
        for (long long j = 0; j < m; j++)
            for (long long i = 0; i < m; i++) {
                long long id = i + m * j + m * m * k;
                double c[3] = {(double)i / (double)n, (double)j / (double)n, (double)k / (double)n};
                if (i > 0 && i < n && j > 0 && j < n && k > 0 && k < n)
                    for (int d = 0; d < 3; d++) {
                        double r = (double)(splitmix64(&s) >> 11) * 0x1.0p-53;
                        c[d] += (2.0 * r - 1.0) * (jitter * h);
                    }
                for (int d = 0; d < 3; d++) X[d * nn + id] = c[d];
            }
    // C3D8 corners N1..N8 of hex (i,j,k); six tets per hex
    static const int T[6][4] = {{1, 3, 4, 7}, {1, 2, 3, 7}, {4, 1, 7, 8}, {1, 5, 7, 8}, {1, 5, 6, 7}, {2, 1, 6, 7}};
    long long e = 0;
    for (long long k = 0; k < n; k++)
        for (long long j = 0; j < n; j++)
            for (long long i = 0; i < n; i++) {
                int32_t N[9];
                N[1] = (int32_t)(i + m * j + m * m * k);
                N[2] = N[1] + 1;
                N[3] = N[1] + 1 + (int32_t)m;
                N[4] = N[1] + (int32_t)m;
                for (int q = 5; q <= 8; q++) N[q] = N[q - 4] + (int32_t)(m * m);
                for (int t = 0; t < 6; t++, e++)
                    for (int q = 0; q < 4; q++) conn[e * 4 + q] = N[T[t][q]];
            }
    return MSX_OK;
}
