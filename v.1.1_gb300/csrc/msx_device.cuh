// msx_device.cuh -- device code of the explicit C3D4 step.
//
// Included by one translation unit per numeric mode.  msx_exact.cu is built
// with --fmad=false and instantiates the reference-order kernels; msx_fast.cu
// is built with contraction on and instantiates the FP64 and mixed kernels.
#pragma once
#include <cfloat>
#include <cmath>
#include "msx_internal.h"

namespace msx {

#define MSX_INF_BITS 0x7FF0000000000000ULL
// FP32 +infinity as the running minimum of the CFL screen (dtmin[2..3])
constexpr unsigned long long kScreenInfBits = 0x7F800000ULL;

// ---------------------------------------------------------------------------
// Reference-order arithmetic (src/mathematics/maths.cpp, geometry.cpp and the
// laws).  These compile to plain mul/add only when contraction is off.
// ---------------------------------------------------------------------------
// maths.cpp:1564-1577 determinantTensor
__device__ __forceinline__ double det3_ref(const double *A)
{
    return A[0] * (A[4] * A[8] - A[7] * A[5]) - A[1] * (A[3] * A[8] - A[6] * A[5]) +
           A[2] * (A[3] * A[7] - A[6] * A[4]);
}

// maths.cpp:2749-2785 inverse
__device__ __forceinline__ void inv3_ref(const double *A, double *Ai)
{
    double idet = 1.0 / det3_ref(A);
    Ai[0] = idet * (A[4] * A[8] - A[5] * A[7]);
    Ai[3] = -idet * (A[3] * A[8] - A[5] * A[6]);
    Ai[6] = idet * (A[3] * A[7] - A[4] * A[6]);
    Ai[1] = -idet * (A[1] * A[8] - A[2] * A[7]);
    Ai[4] = idet * (A[0] * A[8] - A[2] * A[6]);
    Ai[7] = -idet * (A[0] * A[7] - A[1] * A[6]);
    Ai[2] = idet * (A[1] * A[5] - A[2] * A[4]);
    Ai[5] = -idet * (A[0] * A[5] - A[2] * A[3]);
    Ai[8] = idet * (A[0] * A[4] - A[1] * A[3]);
}

// geometry.cpp:90-136 areaTriangle (3D) of triangle (p, q, r): 0.5*|(p-r)x(q-r)|
__device__ __forceinline__ double area_tri_ref(const double *p, const double *q, const double *r)
{
    double A0 = p[0] - r[0], A1 = p[1] - r[1], A2 = p[2] - r[2];
    double B0 = q[0] - r[0], B1 = q[1] - r[1], B2 = q[2] - r[2];
    double C0 = A1 * B2 - A2 * B1;
    double C1 = A2 * B0 - A0 * B2;
    double C2 = A0 * B1 - A1 * B0;
    return 0.5 * sqrt(C0 * C0 + C1 * C1 + C2 * C2);
}

// geometry.cpp:264-301 inscribedSphere x 2 (classLinearTetrahedra.cpp:146-163);
// *det_edges (when given) receives the determinant of the edge rows p1-p0,
// p2-p0, p3-p0 that the volume comes from.
__device__ __forceinline__ double char_length_ref(const double *x, double *det_edges = nullptr)
{
    const double *p0 = x, *p1 = x + 3, *p2 = x + 6, *p3 = x + 9;
    double s1 = area_tri_ref(p0, p1, p2);
    double s2 = area_tri_ref(p1, p2, p3);
    double s3 = area_tri_ref(p0, p2, p3);
    double s4 = area_tri_ref(p0, p1, p3);
    double A = fabs(s1) + fabs(s2) + fabs(s3) + fabs(s4);
    double M[9] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], p2[0] - p0[0], p2[1] - p0[1],
                   p2[2] - p0[2], p3[0] - p0[0], p3[1] - p0[1], p3[2] - p0[2]};
    const double D = det3_ref(M);
    if (det_edges) *det_edges = D;
    double V = 1.0 / 6.0 * fabs(D);
    double r = 3.0 * V / A;
    return 2 * r;
}

// First Piola stress in the reference's operation order:
// hyperElasticNeoHookean.cpp:84-127 (Neo-Hookean), :235-259 (compressible),
// hyperElasticStVenantKirchhoff.cpp:64-101,219-222 (StVK), linearElastic.cpp
// :58-82,114-145 (linear elastic: the small-strain stress is returned as P).
__device__ __forceinline__ void stress_ref(const MatParams &m, const double *F, double *P)
{
    if (m.law == 1) {
        double J = det3_ref(F), C[9], iC[9], S[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += F[k * 3 + i] * F[k * 3 + j];
                C[i * 3 + j] = c;
            }
        inv3_ref(C, iC);
#pragma unroll
        for (int i = 0; i < 9; i++) S[i] = 0;
#pragma unroll
        for (int i = 0; i < 3; i++) S[i * 3 + i] += m.mu;
        double alpha = m.lambda * log(J) - m.mu;
#pragma unroll
        for (int i = 0; i < 9; i++) S[i] += alpha * iC[i];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += F[i * 3 + k] * S[k * 3 + j];
                P[i * 3 + j] = c;
            }
    } else if (m.law == 0) {
        double B[9], iF[9], Ca[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += F[i * 3 + k] * F[j * 3 + k];
                B[i * 3 + j] = c;
            }
        double J = det3_ref(F);
        inv3_ref(F, iF);
        double trB = 0;
#pragma unroll
        for (int i = 0; i < 3; i++) trB += B[i * 3 + i];
        double fact1 = pow(J, 5.0 / 3.0);
        double fact2 = m.mu / fact1;
#pragma unroll
        for (int i = 0; i < 9; i++) Ca[i] = 0 + fact2 * B[i];
        double fact3 = -(m.mu / 3.0) * trB / fact1 + m.K1 * (J - 1.0);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) Ca[i * 3 + j] += fact3 * (i == j ? 1.0 : 0.0);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += Ca[i * 3 + k] * iF[j * 3 + k] * J;
                P[i * 3 + j] = c;
            }
    } else if (m.law == 3) {
        // linearElastic.cpp:71-76 E = (F + F^T)/2 - I, :114-145 P = mu2 E + lam tr(E) I
        double E[9], trE = 0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) E[i * 3 + j] = 0.5 * (F[i * 3 + j] + F[j * 3 + i] - 2. * (i == j ? 1. : 0.));
#pragma unroll
        for (int i = 0; i < 3; i++) trE += E[i * 3 + i];
#pragma unroll
        for (int i = 0; i < 9; i++) P[i] = E[i] * m.mu2;
#pragma unroll
        for (int i = 0; i < 3; i++) P[i * 3 + i] += m.lam_stvk * trE;
    } else {
        double C[9], S[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += F[k * 3 + i] * F[k * 3 + j];
                C[i * 3 + j] = c;
            }
        double trE = 0;
#pragma unroll
        for (int i = 0; i < 9; i++) S[i] = 0.5 * (C[i] - ((i % 4) == 0 ? 1.0 : 0.0));
#pragma unroll
        for (int i = 0; i < 3; i++) trE += S[i * 3 + i];
#pragma unroll
        for (int i = 0; i < 9; i++) S[i] = S[i] * m.mu2;
#pragma unroll
        for (int i = 0; i < 3; i++) S[i * 3 + i] += m.lam_stvk * trE;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += F[i * 3 + k] * S[k * 3 + j];
                P[i * 3 + j] = c;
            }
    }
}

// ---------------------------------------------------------------------------
// Shared pieces
// ---------------------------------------------------------------------------
__device__ __forceinline__ const MatParams &mat_of(const Problem &p, long long e)
{
    return p.mats[p.mat ? p.mat[e] : 0];
}

// Element birth (the reference's *ACTIVATION option: solvers.cpp:403-433 with
// the laws' checkActivation): a St-Venant-Kirchhoff or linear-elastic element
// is alive once its activation time is <= t; a dead element adds no internal
// force (solverExplicit.cpp:370-371).  act_t is null without the option.
__device__ __forceinline__ bool elem_dead(const Problem &p, long long e, double t)
{
    return p.act_t && mat_of(p, e).law >= 2 && t < p.act_t[e];
}

// Block-wide min of a positive double, then one integer atomicMin on its bit
// pattern (monotone for non-negative doubles; exact and order independent).
__device__ __forceinline__ void block_min_to(double v, unsigned long long *slot)
{
    __shared__ double wmin[32];
    if (!(v >= 0.0)) v = INFINITY;    // NaN or negative: ignored
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) wmin[w] = v;
    __syncthreads();
    if (w == 0) {
        int nw = (blockDim.x + 31) >> 5;
        v = l < nw ? wmin[l] : INFINITY;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (l == 0 && v < INFINITY) atomicMin(slot, (unsigned long long)__double_as_longlong(v));
    }
    __syncthreads();   // wmin may be reused by the next call
}

// The control decision of the node kernel: derived identically in every
// thread from the previous slot (solverExplicit.cpp:217-276).
struct StepDecision {
    Ctrl next;
    bool run;
};

__device__ __forceinline__ StepDecision decide_step(const Problem &p, const Ctrl &cp, int parity)
{
    StepDecision d;
    d.next = cp;
    d.next.ran = 0;
    d.run = false;
    if (cp.stop) return d;
    if (cp.ran && p.flags[parity]) {        // uK[1] not finite after the last step
        d.next.status = 4;
        d.next.stop = 1;
        return d;
    }
    if (cp.t < p.tf - 1E-12 && cp.step < cp.limit) {
        double t = cp.t, dt = cp.dt;
        if (t + dt > p.tf) {
            dt = p.tf - t;
            t = p.tf;
        } else {
            t += dt;
        }
        double dtn = __longlong_as_double((long long)p.dtmin[parity]);
        dtn = dtn * p.sf;
        d.next.t = t;
        if (dtn < 1E-20) {
            d.next.status = 3;
            d.next.stop = 1;
            d.next.dt = dtn;
        } else {
            d.next.dt = dtn;
            d.next.step = cp.step + 1;
            d.next.ran = 1;
            d.run = true;
        }
    } else {
        // stopped at tf or at the step limit: keep the CFL min of the next step
        // so that a later call can resume the block where it left off
        d.next.stop = 1;
        d.next.pending = p.dtmin[parity];
    }
    return d;
}

// Dirichlet increment of one entry at block step `step` (solverExplicit.cpp:545-575)
__device__ __forceinline__ double bc_increment(const BCEntry &b, double dt, long long step)
{
    if (b.mode == 1) return step == 1 ? b.val : 0.0;
    if (b.mode == 2) {
        double r = (b.ramp_steps > 0 && step < b.ramp_steps) ? (double)step / (double)b.ramp_steps : 1.0;
        return b.val * r * dt;
    }
    return b.val * dt;
}

// ---------------------------------------------------------------------------
// Node kernel: post-update of step n-1 (a = -f_int/m, v += dt (a_prev+a)/2,
// nonlinearSystem.cpp:1034-1117), control of step n, prediction
// u += dt v + dt^2/2 a (nonlinearSystem.cpp:1186-1200) and Dirichlet values.
// One thread per node, three components.
// ---------------------------------------------------------------------------
// Dirichlet records of node i: per component (first entry, count); count 0 = active.
__device__ __forceinline__ void node_bc_records(const Problem &p, long long i, int2 *br)
{
    br[0] = br[1] = br[2] = make_int2(0, 0);
    int rec = p.node_bc[i];
    if (rec >= 0) {
        br[0] = p.bc_rec[rec * 3 + 0];
        br[1] = p.bc_rec[rec * 3 + 1];
        br[2] = p.bc_rec[rec * 3 + 2];
    }
}

// External force of DOF d at time t (the step being completed): its terms in
// deck order, summed from 0 as NeumannBCManagement fills the force vector
// (boundaryConditions.cpp:75-138; nodal forces m t inside [t0, tf],
// classNodes.h:101-109).
__device__ __forceinline__ double ext_force_dof(const Problem &p, long long d, double t)
{
    double fx = 0.0;
    for (int k = p.ext_ptr[d]; k < p.ext_ptr[d + 1]; k++) {
        const unsigned term = p.ext_term[k], idx = term & ((1u << kExtIndexBits) - 1u);
        double v;
        switch (term >> kExtIndexBits) {
        case EXT_FORCE: {
            const ForceEntry f = p.nfs[idx];
            v = (t >= f.t0 && t <= f.tf) ? f.m * t : 0;
            break;
        }
        case EXT_GRAV_ELEM: v = p.grav_e[idx]; break;
        case EXT_GRAV_NODE: v = p.grav_n[idx]; break;
        default: v = p.fcon[idx]; break;
        }
        fx += v;
    }
    return fx;
}

// One DOF: post-update of step n-1 with the gathered internal force s and
// external force fx (a = (fx - s)/m, v += dt (a_prev + a)/2), then the
// prediction (active) or the Dirichlet values (constrained) of step n.  The
// reference-order mode keeps the reference's operations; the others use
// v += (dt/2)(a_prev + a) and u += dt (v + (dt/2) a) with 1/m.
template <int MODE>
__device__ __forceinline__ void dof_update(const Problem &p, long long dof, double ui, double vi, double ai, double s,
                                           double fx, bool loads, int2 br, const Ctrl &cp, const StepDecision &d,
                                           double mass, double minv)
{
    const bool act = br.y == 0;
    bool changed = false;
    if (cp.ran && act) {
        double an;
        if (MODE == MODE_EXACT) {
            double val = -s + fx;
            double rhs = 0;
            rhs += val;
            an = rhs / mass;
            vi += cp.dt * ((1. - 0.5) * ai + 0.5 * an);
        } else {
            an = (loads ? fx - s : -s) * minv;
            vi = fma(0.5 * cp.dt, ai + an, vi);
        }
        ai = an;
        changed = true;
    }
    if (d.run) {
        const double dtn = d.next.dt;
        if (act) {
            if (MODE == MODE_EXACT) ui += dtn * vi + 0.5 * dtn * dtn * ai;
            else ui = fma(dtn, fma(0.5 * dtn, ai, vi), ui);
        } else {
            for (int k = br.x; k < br.x + br.y; k++) {
                double Ud = bc_increment(p.bcs[k], dtn, d.next.step);
                ui += Ud;
                vi = Ud;
                ai = 0.;
            }
        }
        changed = true;
    }
    if (changed) {
        p.u[dof] = ui;
        p.v[dof] = vi;
        p.a[dof] = ai;
        if (MODE == MODE_MIXED) {
            float hi = (float)ui;
            p.uhl[dof] = make_float2(hi, (float)(ui - (double)hi));
        }
    }
}

// Node kernel body, one thread per node (reference-order mode): corner forces
// of the incident elements summed in element order, then the three DOFs.
template <int MODE>
__device__ __forceinline__ void node_body(const Problem &p, long long i, const Ctrl &cp, const StepDecision &d)
{
    int2 br[3];
    node_bc_records(p, i, br);
    double s[3] = {0.0, 0.0, 0.0};
    if (cp.ran && (br[0].y == 0 || br[1].y == 0 || br[2].y == 0)) {
        for (int k = p.node_ptr[i]; k < p.node_ptr[i + 1]; k++) {
            const double *f = p.fe + (long long)p.node_inc[k] * 3;
            s[0] += f[0];
            s[1] += f[1];
            s[2] += f[2];
        }
    }
    double fx[3] = {0.0, 0.0, 0.0};
    if (cp.ran && p.ext_ptr)
        for (int c = 0; c < 3; c++) fx[c] = ext_force_dof(p, i + c * p.nn, cp.t);
    const double mass = MODE == MODE_EXACT ? p.mass[i] : 0.0, minv = MODE == MODE_EXACT ? 0.0 : p.minv[i];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const long long dof = i + c * p.nn;
        dof_update<MODE>(p, dof, p.u[dof], p.v[dof], p.a[dof], s[c], fx[c], true, br[c], cp, d, mass, minv);
    }
}

// Rounding error of s = fl(a + b): a + b = s + err exactly (Knuth's TwoSum).
__device__ __forceinline__ float two_sum_err(float a, float b, float s)
{
    float bp = s - a;
    return (a - (s - bp)) + (b - bp);
}

// Neumaier merge of two compensated FP32 partial sums (lo first).
__device__ __forceinline__ void neumaier_merge(float &sh, float &sc, float oh, float oc)
{
    float t = sh + oh;
    float e = fabsf(sh) >= fabsf(oh) ? (sh - t) + oh : (oh - t) + sh;
    sh = t;
    sc = (sc + oc) + e;
}

// ---------------------------------------------------------------------------
// Double-word ("double-float") arithmetic: a value is a pair (hi, lo) of FP32
// numbers with value hi + lo and |lo| <= ulp(hi)/2, about 48 significant
// bits.  The mixed mode keeps the nodal state u, v, a in this form while a
// block runs, so its node update runs on the FP32 pipe (on this GPU the FP64
// pipe issues about 1/64 of the FP32 rate).  Algorithms: TwoSum (Knuth),
// Fast2Sum (Dekker), and the accurate double-word sum and double-word product
// of Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44 (2017), Algs. 6, 12.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 df_fast2sum(float a, float b)   // needs |a| >= |b| (or a = 0)
{
    float s = a + b;
    return make_float2(s, b - (s - a));
}

__device__ __forceinline__ float2 df_two_sum(float a, float b)
{
    float s = a + b;
    return make_float2(s, two_sum_err(a, b, s));
}

__device__ __forceinline__ float2 df_add(float2 x, float2 y)
{
    float2 s = df_two_sum(x.x, y.x), t = df_two_sum(x.y, y.y);
    float2 v = df_fast2sum(s.x, s.y + t.x);
    return df_fast2sum(v.x, t.y + v.y);
}

__device__ __forceinline__ float2 df_mul(float2 x, float2 y)
{
    float ch = x.x * y.x;
    float cl1 = fmaf(x.x, y.x, -ch);
    float cl2 = fmaf(x.y, y.x, fmaf(x.x, y.y, x.y * y.y));
    return df_fast2sum(ch, cl1 + cl2);
}

__device__ __forceinline__ float2 df_neg(float2 x) { return make_float2(-x.x, -x.y); }

// nearest double-word to an FP64 value (FP64 pipe: control values and loads only)
__device__ __forceinline__ float2 df_from(double x)
{
    float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// Per-solve quantities of the node kernel, derived once per block and solve
// from the solve's control slot (not once per tile).
struct NodeStep {
    bool ran, run, loads;       // step n-1 ran / step n runs / external loads present
    long long step;             // block step number of step n
    double t;                   // time of step n-1 (external forces)
    double hdt, dtn, hdtn;      // dt/2 of the step being completed; dt, dt/2 of the next
    float2 hdt2, dtn2, hdtn2;   // the same as double-words (mixed)
};

template <int MODE>
__device__ __forceinline__ void node_step(const Problem &p, int parity, NodeStep &ns)
{
    const Ctrl cp = p.ctrl[parity ^ 1];
    const StepDecision d = decide_step(p, cp, parity);
    ns.ran = cp.ran;
    ns.run = d.run;
    ns.step = d.next.step;
    ns.t = cp.t;
    ns.hdt = 0.5 * cp.dt;
    ns.dtn = d.next.dt;
    ns.hdtn = 0.5 * ns.dtn;
    if (MODE == MODE_MIXED || MODE == MODE_DW) {
        ns.hdt2 = df_from(ns.hdt);
        ns.dtn2 = df_from(ns.dtn);
        ns.hdtn2 = df_from(ns.hdtn);
    }
    ns.loads = p.ext_ptr != nullptr;
}

// Node kernel bodies of the tiled FP64 and mixed kernels: four lanes per node.
// The node's corner forces sit in its CSR slots [node_ptr[i], node_ptr[i+1]),
// in element order; lane q sums slots k0+q, k0+q+4, ...  The lane sums l_q
// are combined as (l0 + l1) + (l2 + l3) for every component (addition and
// the compensated merge are commutative, so the result does not depend on
// which lane adds): each lane receives only what it or the lane it serves
// next needs.  Lane c < 3 then updates DOF c: a = (f_ext - f_int)/m,
// v += (dt/2)(a_prev + a), u += dt (v + (dt/2) a), or the Dirichlet values.
// The DOF state, mass and Dirichlet record are loaded before the gather so
// their latency overlaps it.  All 32 lanes of a warp call these together
// (valid = false past the tile's end).
template <typename T>
__device__ __forceinline__ T pick3(int c, T a, T b, T d) { return c == 0 ? a : (c == 1 ? b : d); }

__device__ __forceinline__ double node_fext(const Problem &p, long long i, int q, const NodeStep &ns)
{
    return ext_force_dof(p, i + (long long)q * p.nn, ns.t);
}

// Biased exponent field of a double (0: zero or subnormal, 0x7FF: Inf or NaN).
__device__ __forceinline__ int dexp_field(double x) { return (__double2hiint(x) >> 20) & 0x7FF; }

// x as an integer multiple of 2^(max(E,1) - 1075 - H), truncated toward zero;
// E is at least x's exponent field and not 0x7FF, 0 <= H <= 10.
__device__ __forceinline__ long long dfixed(double x, int E, int H)
{
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7FF);
    unsigned long long m = (unsigned long long)b & 0xFFFFFFFFFFFFFull;
    if (ex) m |= 1ull << 52;
    const int d = max(E, 1) - max(ex, 1);
    const unsigned long long t = d > 63 ? 0ull : (m << H) >> d;
    return b < 0 ? -(long long)t : (long long)t;
}

// x * 2^k for an integer-valued x (|x| < 2^63) and -1085 <= k <= 971: exact
// unless the product is subnormal, then rounded once (the first factor of the
// two-step case keeps x * 2^-600 normal and exact).
__device__ __forceinline__ double pow2_scale(double x, int k)
{
    if (k < -1022) {
        x *= __longlong_as_double((long long)(1023 - 600) << 52);
        k += 600;
    }
    return x * __longlong_as_double((long long)(k + 1023) << 52);
}

// A 24-byte corner slot of the FP64 layout (slot k at byte 24 k: 16-byte
// aligned for even k) in one 16-byte and one 8-byte access instead of three
// 8-byte ones: the 16-byte half holds values 0-1 of an even slot, 1-2 of an
// odd one.  The selects keep the warp on one path.
__device__ __forceinline__ void ld_slot24(const double *base, long long k, double &x, double &y, double &z)
{
    const bool odd = k & 1;
    const double *s = base + 3 * k;
    const double2 v = __ldg(reinterpret_cast<const double2 *>(s + (odd ? 1 : 0)));
    const double w = __ldg(s + (odd ? 0 : 2));
    x = odd ? w : v.x;
    y = odd ? v.x : v.y;
    z = odd ? v.y : w;
}
__device__ __forceinline__ void st_slot24(double *base, long long k, double x, double y, double z)
{
    const bool odd = k & 1;
    double *s = base + 3 * k;
    *reinterpret_cast<double2 *>(s + (odd ? 1 : 0)) = odd ? make_double2(y, z) : make_double2(x, y);
    s[odd ? 0 : 2] = odd ? x : z;
}

__device__ __forceinline__ void node_quad_fp64(const Problem &p, long long i, bool valid, const NodeStep &ns)
{
    const int q = threadIdx.x & 3;
    const bool odd = q & 1;
    const bool own = valid && q < 3;   // this lane updates DOF q of node i
    const long long dof = i + (long long)q * p.nn;
    double ui = 0, vi = 0, ai = 0, minv = 0;
    int rec = -1;
    if (own) {
        ui = p.u[dof];
        vi = p.v[dof];
        ai = p.a[dof];
        minv = p.minv[i];
        rec = p.node_bc[i];
    }
    int k0 = 0, k1 = 0;
    if (valid && ns.ran) {
        k0 = p.node_ptr[i];
        k1 = p.node_ptr[i + 1];
    }
    // The node's f_int per component as one exact integer sum, rounded once:
    // each term's 53-bit significand aligned to the largest exponent E of that
    // component among the node's terms, with H guard bits below it, summed in
    // int64 on the integer pipes instead of ~24 dependent FP64 additions.  With
    // n terms, H = 10 - ceil(log2 n) keeps the sum below 2^63; bits below the
    // guard bits are truncated (at most one unit of 2^(E - 1075 - H) per term).
    // The sum does not depend on the order of the terms.  Nodes with an
    // infinite or NaN term, or too many terms for H >= 0 (and the other nodes of
    // their warp), add in FP64.
    const int n = k1 - k0;   // the same for the node's four lanes
    int e0 = 0, e1 = 0, e2 = 0;
    for (int k = k0 + q; k < k1; k += 4) {
        double f0, f1, f2;
        ld_slot24(p.fe, k, f0, f1, f2);
        e0 = max(e0, dexp_field(f0));
        e1 = max(e1, dexp_field(f1));
        e2 = max(e2, dexp_field(f2));
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
        e0 = max(e0, __shfl_xor_sync(0xffffffffu, e0, o));
        e1 = max(e1, __shfl_xor_sync(0xffffffffu, e1, o));
        e2 = max(e2, __shfl_xor_sync(0xffffffffu, e2, o));
    }
    const int H = 10 - (n > 1 ? 32 - __clz(n - 1) : 0);
    // one path for the whole warp: both use shuffles over all 32 lanes (lanes
    // past the tile's end have no terms and vote for the integer path)
    const bool fixed = __all_sync(0xffffffffu, H >= 0 && max(e0, max(e1, e2)) < 0x7FF);
    double s;
    if (fixed) {
        long long a0 = 0, a1 = 0, a2 = 0;
        for (int k = k0 + q; k < k1; k += 4) {
            double f0, f1, f2;
            ld_slot24(p.fe, k, f0, f1, f2);
            a0 += dfixed(f0, e0, H);
            a1 += dfixed(f1, e1, H);
            a2 += dfixed(f2, e2, H);
        }
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        }
        if (!own) return;
        s = pow2_scale(__ll2double_rn(pick3(q, a0, a1, a2)), max(pick3(q, e0, e1, e2), 1) - 1075 - H);
    } else {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int k = k0 + q; k < k1; k += 4) {
            const double *f = p.fe + (long long)k * 3;
            s0 += f[0];
            s1 += f[1];
            s2 += f[2];
        }
        // pairs (0,1), (2,3): even lanes need components 0 and 2, odd lanes 1
        double x = __shfl_xor_sync(0xffffffffu, odd ? s0 : s1, 1), y = __shfl_xor_sync(0xffffffffu, s2, 1);
        if (odd) {
            s1 += x;
        } else {
            s0 += x;
            s2 += y;
        }
        // across pairs: lanes 0 <-> 2 exchange components 2 / 0, lane 1 <- 3 component 1
        double z = __shfl_xor_sync(0xffffffffu, odd ? s1 : (q == 0 ? s2 : s0), 2);
        if (!own) return;
        s = pick3(q, s0, s1, s2) + z;
    }
    const int2 br = rec >= 0 ? p.bc_rec[rec * 3 + q] : make_int2(0, 0);
    const bool act = br.y == 0;
    bool changed = false;
    if (ns.ran && act) {
        const double an = (ns.loads ? node_fext(p, i, q, ns) - s : -s) * minv;
        vi = fma(ns.hdt, ai + an, vi);
        ai = an;
        changed = true;
    }
    if (ns.run) {
        if (act) {
            ui = fma(ns.dtn, fma(ns.hdtn, ai, vi), ui);
        } else {
            for (int k = br.x; k < br.x + br.y; k++) {
                double Ud = bc_increment(p.bcs[k], ns.dtn, ns.step);
                ui += Ud;
                vi = Ud;
                ai = 0.;
            }
        }
        changed = true;
    }
    if (changed) {
        p.u[dof] = ui;
        p.v[dof] = vi;
        p.a[dof] = ai;
        if (p.u4) p.u4[4LL * i + q] = ui;
    }
}

// The mixed mode's acceleration, one FP32 per DOF in the storage of ahl: a is
// recomputed every step from the FP32 corner forces (compensated sum / m), so
// FP32 holds all it carries; u and v, the accumulated state, stay double-words.
__device__ __forceinline__ float *mixed_a32(const Problem &p) { return reinterpret_cast<float *>(p.ahl); }

__device__ __forceinline__ void node_quad_mixed(const Problem &p, long long i, bool valid, const NodeStep &ns)
{
    const int q = threadIdx.x & 3;
    const bool odd = q & 1;
    const bool own = valid && q < 3;
    const long long dof = i + (long long)q * p.nn;
    float2 uq = make_float2(0.f, 0.f), vq = uq, aq = uq, minv = uq;
    int rec = -1;
    if (own) {
        uq = p.uhl[dof];
        vq = p.vhl[dof];
        aq = make_float2(mixed_a32(p)[dof], 0.f);
        minv = p.minv2[i];
        rec = p.node_bc[i];
    }
    int k0 = 0, k1 = 0;
    if (valid && ns.ran) {
        k0 = p.node_ptr[i];
        k1 = p.node_ptr[i + 1];
    }
    // compensated FP32 sums (Neumaier) of the FP32 corner forces
    const float4 *fe = reinterpret_cast<const float4 *>(p.fe32);
    float h0 = 0.f, h1 = 0.f, h2 = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
    int k = k0 + q;
    if (k < k1) {
        const float4 f = fe[k];
        h0 = f.x;
        h1 = f.y;
        h2 = f.z;
        k += 4;
    }
    for (; k < k1; k += 4) {
        const float4 f = fe[k];
        neumaier_merge(h0, c0, f.x, 0.0f);
        neumaier_merge(h1, c1, f.y, 0.0f);
        neumaier_merge(h2, c2, f.z, 0.0f);
    }
    float ah = odd ? h0 : h1, ac = odd ? c0 : c1;
    float xh = __shfl_xor_sync(0xffffffffu, ah, 1), xc = __shfl_xor_sync(0xffffffffu, ac, 1);
    float yh = __shfl_xor_sync(0xffffffffu, h2, 1), yc = __shfl_xor_sync(0xffffffffu, c2, 1);
    if (odd) {
        neumaier_merge(h1, c1, xh, xc);
    } else {
        neumaier_merge(h0, c0, xh, xc);
        neumaier_merge(h2, c2, yh, yc);
    }
    float sh = odd ? h1 : (q == 0 ? h2 : h0), sc = odd ? c1 : (q == 0 ? c2 : c0);
    float zh = __shfl_xor_sync(0xffffffffu, sh, 2), zc = __shfl_xor_sync(0xffffffffu, sc, 2);
    float mh = pick3(q, h0, h1, h2), mc = pick3(q, c0, c1, c2);
    neumaier_merge(mh, mc, zh, zc);
    if (!own) return;
    const float2 s = df_two_sum(mh, mc);
    const int2 br = rec >= 0 ? p.bc_rec[rec * 3 + q] : make_int2(0, 0);
    const bool act = br.y == 0;
    bool changed = false;
    if (ns.ran && act) {
        const float2 f = ns.loads ? df_add(df_from(node_fext(p, i, q, ns)), df_neg(s)) : df_neg(s);
        const float2 an = df_mul(f, minv);
        vq = df_add(vq, df_mul(ns.hdt2, df_add(aq, an)));
        aq = make_float2(__fadd_rn(an.x, an.y), 0.f);   // as stored: the prediction uses what a later call reads
        changed = true;
    }
    if (ns.run) {
        if (act) {
            uq = df_add(uq, df_mul(ns.dtn2, df_add(vq, df_mul(ns.hdtn2, aq))));
        } else {
            for (int k = br.x; k < br.x + br.y; k++) {
                const float2 Ud = df_from(bc_increment(p.bcs[k], ns.dtn, ns.step));
                uq = df_add(uq, Ud);
                vq = Ud;
                aq = make_float2(0.f, 0.f);
            }
        }
        changed = true;
    }
    if (changed) {
        p.uhl[dof] = uq;
        p.vhl[dof] = vq;
        mixed_a32(p)[dof] = aq.x;
    }
}

// Writes the new control slot and clears the slots the element kernel fills.
__device__ __forceinline__ void publish_step(const Problem &p, const StepDecision &d, int parity)
{
    p.ctrl[parity] = d.next;
    p.dtmin[parity ^ 1] = MSX_INF_BITS;
    p.dtmin[2 + (parity ^ 1)] = kScreenInfBits;
    p.flags[parity ^ 1] = 0;
}

template <int MODE>
__global__ void __launch_bounds__(kNodeBlock) node_kernel(Problem p, int parity)
{
    const Ctrl cp = p.ctrl[parity ^ 1];
    StepDecision d = decide_step(p, cp, parity);
    if (blockIdx.x == 0 && threadIdx.x == 0) publish_step(p, d, parity);
    if (!cp.ran && !d.run) return;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < p.nn) node_body<MODE>(p, i, cp, d);
}

// ---------------------------------------------------------------------------
// Element kernels: F, P, wJ B^T P corner forces and the deformed CFL length.
// ---------------------------------------------------------------------------

// Reference operation order (used with contraction off).
__device__ __forceinline__ float f32_trunc(double x);
__device__ __forceinline__ float cfl_screen(const Problem &p, long long e, const float *g, const float *du,
                                            const MatParams &m);

// Exact CFL value of one element, min(L_ref, L(X+u)) / c, in the reference's
// order (solvers.cpp:304-317: deformed inscribed sphere).
__device__ __forceinline__ double cfl_exact_ref(const Problem &p, long long e)
{
    const long long nn = p.nn;
    const int4 cn = p.conn[e];
    const int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double x[12];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            x[a * 3 + k] = p.X[k * nn + nd[a]];
            x[a * 3 + k] += p.u[nd[a] + k * nn];
        }
    double dist = char_length_ref(x);
    double Lr = p.Lref[e];
    double mlen = (dist < Lr) ? dist : Lr;
    return mlen / mat_of(p, e).c;
}

// SCREEN: return the FP32 screen value of the CFL (cfl_screen) instead of the
// exact one; the caller rechecks the elements near its block's minimum.
template <bool FORCE_ONLY, bool SCREEN = false, bool VISC = false>
__device__ __forceinline__ double elem_body_exact(const Problem &p, long long e, int parity)
{
    const long long ne = p.ne, nn = p.nn;
    double vmin = INFINITY;
    {
        int4 cn = p.conn[e];
        int nd[4] = {cn.x, cn.y, cn.z, cn.w};
        double dphi[12];
#pragma unroll
        for (int k = 0; k < 9; k++) dphi[3 + k] = p.G[k * ne + e];
#pragma unroll
        for (int j = 0; j < 3; j++) dphi[j] = (-dphi[3 + j] - dphi[6 + j]) - dphi[9 + j];
        double ue[12];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) ue[a * 3 + i] = p.u[nd[a] + i * nn];
        // constitutiveManager.cpp:151-164
        double F[9], P[9];
#pragma unroll
        for (int i = 0; i < 9; i++) F[i] = 0.;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            F[i * 3 + i] += 1.;
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int j = 0; j < 3; j++) F[i * 3 + j] += dphi[a * 3 + j] * ue[a * 3 + i];
        }
        const MatParams &m = mat_of(p, e);
        stress_ref(m, F, P);
        // constitutiveAlgorithms.cpp:46-56
        double wJ = p.wJ[e];
        double *fe = p.fe + e * 12;
        const bool dead = !FORCE_ONLY && elem_dead(p, e, p.ctrl[parity].t);
        double Pv[9];
        if (VISC && !FORCE_ONLY) {
            // bulkViscosity in the reference's order (solverExplicit.cpp:514-541; sumTensorTensor,
            // multiSTensorScalar, getTrace, multSTensor3SecondTranspose: maths.cpp:1169-1175,
            // 1604-1610, 2257-2286); F_prev's diagonal rolls to F's
            double *f0 = p.visc_f0;
            const double dt = p.ctrl[parity].dt;
            double Fd[3] = {0., 0., 0.};
            if (dt != 0) {
                const double r = 1 / dt;
#pragma unroll
                for (int c = 0; c < 3; c++) Fd[c] = (F[c * 4] + (-1) * f0[c * ne + e]) * r;
            }
            double trD = 0;
#pragma unroll
            for (int c = 0; c < 3; c++) trD += Fd[c];
#pragma unroll
            for (int c = 0; c < 3; c++) f0[c * ne + e] = F[c * 4];
            const double J1 = det3_ref(F);
            const double Rho_1 = m.rho / J1;
            const double qBV = Rho_1 * p.visc_h *
                               (p.visc_c1 * p.visc_c1 * p.visc_h * fabs(trD) * ((trD < 0.) ? trD : 0.) +
                                p.visc_cl * p.visc_c0 * trD);
            double Cv[9], iF[9];
#pragma unroll
            for (int k = 0; k < 9; k++) Cv[k] = (k % 4 == 0) ? -1 * qBV : 0.0;
            inv3_ref(F, iF);
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    double s = 0;
#pragma unroll
                    for (int k = 0; k < 3; k++) s += Cv[i * 3 + k] * iF[j * 3 + k];
                    Pv[i * 3 + j] = s * (-1 * J1);
                }
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) {
                double f = 0;
#pragma unroll
                for (int J = 0; J < 3; J++) f += wJ * P[i * 3 + J] * dphi[a * 3 + J];
                f = 0 + f;
                if (VISC && !FORCE_ONLY)   // the viscous pass's terms, as computeInternalForce adds them
#pragma unroll
                    for (int J = 0; J < 3; J++) f += wJ * Pv[i * 3 + J] * dphi[a * 3 + J];
                fe[a * 3 + i] = dead ? 0.0 : f;
            }
        if (!FORCE_ONLY && SCREEN) {
            float du32[9];
#pragma unroll
            for (int a = 1; a < 4; a++)
#pragma unroll
                for (int i = 0; i < 3; i++) du32[(a - 1) * 3 + i] = f32_trunc(ue[a * 3 + i] - ue[i]);
            float g32[9];
#pragma unroll
            for (int k = 0; k < 9; k++) g32[k] = f32_trunc(dphi[3 + k]);
            vmin = (double)cfl_screen(p, e, g32, du32, m);
            if (e == 0 && !isfinite(p.u[1])) atomicOr(p.flags + (parity ^ 1), 1);
        } else if (!FORCE_ONLY) {
            // solvers.cpp:304-317: deformed inscribed sphere
            double x[12];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    x[a * 3 + k] = p.X[k * nn + nd[a]];
                    x[a * 3 + k] += ue[a * 3 + k];
                }
            double dist = char_length_ref(x);
            double Lr = p.Lref[e];
            double mlen = (dist < Lr) ? dist : Lr;
            vmin = mlen / m.c;
            if (e == 0 && !isfinite(p.u[1])) atomicOr(p.flags + (parity ^ 1), 1);
        }
    }
    return vmin;
}

template <bool FORCE_ONLY>
__global__ void __launch_bounds__(kElemBlock) elem_kernel_exact(Problem p, int parity)
{
    if (!FORCE_ONLY && !p.ctrl[parity].ran) return;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = e < p.ne ? elem_body_exact<FORCE_ONLY>(p, e, parity) : INFINITY;
    if (!FORCE_ONLY) block_min_to(v, p.dtmin + (parity ^ 1));
}

// Plain FP64 with contraction: H from node differences, laws written through
// the cofactor of F (F C^-1 = F^-T = cof(F)/J), the 4th corner force as minus
// the sum of the other three.  Same algebra as the reference, fewer FP64
// operations.
__device__ __forceinline__ void cofactor(const double *F, double *K)
{
    K[0] = F[4] * F[8] - F[5] * F[7];
    K[1] = F[5] * F[6] - F[3] * F[8];
    K[2] = F[3] * F[7] - F[4] * F[6];
    K[3] = F[2] * F[7] - F[1] * F[8];
    K[4] = F[0] * F[8] - F[2] * F[6];
    K[5] = F[1] * F[6] - F[0] * F[7];
    K[6] = F[1] * F[5] - F[2] * F[4];
    K[7] = F[2] * F[3] - F[0] * F[5];
    K[8] = F[0] * F[4] - F[1] * F[3];
}

// Artificial bulk viscosity (the second pass of computeInternalForce,
// solverExplicit.cpp:381-421, with bulkViscosity, :514-541): the viscous
// Cauchy stress -qBV I maps to the Piola stress J qBV F^-T = qBV cof(F), with
// qBV = rho/J h (c1^2 h |trD| min(0, trD) + cl c0 trD) and trD = tr(Fdot),
// Fdot = (F - F_prev)/dt.  Only F_prev's diagonal enters, so that is what an
// element keeps; h and c0 stand for the reference's solvers::_elementSize and
// _c0.  FP64 form; the mixed and reference-order forms sit in their bodies.
__device__ __forceinline__ double visc_q(const Problem &p, double rho, double J, double trD)
{
    return rho / J * p.visc_h * (p.visc_c1 * p.visc_c1 * p.visc_h * fabs(trD) * fmin(0.0, trD) +
                                 p.visc_cl * p.visc_c0 * trD);
}

// P += wJ qBV cof(F) for F in FP64 (FP64 and double-word modes); rolls the
// element's F_prev diagonal to F's.
__device__ __forceinline__ void visc_bulk_fp64(const Problem &p, long long e, const double *F, double wJ, double rho,
                                               double idt, double *Pv)
{
    const long long ne = p.ne;
    double *f0 = p.visc_f0;
    const double trD = ((F[0] - f0[e]) + (F[4] - f0[ne + e]) + (F[8] - f0[2 * ne + e])) * idt;
    f0[e] = F[0];
    f0[ne + e] = F[4];
    f0[2 * ne + e] = F[8];
    double K[9];
    cofactor(F, K);
    const double J = F[0] * K[0] + F[1] * K[1] + F[2] * K[2];
    const double w = wJ * visc_q(p, rho, J, trD);
#pragma unroll
    for (int k = 0; k < 9; k++) Pv[k] = w * K[k];
}

// ln J for J = det F in FP64.  For |J - 1| < 2^-7 (the usual case) the
// series of log1p(x), x = J - 1, to x^9 by Horner's rule: truncation below
// |x|^10/10 < 1e-22 |x|, so its error is that of the rounded coefficients,
// about 1 ulp of ln J; x itself carries J's rounding, as log(J) does.
// Otherwise the library log.
__device__ __forceinline__ double log_near1(double J)
{
    const double x = J - 1.0;
    if (!(fabs(x) < 0.0078125)) return log(J);
    double q = 1.0 / 9.0;
    q = fma(q, -x, 1.0 / 8.0);
    q = fma(q, -x, 1.0 / 7.0);
    q = fma(q, -x, 1.0 / 6.0);
    q = fma(q, -x, 1.0 / 5.0);
    q = fma(q, -x, 1.0 / 4.0);
    q = fma(q, -x, 1.0 / 3.0);
    q = fma(q, -x, 1.0 / 2.0);
    q = fma(q, -x, 1.0);
    return q * x;
}

// wJ * P written through the cofactor; the quadrature weight is folded into
// the law's scalar coefficients instead of scaling the nine entries of P.
__device__ __forceinline__ void stress_fast(const MatParams &m, const double *F, double wJ, double *P)
{
    if (m.law == 3) {
        // linear elastic: wJ P = wJ (mu2 E + lam tr(E) I), E = (F + F^T)/2 - I
        const double h = m.mu2 * wJ;
        const double E00 = F[0] - 1.0, E11 = F[4] - 1.0, E22 = F[8] - 1.0;
        const double dg = m.lam_stvk * ((E00 + E11) + E22) * wJ;
        P[0] = h * E00 + dg;
        P[4] = h * E11 + dg;
        P[8] = h * E22 + dg;
        P[1] = P[3] = 0.5 * h * (F[1] + F[3]);
        P[2] = P[6] = 0.5 * h * (F[2] + F[6]);
        P[5] = P[7] = 0.5 * h * (F[5] + F[7]);
        return;
    }
    if (m.law == 2) {
        // S = mu2 E + lam tr(E) I, E = (F^T F - I)/2; wJ P = F (wJ S)
        double C00 = F[0] * F[0] + F[3] * F[3] + F[6] * F[6];
        double C11 = F[1] * F[1] + F[4] * F[4] + F[7] * F[7];
        double C22 = F[2] * F[2] + F[5] * F[5] + F[8] * F[8];
        double C01 = F[0] * F[1] + F[3] * F[4] + F[6] * F[7];
        double C02 = F[0] * F[2] + F[3] * F[5] + F[6] * F[8];
        double C12 = F[1] * F[2] + F[4] * F[5] + F[7] * F[8];
        double trE = 0.5 * ((C00 - 1.0) + (C11 - 1.0) + (C22 - 1.0));
        double h = 0.5 * m.mu2 * wJ, dg = m.lam_stvk * trE * wJ;
        double S00 = h * (C00 - 1.0) + dg, S11 = h * (C11 - 1.0) + dg, S22 = h * (C22 - 1.0) + dg;
        double S01 = h * C01, S02 = h * C02, S12 = h * C12;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            double f0 = F[i * 3], f1 = F[i * 3 + 1], f2 = F[i * 3 + 2];
            P[i * 3 + 0] = f0 * S00 + f1 * S01 + f2 * S02;
            P[i * 3 + 1] = f0 * S01 + f1 * S11 + f2 * S12;
            P[i * 3 + 2] = f0 * S02 + f1 * S12 + f2 * S22;
        }
        return;
    }
    double K[9];
    cofactor(F, K);
    double J = F[0] * K[0] + F[1] * K[1] + F[2] * K[2];
    double iJ = 1.0 / J;
    double a1, g;
    if (m.law == 1) {
        // P = mu F + (lambda ln J - mu) F^-T
        a1 = m.mu * wJ;
        g = (m.lambda * log_near1(J) - m.mu) * iJ * wJ;
    } else {
        // P = mu J^-2/3 F + (-mu/3 trB J^-5/3 + K1 (J-1)) cof(F)
        double r = rcbrt(J);
        double j23 = r * r;
        double trB = 0;
#pragma unroll
        for (int k = 0; k < 9; k++) trB += F[k] * F[k];
        a1 = m.mu * j23 * wJ;
        g = (-(m.mu / 3.0) * trB * j23 * iJ + m.K1 * (J - 1.0)) * wJ;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) P[k] = a1 * F[k] + g * K[k];
}

// Inscribed-sphere diameter from the three edge vectors at vertex 0:
// 2 r = 2 |e1.(e2 x e3)| / (|e1xe2| + |e1xe3| + |e2xe3| + |(e2-e1)x(e3-e1)|).
template <typename T>
__device__ __forceinline__ T char_length_edges(const T *e1, const T *e2, const T *e3)
{
    T A0 = e1[1] * e2[2] - e1[2] * e2[1], A1 = e1[2] * e2[0] - e1[0] * e2[2], A2 = e1[0] * e2[1] - e1[1] * e2[0];
    T B0 = e1[1] * e3[2] - e1[2] * e3[1], B1 = e1[2] * e3[0] - e1[0] * e3[2], B2 = e1[0] * e3[1] - e1[1] * e3[0];
    T C0 = e2[1] * e3[2] - e2[2] * e3[1], C1 = e2[2] * e3[0] - e2[0] * e3[2], C2 = e2[0] * e3[1] - e2[1] * e3[0];
    T D0 = C0 + A0 - B0, D1 = C1 + A1 - B1, D2 = C2 + A2 - B2;
    T s = sqrt(A0 * A0 + A1 * A1 + A2 * A2) + sqrt(B0 * B0 + B1 * B1 + B2 * B2) +
          sqrt(C0 * C0 + C1 * C1 + C2 * C2) + sqrt(D0 * D0 + D1 * D1 + D2 * D2);
    T v6 = fabs(e1[0] * C0 + e1[1] * C1 + e1[2] * C2);
    return T(2) * v6 / s;
}

// Exact FP64 CFL value of one element, min(L_ref, L(X+u)) / c, for the
// elements the FP32 screen keeps (solvers.cpp:296-320).
static __device__ __noinline__ double cfl_fp64(const Problem &p, long long e)
{
    const long long nn = p.nn;
    int4 cn = p.conn[e];
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double x0[3], e1[3], e2[3], e3[3];
#pragma unroll
    for (int k = 0; k < 3; k++) x0[k] = p.X[k * nn + nd[0]] + p.u[k * nn + nd[0]];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        e1[k] = (p.X[k * nn + nd[1]] + p.u[k * nn + nd[1]]) - x0[k];
        e2[k] = (p.X[k * nn + nd[2]] + p.u[k * nn + nd[2]]) - x0[k];
        e3[k] = (p.X[k * nn + nd[3]] + p.u[k * nn + nd[3]]) - x0[k];
    }
    double dist = char_length_edges<double>(e1, e2, e3);
    double Lr = p.Lref[e];
    return ((dist < Lr) ? dist : Lr) / mat_of(p, e).c;
}

// x rounded toward zero to FP32 with integer operations only (the FP64->FP32
// conversion instruction would take the FP64 pipe): relative error below
// 2^-23 in FP32's normal range, signed zero below it, signed infinity above.
__device__ __forceinline__ float f32_trunc(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned sign = hi & 0x80000000u;
    const int ex = (int)((hi >> 20) & 0x7FFu) - (1023 - 127);
    const unsigned mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned r = ex <= 0 ? sign : (ex >= 255 ? (sign | 0x7F800000u) : (sign | ((unsigned)ex << 23) | mant));
    return __uint_as_float(r);
}

// FP32 estimate of an element's CFL value: the reference edges X_b - X_0 are
// the columns of G^-1 (g: the rows of G, the gradients of shape functions
// 1-3, in FP32), cof(G)^T / det G, plus the displacement differences du.  Its
// relative error stays below ~3e-4 unless the tet is a sliver (6V below
// 0.063 |e1||e2||e3|, where the FP32 inverse loses accuracy) or a reference
// sliver (a negative Lref32, set at set-up); those are returned as -1 so that
// the caller always recomputes them in FP64.  The same screen as the mixed
// kernel's, with no streamed edge data.
__device__ __forceinline__ float cfl_screen_edges(const Problem &p, long long e, const float *e1, const float *e2,
                                                  const float *e3, const MatParams &m)
{
    const float C0 = e2[1] * e3[2] - e2[2] * e3[1], C1 = e2[2] * e3[0] - e2[0] * e3[2],
                C2 = e2[0] * e3[1] - e2[1] * e3[0];
    const float v6 = fabsf(e1[0] * C0 + e1[1] * C1 + e1[2] * C2);
    const float l1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
    const float l2 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
    const float l3 = e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2];
    const float dist = char_length_edges<float>(e1, e2, e3);
    const float Lr = __ldg(p.Lref32 + e);
    const float dt = ((dist < Lr) ? dist : Lr) * m.inv_c_f;
    const bool sliver = !(v6 * v6 >= 4e-3f * l1 * l2 * l3) || !(dt > 0.0f);
    return sliver ? -1.0f : dt;
}

__device__ __forceinline__ float cfl_screen(const Problem &p, long long e, const float *g, const float *du,
                                            const MatParams &m)
{
    float C[9];
    C[0] = g[4] * g[8] - g[5] * g[7];
    C[1] = g[5] * g[6] - g[3] * g[8];
    C[2] = g[3] * g[7] - g[4] * g[6];
    C[3] = g[2] * g[7] - g[1] * g[8];
    C[4] = g[0] * g[8] - g[2] * g[6];
    C[5] = g[1] * g[6] - g[0] * g[7];
    C[6] = g[1] * g[5] - g[2] * g[4];
    C[7] = g[2] * g[3] - g[0] * g[5];
    C[8] = g[0] * g[4] - g[1] * g[3];
    const float idet = 1.0f / (g[0] * C[0] + g[1] * C[1] + g[2] * C[2]);
    float e1[3], e2[3], e3[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        e1[i] = C[i] * idet + du[i];
        e2[i] = C[3 + i] * idet + du[3 + i];
        e3[i] = C[6 + i] * idet + du[6 + i];
    }
    return cfl_screen_edges(p, e, e1, e2, e3, m);
}

// Plain FP64, compressible neo-Hookean, without forming F: with the deformed
// edges e_b = E_b + (u_b - u_0) (b = 1..3, E_b the reference edges), the
// corner force of node a = 1..3 is
//   f_a = wJ P g_a = wJ mu F g_a + wJ (lambda ln J - mu) F^-T g_a,
//   F g_a = sum_b M_ab e_b        (F = I + du G and E G = I give F = e G, and
//                                  G g_a = (g_b . g_a)_b = M_a),
//   F^-T g_a = (e_c x e_d) / det e   (the rows of e^-1: e2 x e3, e3 x e1, e1 x e2),
//   J = det e / det E,
// and f_0 = -(f_1 + f_2 + f_3): about 113 FP64 operations per element instead
// of the cofactor form's 130.  The CFL screen takes the deformed edges
// directly (truncated to FP32).
template <bool ACT>
__device__ __forceinline__ float elem_body_fp64_cnh(const Problem &p, long long e, int parity, double t,
                                                    const MatParams &m, const int *nd)
{
    const long long ne = p.ne, nn = p.nn;
    double ua[4][3];
    if (p.u4) {
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const double2 xy = __ldg(reinterpret_cast<const double2 *>(p.u4) + 2LL * nd[a]);
            ua[a][0] = xy.x;
            ua[a][1] = xy.y;
            ua[a][2] = __ldg(p.u4 + 4LL * nd[a] + 2);
        }
    } else {
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) ua[a][i] = p.u[nd[a] + i * nn];
    }
    double ed[9];   // ed[(b-1)*3 + i]: component i of the deformed edge e_b
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int i = 0; i < 3; i++) ed[b * 3 + i] = __ldg(p.Eref + (b * 3 + i) * ne + e) + (ua[b + 1][i] - ua[0][i]);
    float scr;
    {
        float e32[9];
#pragma unroll
        for (int k = 0; k < 9; k++) e32[k] = f32_trunc(ed[k]);
        scr = cfl_screen_edges(p, e, e32, e32 + 3, e32 + 6, m);
    }
    const double *e1 = ed, *e2 = ed + 3, *e3 = ed + 6;
    double cr[9];   // cr[(a-1)*3 + i] = det(e) (F^-T g_a)_i
    cr[0] = e2[1] * e3[2] - e2[2] * e3[1];
    cr[1] = e2[2] * e3[0] - e2[0] * e3[2];
    cr[2] = e2[0] * e3[1] - e2[1] * e3[0];
    cr[3] = e3[1] * e1[2] - e3[2] * e1[1];
    cr[4] = e3[2] * e1[0] - e3[0] * e1[2];
    cr[5] = e3[0] * e1[1] - e3[1] * e1[0];
    cr[6] = e1[1] * e2[2] - e1[2] * e2[1];
    cr[7] = e1[2] * e2[0] - e1[0] * e2[2];
    cr[8] = e1[0] * e2[1] - e1[1] * e2[0];
    const double dete = e1[0] * cr[0] + e1[1] * cr[1] + e1[2] * cr[2];
    const double J = dete * __ldg(p.rdetE + e);
    const double wJ = __ldg(p.wJ + e);
    const double c1 = m.mu * wJ;
    const double c2 = (m.lambda * log_near1(J) - m.mu) * (wJ / dete);
    double Mv[6];
#pragma unroll
    for (int k = 0; k < 6; k++) Mv[k] = __ldg(p.Mg + k * ne + e);
    const int mi[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};   // M_ab at Mv[mi[(a-1)*3 + (b-1)]]
    double f[12];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const double Fg = e1[i] * Mv[mi[a * 3]] + e2[i] * Mv[mi[a * 3 + 1]] + e3[i] * Mv[mi[a * 3 + 2]];
            f[(a + 1) * 3 + i] = c1 * Fg + c2 * cr[a * 3 + i];
        }
#pragma unroll
    for (int i = 0; i < 3; i++) f[i] = -(f[3 + i] + f[6 + i] + f[9 + i]);
    if (ACT && elem_dead(p, e, t))
#pragma unroll
        for (int k = 0; k < 12; k++) f[k] = 0.0;
    const int4 sl = __ldg(p.slot + e);
    const int ks[4] = {sl.x, sl.y, sl.z, sl.w};
#pragma unroll
    for (int a = 0; a < 4; a++) st_slot24(p.fe, ks[a], f[a * 3], f[a * 3 + 1], f[a * 3 + 2]);
    if (e == 0 && !isfinite(p.u[1])) atomicOr(p.flags + (parity ^ 1), 1);
    return scr;
}

// Plain FP64 with contraction: H from node differences, laws through the
// cofactor (F C^-1 = F^-T = cof(F)/J), wJ folded into the law's coefficients,
// the 4th corner force as minus the sum of the other three.  Same algebra as
// the reference, about half its FP64 operations.  Returns the FP32 CFL screen
// value (see cfl_screen).
template <bool FORCE_ONLY, bool ACT = false, bool VISC = false>
__device__ __forceinline__ float elem_body_fp64(const Problem &p, long long e, int parity, double t = 0.0,
                                                double idt = 0.0)
{
    const long long ne = p.ne, nn = p.nn;
    int4 cn = p.conn[e];
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    const MatParams &m = mat_of(p, e);
    if (!FORCE_ONLY && !VISC && p.Eref && m.law == 1) return elem_body_fp64_cnh<ACT>(p, e, parity, t, m, nd);
    double G[9];
#pragma unroll
    for (int k = 0; k < 9; k++) G[k] = __ldg(p.G + k * ne + e);
    double u0[3], du[9];
    if (!FORCE_ONLY && p.u4) {
        double ua[4][3];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const double2 xy = __ldg(reinterpret_cast<const double2 *>(p.u4) + 2LL * nd[a]);
            ua[a][0] = xy.x;
            ua[a][1] = xy.y;
            ua[a][2] = __ldg(p.u4 + 4LL * nd[a] + 2);
        }
#pragma unroll
        for (int a = 1; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) du[(a - 1) * 3 + i] = ua[a][i] - ua[0][i];
    } else {
#pragma unroll
        for (int i = 0; i < 3; i++) u0[i] = p.u[nd[0] + i * nn];
#pragma unroll
        for (int a = 1; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) du[(a - 1) * 3 + i] = p.u[nd[a] + i * nn] - u0[i];
    }
    double F[9], P[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            // the identity enters the FMA chain (no separate 0 + x or 1 + x)
            F[i * 3 + j] = fma(du[i], G[j], fma(du[3 + i], G[3 + j], i == j ? fma(du[6 + i], G[6 + j], 1.0)
                                                                             : du[6 + i] * G[6 + j]));
    float scr = 0.0f;
    if (!FORCE_ONLY) {   // the CFL screen first, so du dies before the stress
        float du32[9], g32[9];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            du32[k] = f32_trunc(du[k]);
            g32[k] = f32_trunc(G[k]);
        }
        scr = cfl_screen(p, e, g32, du32, m);
    }
    stress_fast(m, F, __ldg(p.wJ + e), P);
    if (VISC && !FORCE_ONLY) {
        double Pv[9];
        visc_bulk_fp64(p, e, F, __ldg(p.wJ + e), m.rho, idt, Pv);
#pragma unroll
        for (int k = 0; k < 9; k++) P[k] += Pv[k];
    }
    double f[12];
#pragma unroll
    for (int a = 1; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++)
            f[a * 3 + i] = P[i * 3] * G[(a - 1) * 3] + P[i * 3 + 1] * G[(a - 1) * 3 + 1] + P[i * 3 + 2] * G[(a - 1) * 3 + 2];
#pragma unroll
    for (int i = 0; i < 3; i++) f[i] = -(f[3 + i] + f[6 + i] + f[9 + i]);
    if (ACT && elem_dead(p, e, t))
#pragma unroll
        for (int k = 0; k < 12; k++) f[k] = 0.0;
    const int4 sl = __ldg(p.slot + e);
    const int ks[4] = {sl.x, sl.y, sl.z, sl.w};
#pragma unroll
    for (int a = 0; a < 4; a++) st_slot24(p.fe, ks[a], f[a * 3], f[a * 3 + 1], f[a * 3 + 2]);
    if (FORCE_ONLY) return 0.0f;
    if (e == 0 && !isfinite(p.u[1])) atomicOr(p.flags + (parity ^ 1), 1);
    return scr;
}

// corner forces only (internal-force hook)
static __global__ void __launch_bounds__(kElemBlock) elem_force_kernel_fp64(Problem p, int parity)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < p.ne) elem_body_fp64<true>(p, e, parity);
}

// ---------------------------------------------------------------------------
// Mixed precision: FP32 kinematics, stress and B^T P written in terms of the
// displacement gradient H = F - I (no 1 - 1 cancellation in FP32); J - 1 and
// ln J in FP32 with an exactly summed trace; FP32 corner forces; an FP32
// screen of the CFL values whose near-minimum elements are recomputed in FP64
// (cfl_dw), so the stable dt is the FP64 minimum.
// cof(I + H) = I + D with D = (tr H + I2) I - (1 + tr H) H^T + (H^2)^T.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void stress_mixed(const MatParams &m, const float *H, float Jm1, float lnJ,
                                             float t, float I2, float *P)
{
    if (m.law == 3) {
        // linear elastic: P = mu2 E + lam tr(E) I with E = (H + H^T)/2
        const float dg = m.lam_stvk_f * t;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++)
                P[i * 3 + j] = m.mu2_f * (0.5f * (H[i * 3 + j] + H[j * 3 + i])) + (i == j ? dg : 0.0f);
        return;
    }
    if (m.law == 2) {
        // E = (H + H^T + H^T H)/2, S = mu2 E + lam tr(E) I, P = (I + H) S
        float E[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++)
                E[i * 3 + j] = 0.5f * (H[i * 3 + j] + H[j * 3 + i] +
                                       (H[i] * H[j] + H[3 + i] * H[3 + j] + H[6 + i] * H[6 + j]));
        float trE = E[0] + E[4] + E[8];
        float S[9];
#pragma unroll
        for (int k = 0; k < 9; k++) S[k] = m.mu2_f * E[k];
        S[0] += m.lam_stvk_f * trE;
        S[4] += m.lam_stvk_f * trE;
        S[8] += m.lam_stvk_f * trE;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++)
                P[i * 3 + j] = S[i * 3 + j] + (H[i * 3] * S[j] + H[i * 3 + 1] * S[3 + j] + H[i * 3 + 2] * S[6 + j]);
        return;
    }
    float D[9];
    float a0 = t + I2, a1 = 1.0f + t;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            // (H^2)^T_ij = sum_k H_jk H_ki
            float h2 = H[j * 3] * H[i] + H[j * 3 + 1] * H[3 + i] + H[j * 3 + 2] * H[6 + i];
            D[i * 3 + j] = (i == j ? a0 : 0.0f) - a1 * H[j * 3 + i] + h2;
        }
    float iJ = 1.0f / (1.0f + Jm1);
    if (m.law == 1) {
        // P = [mu (Jm1 I + (1+Jm1) H - D) + lambda lnJ (I + D)] / J
        float lj = m.lambda_f * lnJ;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            float dg = (k % 4 == 0) ? 1.0f : 0.0f;
            P[k] = (m.mu_f * (Jm1 * dg + (1.0f + Jm1) * H[k] - D[k]) + lj * (dg + D[k])) * iJ;
        }
    } else {
        // P = mu J^-2/3 [(Jm1 - beta) I + (1+Jm1) H - (1+beta) D]/J + K Jm1 (I + D)
        float hh = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; k++) hh += H[k] * H[k];
        float beta = (2.0f * t + hh) * (1.0f / 3.0f);
        float j23 = expf(-(2.0f / 3.0f) * lnJ) * m.mu_f * iJ;
        float kj = m.K1_f * Jm1;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            float dg = (k % 4 == 0) ? 1.0f : 0.0f;
            P[k] = j23 * ((Jm1 - beta) * dg + (1.0f + Jm1) * H[k] - (1.0f + beta) * D[k]) + kj * (dg + D[k]);
        }
    }
}

template <bool FORCE_ONLY, bool ACT = false, bool VISC = false>
__device__ __forceinline__ float elem_body_mixed(const Problem &p, long long e, int parity, int4 cn, double t = 0.0,
                                                 float idtf = 0.0f)
{
    const long long ne = p.ne, nn = p.nn;
    float vmin = INFINITY;
    {
        int nd[4] = {cn.x, cn.y, cn.z, cn.w};
        float G[9];
#pragma unroll
        for (int k = 0; k < 9; k++) G[k] = __ldg(p.G32 + k * ne + e);
        // du = u_a - u_0 from the (hi, lo) split: the hi difference is exact for
        // nearby values, the lo difference restores the bits FP32 drops
        float2 h0[3];
#pragma unroll
        for (int i = 0; i < 3; i++) h0[i] = p.uhl[nd[0] + i * nn];
        float du[9];
#pragma unroll
        for (int a = 1; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) {
                float2 ha = p.uhl[nd[a] + i * nn];
                du[(a - 1) * 3 + i] = (ha.x - h0[i].x) + (ha.y - h0[i].y);
            }
        float H[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) H[i * 3 + j] = du[i] * G[j] + du[3 + i] * G[3 + j] + du[6 + i] * G[6 + j];
        // J - 1 = tr H + (I2(H) + det H).  The trace carries J - 1 and may
        // cancel (nearly isochoric motion), so it is summed without rounding,
        // as s + err by TwoSum; I2 and det H are O(|H|^2) and their FP32
        // rounding lies far below the FP32 precision of J - 1.  So J - 1 is
        // good to FP32 relative precision, and so is ln J = log1p(J - 1);
        // F = I + H is never formed or reduced.
        float tf = H[0] + H[4] + H[8];
        float I2f = (H[0] * H[4] - H[1] * H[3]) + (H[4] * H[8] - H[5] * H[7]) + (H[0] * H[8] - H[2] * H[6]);
        float I3f = H[0] * (H[4] * H[8] - H[5] * H[7]) - H[1] * (H[3] * H[8] - H[5] * H[6]) +
                    H[2] * (H[3] * H[7] - H[4] * H[6]);
        const float s1 = H[0] + H[4], s2 = s1 + H[8];
        const float terr = two_sum_err(H[0], H[4], s1) + two_sum_err(s1, H[8], s2);
        const float Jm1 = s2 + (terr + (I2f + I3f));
        const float lnJ = log1pf(Jm1);
        const MatParams &m = mat_of(p, e);
        float P[9];
        stress_mixed(m, H, Jm1, lnJ, tf, I2f, P);
        if (VISC && !FORCE_ONLY) {
            // bulk viscosity in FP32: P += qBV cof(I + H) = qBV (I + D), D as in stress_mixed
            float *h0 = p.visc_h0;
            const float trD = ((H[0] - h0[e]) + (H[4] - h0[ne + e]) + (H[8] - h0[2 * ne + e])) * idtf;
            h0[e] = H[0];
            h0[ne + e] = H[4];
            h0[2 * ne + e] = H[8];
            const float q = m.rho_f / (1.0f + Jm1) * p.visc_hf *
                            (p.visc_c1sq_hf * fabsf(trD) * fminf(0.0f, trD) + p.visc_clc0f * trD);
            const float a0 = tf + I2f, a1 = 1.0f + tf;
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    const float h2 = H[j * 3] * H[i] + H[j * 3 + 1] * H[3 + i] + H[j * 3 + 2] * H[6 + i];
                    const float Dij = (i == j ? a0 : 0.0f) - a1 * H[j * 3 + i] + h2;
                    P[i * 3 + j] += q * ((i == j ? 1.0f : 0.0f) + Dij);
                }
        }
        float wJ = __ldg(p.wJ32 + e);
#pragma unroll
        for (int k = 0; k < 9; k++) P[k] *= wJ;
        float f[12];
#pragma unroll
        for (int a = 1; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++)
                f[a * 3 + i] = P[i * 3] * G[(a - 1) * 3] + P[i * 3 + 1] * G[(a - 1) * 3 + 1] +
                               P[i * 3 + 2] * G[(a - 1) * 3 + 2];
#pragma unroll
        for (int i = 0; i < 3; i++) f[i] = -(f[3 + i] + f[6 + i] + f[9 + i]);
        if (ACT && elem_dead(p, e, t))
#pragma unroll
            for (int k = 0; k < 12; k++) f[k] = 0.f;
        // one 16-byte store per corner (a padded slot) rather than three scalar ones
        const int4 sl = __ldg(p.slot + e);
        float4 *fe = reinterpret_cast<float4 *>(p.fe32);
        fe[sl.x] = make_float4(f[0], f[1], f[2], 0.f);
        fe[sl.y] = make_float4(f[3], f[4], f[5], 0.f);
        fe[sl.z] = make_float4(f[6], f[7], f[8], 0.f);
        fe[sl.w] = make_float4(f[9], f[10], f[11], 0.f);
        if (!FORCE_ONLY) {
            // reference edges X_b - X_0 = columns of G^-1 (G's rows are the
            // gradients of shape functions 1-3): cof(G)^T / det G in FP32,
            // instead of streaming them; only the CFL value uses them
            float C[9];
            C[0] = G[4] * G[8] - G[5] * G[7];
            C[1] = G[5] * G[6] - G[3] * G[8];
            C[2] = G[3] * G[7] - G[4] * G[6];
            C[3] = G[2] * G[7] - G[1] * G[8];
            C[4] = G[0] * G[8] - G[2] * G[6];
            C[5] = G[1] * G[6] - G[0] * G[7];
            C[6] = G[1] * G[5] - G[2] * G[4];
            C[7] = G[2] * G[3] - G[0] * G[5];
            C[8] = G[0] * G[4] - G[1] * G[3];
            const float idet = 1.0f / (G[0] * C[0] + G[1] * C[1] + G[2] * C[2]);
            float e1[3], e2[3], e3[3];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                e1[i] = C[i] * idet + du[i];
                e2[i] = C[3 + i] * idet + du[3 + i];
                e3[i] = C[6 + i] * idet + du[6 + i];
            }
            // FP32 screen of the CFL value, as cfl_screen: slivers (6V below
            // 0.063 |e1||e2||e3|, where the FP32 edges lose accuracy) and
            // reference slivers (a negative Lref32, set at set-up) come back
            // negative, so the caller recomputes them in FP64
            const float C0 = e2[1] * e3[2] - e2[2] * e3[1], C1 = e2[2] * e3[0] - e2[0] * e3[2],
                        C2 = e2[0] * e3[1] - e2[1] * e3[0];
            const float v6 = fabsf(e1[0] * C0 + e1[1] * C1 + e1[2] * C2);
            const float l1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
            const float l2 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
            const float l3 = e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2];
            float dist = char_length_edges<float>(e1, e2, e3);
            float Lr = __ldg(p.Lref32 + e);
            vmin = ((dist < Lr) ? dist : Lr) * m.inv_c_f;
            if (!(v6 * v6 >= 4e-3f * l1 * l2 * l3) || !(vmin > 0.0f)) vmin = -1.0f;
            if (e == 0 && !isfinite(p.uhl[1].x)) atomicOr(p.flags + (parity ^ 1), 1);
        }
    }
    return vmin;
}

// corner forces only (internal-force hook)
static __global__ void __launch_bounds__(kElemBlock) elem_force_kernel_mixed(Problem p, int parity)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < p.ne) elem_body_mixed<true>(p, e, parity, p.conn[e]);
}


// ---------------------------------------------------------------------------
// Double-word mode: the algebra of elem_body_fp64 (F from node differences,
// the laws through cof(F), B^T P with wJ folded in) evaluated in double-word
// arithmetic on the FP32 pipe, with the nodal state and the corner forces as
// double-words too.  A double-word operation costs 4-20 FP32 operations and
// carries about 2^-47 relative error against FP64's 2^-53; on this GPU the
// FP64 pipe issues 1/64 of the FP32 rate, so the element work runs several
// times faster than in FP64 while results stay within a few 1e-13 of it.
// The error-free pieces (TwoSum, Fast2Sum, the FMA product split) use the
// _rn intrinsics, which the compiler never fuses into an FMA.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float dw_err(float a, float b, float s)   // a + b - s for s = fl(a + b)
{
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ float2 dw_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return make_float2(s, dw_err(a, b, s));
}

__device__ __forceinline__ float2 dw_fast(float a, float b)   // |a| >= |b| or a = 0
{
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ float2 dw_neg(float2 x) { return make_float2(-x.x, -x.y); }
__device__ __forceinline__ float2 dw_scale2(float2 x, float p2) { return make_float2(x.x * p2, x.y * p2); }  // p2 = 2^k

// Joldes, Muller, Popescu (2017) Alg. 6 (accurate sum), Alg. 12 (product),
// Alg. 4 (double-word + FP32), Alg. 9 (double-word * FP32).
__device__ __forceinline__ float2 dw_add(float2 x, float2 y)
{
    const float2 s = dw_two_sum(x.x, y.x), t = dw_two_sum(x.y, y.y);
    const float2 v = dw_fast(s.x, __fadd_rn(s.y, t.x));
    return dw_fast(v.x, __fadd_rn(t.y, v.y));
}

// x + y with absolute error a few 2^-48 (|x| + |y|) (the "sloppy" sum, JMP
// Alg. 5): enough where the inputs' own rounding is of that size, as for node
// differences and sums of corner forces; no bound relative to |x + y|.
__device__ __forceinline__ float2 dw_add_sloppy(float2 x, float2 y)
{
    const float2 s = dw_two_sum(x.x, y.x);
    return dw_fast(s.x, __fadd_rn(s.y, __fadd_rn(x.y, y.y)));
}

__device__ __forceinline__ float2 dw_mul(float2 x, float2 y)
{
    const float ch = __fmul_rn(x.x, y.x);
    const float cl1 = fmaf(x.x, y.x, -ch);
    const float cl2 = fmaf(x.y, y.x, fmaf(x.x, y.y, __fmul_rn(x.y, y.y)));
    return dw_fast(ch, __fadd_rn(cl1, cl2));
}

__device__ __forceinline__ float2 dw_add_f(float2 x, float y)
{
    const float2 s = dw_two_sum(x.x, y);
    return dw_fast(s.x, __fadd_rn(x.y, s.y));
}

__device__ __forceinline__ float2 dw_mul_f(float2 x, float y)
{
    const float ch = __fmul_rn(x.x, y);
    return dw_fast(ch, fmaf(x.y, y, fmaf(x.x, y, -ch)));
}

__device__ __forceinline__ float2 dw_from(double x)
{
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// Compensated dot products of double-words (Ogita, Rump, Oishi, "Accurate sum
// and dot product", SIAM J. Sci. Comput. 26 (2005), Dot2, with the low words'
// cross terms): each hi*hi product is split exactly by an FMA and summed with
// TwoSum; the product and sum errors and the hi*lo terms gather in one FP32
// correction c.  Result s + c by Fast2Sum (exact unless the sum cancels below
// |c|, where its error is still of the order 2^-48 sum |a_k b_k|); error a few
// 2^-48 sum |a_k b_k|, the size of FP64's 2^-53 sum |a_k b_k| times ~30.
__device__ __forceinline__ void dw_acc(float &s, float &c, float2 x, float2 y)
{
    const float p = __fmul_rn(x.x, y.x);
    c = fmaf(x.y, y.x, fmaf(x.x, y.y, c + fmaf(x.x, y.x, -p)));
    const float t = __fadd_rn(s, p);
    c += dw_err(s, p, t);
    s = t;
}

__device__ __forceinline__ float2 dw_dot2(float2 a0, float2 b0, float2 a1, float2 b1)
{
    float s = __fmul_rn(a0.x, b0.x);
    float c = fmaf(a0.y, b0.x, fmaf(a0.x, b0.y, fmaf(a0.x, b0.x, -s)));
    dw_acc(s, c, a1, b1);
    return dw_fast(s, c);
}

// init + a0 b0 + a1 b1 + a2 b2 (init an FP32 constant, e.g. the identity's 1)
__device__ __forceinline__ float2 dw_dot3(float2 a0, float2 b0, float2 a1, float2 b1, float2 a2, float2 b2,
                                          float init)
{
    float s, c;
    if (init == 0.0f) {   // a constant at every call: resolved at compile time
        s = __fmul_rn(a0.x, b0.x);
        c = fmaf(a0.y, b0.x, fmaf(a0.x, b0.y, fmaf(a0.x, b0.x, -s)));
    } else {
        s = init;
        c = 0.0f;
        dw_acc(s, c, a0, b0);
    }
    dw_acc(s, c, a1, b1);
    dw_acc(s, c, a2, b2);
    return dw_fast(s, c);
}

// ln(1 + x) for a double-word x.  For |x| < 2^-7: x - x^2/2 + x^3/3 in
// double-words plus the tail x^4 (-1/4 + x/5 - x^2/6 + x^3/7 - x^4/8) in FP32
// (|tail| < 2^-21 |x|, so its FP32 rounding stays below 2^-45 |x|; the next
// term is below 2^-56 |x|).  Otherwise the FP64 library log.
__device__ __forceinline__ float2 dw_log1p(float2 x)
{
    if (!(fabsf(x.x) < 0.0078125f)) return dw_from(log(1.0 + ((double)x.x + (double)x.y)));
    const float2 third = make_float2(0x1.555556p-2f, -0x1.555556p-27f);
    const float2 x2 = dw_mul(x, x), x3 = dw_mul(x2, x);
    const float2 lead = dw_add(dw_add(x, dw_scale2(x2, -0.5f)), dw_mul(x3, third));
    const float xf = x.x;
    const float tail = (x2.x * x2.x) * fmaf(xf, fmaf(xf, fmaf(xf, fmaf(xf, -0.125f, 1.0f / 7.0f), -1.0f / 6.0f), 0.2f), -0.25f);
    return dw_add_f(lead, tail);
}

// 1 / y: one Newton step from the FP32 reciprocal.
__device__ __forceinline__ float2 dw_rcp(float2 y)
{
    const float r0 = __frcp_rn(y.x);
    const float2 p = dw_mul_f(y, r0);                       // y r0 = 1 - e
    const float e = __fsub_rn(__fsub_rn(1.0f, p.x), p.y);
    return dw_fast(r0, __fmul_rn(r0, e));
}

// wJ * P through the cofactor, as stress_fast does in FP64.
__device__ __forceinline__ void stress_dw(const MatParams &m, const float2 *F, float2 wJ, float2 *P)
{
    if (m.law == 3) {
        // linear elastic: wJ P = wJ (mu2 E + lam tr(E) I), E = (F + F^T)/2 - I
        const float2 h = dw_mul(m.mu2_w, wJ);
        const float2 E00 = dw_add_f(F[0], -1.0f), E11 = dw_add_f(F[4], -1.0f), E22 = dw_add_f(F[8], -1.0f);
        const float2 dg = dw_mul(dw_mul(m.lam_stvk_w, dw_add(dw_add(E00, E11), E22)), wJ);
        P[0] = dw_add(dw_mul(h, E00), dg);
        P[4] = dw_add(dw_mul(h, E11), dg);
        P[8] = dw_add(dw_mul(h, E22), dg);
        P[1] = P[3] = dw_mul(h, dw_scale2(dw_add(F[1], F[3]), 0.5f));
        P[2] = P[6] = dw_mul(h, dw_scale2(dw_add(F[2], F[6]), 0.5f));
        P[5] = P[7] = dw_mul(h, dw_scale2(dw_add(F[5], F[7]), 0.5f));
        return;
    }
    if (m.law == 2) {
        // S = mu2 E + lam tr(E) I with E = (F^T F - I)/2; C_ii - 1 from the dot's initial -1
        const float2 C00 = dw_dot3(F[0], F[0], F[3], F[3], F[6], F[6], -1.0f);
        const float2 C11 = dw_dot3(F[1], F[1], F[4], F[4], F[7], F[7], -1.0f);
        const float2 C22 = dw_dot3(F[2], F[2], F[5], F[5], F[8], F[8], -1.0f);
        const float2 C01 = dw_dot3(F[0], F[1], F[3], F[4], F[6], F[7], 0.0f);
        const float2 C02 = dw_dot3(F[0], F[2], F[3], F[5], F[6], F[8], 0.0f);
        const float2 C12 = dw_dot3(F[1], F[2], F[4], F[5], F[7], F[8], 0.0f);
        const float2 trE = dw_scale2(dw_add(dw_add(C00, C11), C22), 0.5f);
        const float2 h = dw_scale2(dw_mul(m.mu2_w, wJ), 0.5f), dg = dw_mul(dw_mul(m.lam_stvk_w, trE), wJ);
        const float2 S00 = dw_add(dw_mul(h, C00), dg), S11 = dw_add(dw_mul(h, C11), dg),
                     S22 = dw_add(dw_mul(h, C22), dg);
        const float2 S01 = dw_mul(h, C01), S02 = dw_mul(h, C02), S12 = dw_mul(h, C12);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float2 f0 = F[i * 3], f1 = F[i * 3 + 1], f2 = F[i * 3 + 2];
            P[i * 3 + 0] = dw_dot3(f0, S00, f1, S01, f2, S02, 0.0f);
            P[i * 3 + 1] = dw_dot3(f0, S01, f1, S11, f2, S12, 0.0f);
            P[i * 3 + 2] = dw_dot3(f0, S02, f1, S12, f2, S22, 0.0f);
        }
        return;
    }
    float2 K[9];
    K[0] = dw_dot2(F[4], F[8], dw_neg(F[5]), F[7]);
    K[1] = dw_dot2(F[5], F[6], dw_neg(F[3]), F[8]);
    K[2] = dw_dot2(F[3], F[7], dw_neg(F[4]), F[6]);
    K[3] = dw_dot2(F[2], F[7], dw_neg(F[1]), F[8]);
    K[4] = dw_dot2(F[0], F[8], dw_neg(F[2]), F[6]);
    K[5] = dw_dot2(F[1], F[6], dw_neg(F[0]), F[7]);
    K[6] = dw_dot2(F[1], F[5], dw_neg(F[2]), F[4]);
    K[7] = dw_dot2(F[2], F[3], dw_neg(F[0]), F[5]);
    K[8] = dw_dot2(F[0], F[4], dw_neg(F[1]), F[3]);
    const float2 J = dw_dot3(F[0], K[0], F[1], K[1], F[2], K[2], 0.0f);
    const float2 x = dw_add_f(J, -1.0f);   // J - 1
    const float2 iJ = dw_rcp(J);
    float2 a1, g;
    if (m.law == 1) {
        // P = mu F + (lambda ln J - mu) cof(F) / J
        a1 = dw_mul(m.mu_w, wJ);
        g = dw_mul(dw_mul(dw_add(dw_mul(m.lambda_w, dw_log1p(x)), dw_neg(m.mu_w)), iJ), wJ);
    } else {
        // P = mu J^-2/3 F + (-mu/3 trB J^-5/3 + K1 (J-1)) cof(F); J^-2/3 from the FP64 library
        const double r = rcbrt((double)J.x + (double)J.y);
        const float2 j23 = dw_from(r * r);
        const float2 trB = dw_add(dw_add(dw_dot3(F[0], F[0], F[1], F[1], F[2], F[2], 0.0f),
                                         dw_dot3(F[3], F[3], F[4], F[4], F[5], F[5], 0.0f)),
                                  dw_dot3(F[6], F[6], F[7], F[7], F[8], F[8], 0.0f));
        a1 = dw_mul(dw_mul(m.mu_w, j23), wJ);
        g = dw_mul(dw_add(dw_neg(dw_mul(dw_mul(dw_mul(m.mu3_w, trB), j23), iJ)), dw_mul(m.K1_w, x)), wJ);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) P[k] = dw_dot2(a1, F[k], g, K[k]);
}

// Exact FP64 CFL value of one element from the double-word displacement.
static __device__ __noinline__ double cfl_dw(const Problem &p, long long e)
{
    const long long nn = p.nn;
    int4 cn = p.conn[e];
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double x[4][3];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float2 w = p.uhl[k * nn + nd[a]];
            x[a][k] = p.X[k * nn + nd[a]] + ((double)w.x + (double)w.y);
        }
    double e1[3], e2[3], e3[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        e1[k] = x[1][k] - x[0][k];
        e2[k] = x[2][k] - x[0][k];
        e3[k] = x[3][k] - x[0][k];
    }
    double dist = char_length_edges<double>(e1, e2, e3);
    double Lr = p.Lref[e];
    return ((dist < Lr) ? dist : Lr) / mat_of(p, e).c;
}

template <bool FORCE_ONLY, bool ACT = false, bool VISC = false>
__device__ __forceinline__ float elem_body_dw(const Problem &p, long long e, int parity, int4 cn, double t = 0.0,
                                              double idt = 0.0)
{
    const long long ne = p.ne, nn = p.nn;
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    float2 G[9];
#pragma unroll
    for (int k = 0; k < 9; k++) G[k] = make_float2(__ldg(p.G32 + k * ne + e), __ldg(p.G32lo + k * ne + e));
    float2 u0[3], du[9];
#pragma unroll
    for (int i = 0; i < 3; i++) u0[i] = p.uhl[nd[0] + i * nn];
#pragma unroll
    for (int a = 1; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++) du[(a - 1) * 3 + i] = dw_add_sloppy(p.uhl[nd[a] + i * nn], dw_neg(u0[i]));
    float2 F[9], P[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            F[i * 3 + j] = dw_dot3(du[i], G[j], du[3 + i], G[3 + j], du[6 + i], G[6 + j], i == j ? 1.0f : 0.0f);
    const MatParams &m = mat_of(p, e);
    stress_dw(m, F, make_float2(__ldg(p.wJ32 + e), __ldg(p.wJ32lo + e)), P);
    if (VISC && !FORCE_ONLY) {
        // bulk viscosity in FP64 from the double-word F (exact as doubles), added as double-words
        double Fd[9], Pv[9];
#pragma unroll
        for (int k = 0; k < 9; k++) Fd[k] = (double)F[k].x + (double)F[k].y;
        visc_bulk_fp64(p, e, Fd, (double)__ldg(p.wJ32 + e) + (double)__ldg(p.wJ32lo + e), m.rho, idt, Pv);
#pragma unroll
        for (int k = 0; k < 9; k++) P[k] = dw_add(P[k], dw_from(Pv[k]));
    }
    float2 f[12];
#pragma unroll
    for (int a = 1; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++)
            f[a * 3 + i] = dw_dot3(P[i * 3], G[(a - 1) * 3], P[i * 3 + 1], G[(a - 1) * 3 + 1], P[i * 3 + 2],
                                   G[(a - 1) * 3 + 2], 0.0f);
#pragma unroll
    for (int i = 0; i < 3; i++) f[i] = dw_neg(dw_add_sloppy(dw_add_sloppy(f[3 + i], f[6 + i]), f[9 + i]));
    if (ACT && elem_dead(p, e, t))
#pragma unroll
        for (int k = 0; k < 12; k++) f[k] = make_float2(0.f, 0.f);
    const int4 sl = __ldg(p.slot + e);
    const int ks[4] = {sl.x, sl.y, sl.z, sl.w};
    float2 *fe = reinterpret_cast<float2 *>(p.fe);
#pragma unroll
    for (int a = 0; a < 4; a++) {
        float2 *fk = fe + (long long)ks[a] * 3;
        fk[0] = f[a * 3];
        fk[1] = f[a * 3 + 1];
        fk[2] = f[a * 3 + 2];
    }
    if (FORCE_ONLY) return 0.0f;
    if (e == 0 && !isfinite(p.uhl[1].x)) atomicOr(p.flags + (parity ^ 1), 1);
    float du32[9], g32[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        du32[k] = du[k].x;
        g32[k] = G[k].x;
    }
    return cfl_screen(p, e, g32, du32, m);
}

// corner forces only (internal-force hook)
static __global__ void __launch_bounds__(kElemBlock) elem_force_kernel_dw(Problem p, int parity)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < p.ne) elem_body_dw<true>(p, e, parity, p.conn[e]);
}

// Node body of the double-word mode: the mixed mode's four-lane gather and
// update, with double-word corner forces summed as (s, c): s the FP32 sum of
// the high words by TwoSum, c the rounding errors plus the low words.
__device__ __forceinline__ void dw_sum_merge(float &s, float &c, float s2, float c2)
{
    const float t = __fadd_rn(s, s2);
    c = c + c2 + dw_err(s, s2, t);
    s = t;
}

__device__ __forceinline__ void node_quad_dw(const Problem &p, long long i, bool valid, const NodeStep &ns)
{
    const int q = threadIdx.x & 3;
    const bool odd = q & 1;
    const bool own = valid && q < 3;
    const long long dof = i + (long long)q * p.nn;
    float2 uq = make_float2(0.f, 0.f), vq = uq, aq = uq, minv = uq;
    int rec = -1;
    if (own) {
        uq = p.uhl[dof];
        vq = p.vhl[dof];
        aq = p.ahl[dof];
        minv = p.minv2[i];
        rec = p.node_bc[i];
    }
    int k0 = 0, k1 = 0;
    if (valid && ns.ran) {
        k0 = p.node_ptr[i];
        k1 = p.node_ptr[i + 1];
    }
    const float2 *fe = reinterpret_cast<const float2 *>(p.fe);
    float h0 = 0.f, h1 = 0.f, h2 = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
    int k = k0 + q;
    if (k < k1) {
        const float2 *f = fe + (long long)k * 3;
        const float2 f0 = f[0], f1 = f[1], f2 = f[2];
        h0 = f0.x, c0 = f0.y;
        h1 = f1.x, c1 = f1.y;
        h2 = f2.x, c2 = f2.y;
        k += 4;
    }
    for (; k < k1; k += 4) {
        const float2 *f = fe + (long long)k * 3;
        const float2 f0 = f[0], f1 = f[1], f2 = f[2];
        dw_sum_merge(h0, c0, f0.x, f0.y);
        dw_sum_merge(h1, c1, f1.x, f1.y);
        dw_sum_merge(h2, c2, f2.x, f2.y);
    }
    float ah = odd ? h0 : h1, ac = odd ? c0 : c1;
    float xh = __shfl_xor_sync(0xffffffffu, ah, 1), xc = __shfl_xor_sync(0xffffffffu, ac, 1);
    float yh = __shfl_xor_sync(0xffffffffu, h2, 1), yc = __shfl_xor_sync(0xffffffffu, c2, 1);
    if (odd) {
        dw_sum_merge(h1, c1, xh, xc);
    } else {
        dw_sum_merge(h0, c0, xh, xc);
        dw_sum_merge(h2, c2, yh, yc);
    }
    float sh = odd ? h1 : (q == 0 ? h2 : h0), sc = odd ? c1 : (q == 0 ? c2 : c0);
    float zh = __shfl_xor_sync(0xffffffffu, sh, 2), zc = __shfl_xor_sync(0xffffffffu, sc, 2);
    float mh = pick3(q, h0, h1, h2), mc = pick3(q, c0, c1, c2);
    dw_sum_merge(mh, mc, zh, zc);
    if (!own) return;
    const float2 s = dw_two_sum(mh, mc);
    const int2 br = rec >= 0 ? p.bc_rec[rec * 3 + q] : make_int2(0, 0);
    const bool act = br.y == 0;
    bool changed = false;
    if (ns.ran && act) {
        const float2 f = ns.loads ? dw_add(dw_from(node_fext(p, i, q, ns)), dw_neg(s)) : dw_neg(s);
        const float2 an = dw_mul(f, minv);
        vq = dw_add(vq, dw_mul(ns.hdt2, dw_add(aq, an)));
        aq = an;
        changed = true;
    }
    if (ns.run) {
        if (act) {
            uq = dw_add(uq, dw_mul(ns.dtn2, dw_add(vq, dw_mul(ns.hdtn2, aq))));
        } else {
            for (int k = br.x; k < br.x + br.y; k++) {
                const float2 Ud = dw_from(bc_increment(p.bcs[k], ns.dtn, ns.step));
                uq = dw_add(uq, Ud);
                vq = Ud;
                aq = make_float2(0.f, 0.f);
            }
        }
        changed = true;
    }
    if (changed) {
        p.uhl[dof] = uq;
        p.vhl[dof] = vq;
        p.ahl[dof] = aq;
    }
}

// Block-wide min of a float, returned to every thread of the block.
__device__ __forceinline__ float block_min_bcast(float v);

// Reference-order element kernel with the FP32 CFL screen: forces in the
// reference's order for every element, the exact reference-order CFL value only
// for the elements of the block within 2^-8 of its FP32 minimum (and slivers),
// a set that always holds the block's exact minimum, so dt is the reference's.
template <bool VISC>
__global__ void __launch_bounds__(kElemBlock) elem_kernel_exact_screened(Problem p, int parity)
{
    if (!p.ctrl[parity].ran) return;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const float d = e < p.ne ? (float)elem_body_exact<false, true, VISC>(p, e, parity) : INFINITY;
    const float bmin = block_min_bcast(d >= 0.0f ? d : INFINITY);
    double v = INFINITY;
    if (e < p.ne && (d < 0.0f || d <= bmin * (1.0f + 1.0f / 256.0f))) v = cfl_exact_ref(p, e);
    block_min_to(v, p.dtmin + (parity ^ 1));
}

__device__ __forceinline__ float block_min_bcast(float v)
{
    __shared__ float wm[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) wm[w] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    float r = INFINITY;
    for (int k = 0; k < nw; k++) r = fminf(r, wm[k]);
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------
// Pooled kernels: many independent solves stepped by one persistent grid.
// Each tile is a contiguous element (or node) range of one solve; CTAs stride
// over the tile list, so the grid size is fixed (a multiple of the SM count)
// and the same graph serves any admitted set.  Per-solve control, CFL slot
// and NaN flag are those of the solve's Problem.
// ---------------------------------------------------------------------------
// Dynamic tile assignment.  sched = {tile count, claim counter, blocks done}.
// Thread 0 claims the block's next tile while the block works on the current
// one; every block makes exactly one claim past the end, and the last block to
// run out puts both counters back to zero for the next launch.  Which block
// runs a tile changes no result.
struct TileQueue {
    int *sched;
    int n;
    __device__ __forceinline__ int claim() { return atomicAdd(sched + 1, 1); }
    __device__ __forceinline__ void finish()
    {
        if (threadIdx.x == 0 && atomicAdd(sched + 2, 1) == (int)gridDim.x - 1) {
            atomicExch(sched + 1, 0);
            atomicExch(sched + 2, 0);
        }
    }
};

// Node kernel over tiles (node ranges of one solve), four lanes per node.
template <int MODE>
__global__ void __launch_bounds__(kStepThreads) pool_node_kernel(const Problem *__restrict__ descs, const Tile *__restrict__ tiles,
                                 int *__restrict__ sched, int parity)
{
    __shared__ int s_tile;
    TileQueue q{sched, sched[0]};
    if (threadIdx.x == 0) s_tile = q.claim();
    __syncthreads();
    int t = s_tile, cur = -1;
    NodeStep ns;
    while (t < q.n) {
        int next = 0;
        if (threadIdx.x == 0) next = q.claim();
        const Tile tl = tiles[t];
        const Problem &p = descs[tl.solve];
        if (tl.solve != cur) {
            node_step<MODE>(p, parity, ns);
            cur = tl.solve;
        }
        if (tl.begin == 0 && threadIdx.x == 0) publish_step(p, decide_step(p, p.ctrl[parity ^ 1], parity), parity);
        if (ns.ran || ns.run) {
            const int per = blockDim.x >> 2;   // every lane runs the same number of passes
            for (long long b = tl.begin; b < tl.end; b += per) {
                long long i = b + (threadIdx.x >> 2);
                if (MODE == MODE_MIXED) node_quad_mixed(p, i, i < tl.end, ns);
                else if (MODE == MODE_DW) node_quad_dw(p, i, i < tl.end, ns);
                else node_quad_fp64(p, i, i < tl.end, ns);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_tile = next;
        __syncthreads();
        t = s_tile;
    }
    q.finish();
}

// The elements of one tile for the tiled element kernel: each thread's
// elements in turn; returns the thread's FP32 minimum of the CFL screen.  The
// FP64 and double-word kernels keep every screen value in sdt; the mixed one
// keeps none and returns -1 once one of its elements was a sliver (a negative
// screen value), so no other register stays live.  The mixed and double-word bodies take the element's
// connectivity loaded one element ahead, so their node gathers wait for one
// memory latency instead of two (connectivity, then the nodes).  ACT: element
// birth is on, and the step's time decides which elements are dead.
template <int MODE, bool ACT, bool VISC>
__device__ __forceinline__ float tile_elements(const Problem &p, const Tile &tl, int parity, float *sdt)
{
    float v32 = INFINITY;
    const double t = ACT ? p.ctrl[parity].t : 0.0;
    const double idt = VISC ? 1.0 / p.ctrl[parity].dt : 0.0;   // the step's dt (bulk viscosity)
    const float idtf = (float)idt;
    long long e = tl.begin + threadIdx.x;
    int4 cn_next = make_int4(0, 0, 0, 0);
    if (MODE == MODE_MIXED || MODE == MODE_DW) {
        if (e < tl.end) cn_next = p.conn[e];
    }
    for (; e < tl.end; e += blockDim.x) {
        const int4 cn = cn_next;
        if ((MODE == MODE_MIXED || MODE == MODE_DW) && e + blockDim.x < tl.end) cn_next = p.conn[e + blockDim.x];
        float d = MODE == MODE_MIXED ? elem_body_mixed<false, ACT, VISC>(p, e, parity, cn, t, idtf)
                                     : (MODE == MODE_DW ? elem_body_dw<false, ACT, VISC>(p, e, parity, cn, t, idt)
                                                        : elem_body_fp64<false, ACT, VISC>(p, e, parity, t, idt));
        if (MODE == MODE_MIXED) {
            v32 = d < 0.0f ? -1.0f : fminf(v32, d);   // -1 sticks: fminf(-1, d) = -1 for d >= 0
        } else {
            sdt[e - tl.begin] = d;
            if (d >= 0.0f) v32 = fminf(v32, d);
        }
    }
    return v32;
}

constexpr int kMixedPending = 2 * kStepThreads;  // deferred FP64 rechecks a mixed CTA can hold

// The pending entries of a mixed CTA (all posted before the caller's last
// barrier): one warp per entry, its lanes over the posting thread's elements
// of that tile (one each when the tile has at most 32 per thread), skipping
// entries above 2^-8 of the solve's running screen minimum.
static __device__ __noinline__ void mixed_flush(const Problem *__restrict__ descs, const Tile *__restrict__ tiles,
                                          const int2 *pend, const float *pendv, int np, int parity)
{
    const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int j = threadIdx.x >> 5; j < np; j += nwarp) {
        const int2 pe = pend[j];
        const Tile tl = tiles[pe.x];
        const Problem &p = descs[tl.solve];
        const float mine = pendv[j];
        if (!(mine < 0.0f)) {
            const unsigned long long g = __ldcg(p.dtmin + 2 + (parity ^ 1));
            if (g < kScreenInfBits && mine > __uint_as_float((unsigned)g) * (1.0f + 1.0f / 256.0f)) continue;
        }
        double v = INFINITY;
        for (long long e = tl.begin + pe.y + (long long)lane * blockDim.x; e < tl.end; e += 32LL * blockDim.x)
            v = fmin(v, cfl_dw(p, e));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v >= 0.0 && v < INFINITY)
            atomicMin(p.dtmin + (parity ^ 1), (unsigned long long)__double_as_longlong(v));
    }
}

// The mixed kernel's tile loop.  Each tile's FP32 screen minimum (over the
// threads that met no sliver) goes to the solve's running minimum (an integer
// atomicMin on its bit pattern, nothing waited for); a thread whose own
// minimum lies within 2^-8 of the tile's, or that met a sliver, posts (tile,
// thread, own minimum) to a per-CTA list.  Once
// the CTA has run out of tiles, every entry whose minimum is still within
// 2^-8 of the solve's running minimum -- by then nearly the step's FP32
// minimum m -- has that thread's elements of that tile recomputed in FP64 by
// one warp of the CTA.  An element x near the exact minimum has
// d(x) <= m (1 + 2^-8) <= (tile minimum) (1 + 2^-8) (the tile minimum, taken
// over part of the elements, is >= m), so its thread posted unless it met a
// sliver, and then it posted anyway; the entry's minimum is <= d(x) <=
// (running minimum) (1 + 2^-8), so it is rechecked.  A tile adds at most one
// entry per thread, so the list is flushed at a tile boundary once it holds
// more than kMixedPending - blockDim entries, and never overflows; the element
// loop itself calls no FP64 code.
template <bool ACT, bool VISC>
__device__ __forceinline__ void mixed_tile_loop(const Problem *__restrict__ descs, const Tile *__restrict__ tiles,
                                                TileQueue &q, int parity)
{
    __shared__ int s_tile, s_npend;
    __shared__ int2 s_pend[kMixedPending];      // (tile, thread)
    __shared__ float s_pendv[kMixedPending];    // the thread's minimum, -1 for a sliver
    if (threadIdx.x == 0) {
        s_tile = q.claim();
        s_npend = 0;
    }
    __syncthreads();
    int t = s_tile;
    while (t < q.n) {
        int next = 0;
        if (threadIdx.x == 0) next = q.claim();
        const Tile tl = tiles[t];
        const Problem &p = descs[tl.solve];
        if (p.ctrl[parity].ran) {
            const float mine = tile_elements<MODE_MIXED, ACT, VISC>(p, tl, parity, nullptr);
            const bool neg = mine < 0.0f;
            const float bmin = block_min_bcast(neg ? INFINITY : mine);
            if (threadIdx.x == 0 && bmin < INFINITY)
                atomicMin(p.dtmin + 2 + (parity ^ 1), (unsigned long long)__float_as_uint(bmin));
            if (neg || (mine < INFINITY && mine <= bmin * (1.0f + 1.0f / 256.0f))) {
                const int k = atomicAdd(&s_npend, 1);   // < kMixedPending: flushed below in time
                s_pend[k] = make_int2(t, (int)threadIdx.x);
                s_pendv[k] = neg ? -1.0f : mine;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_tile = next;
        __syncthreads();
        if (s_npend > kMixedPending - (int)blockDim.x) {   // the same value in every thread
            mixed_flush(descs, tiles, s_pend, s_pendv, s_npend, parity);
            __syncthreads();
            if (threadIdx.x == 0) s_npend = 0;
            __syncthreads();
        }
        t = s_tile;
    }
    mixed_flush(descs, tiles, s_pend, s_pendv, s_npend, parity);   // posted before the loop's last barrier
}

// Element kernel over tiles.  Each element's FP32 CFL screen value is
// compared with the solve's running FP32 minimum of the screen (a per-step
// slot that every tile lowers by an integer atomicMin on its bit pattern):
// elements within 2^-8 of it, and slivers, recompute the exact FP64 value,
// whose minimum goes to the solve's CFL slot.  The screen's error stays far
// below 2^-9 outside slivers, so that set always holds the step's exact
// minimum.  FP64 and double-word keep the tile's screen values in shared
// memory, list the candidates and recompute them by consecutive threads; the
// mixed kernel defers its few rechecks to the end of the CTA's tiles
// (mixed_tile_loop).  ACT: the instantiation with element birth (single
// solves whose block has it on), VISC the one with artificial bulk viscosity;
// the plain one carries no trace of either.
template <int MODE, bool ACT = false, bool VISC = false>
__global__ void __launch_bounds__(kStepThreads, MODE == MODE_MIXED ? 4 : (MODE == MODE_DW ? 3 : 2)) pool_elem_kernel(const Problem *__restrict__ descs,
                                                                 const Tile *__restrict__ tiles,
                                                                 int *__restrict__ sched, int parity)
{
    __shared__ float sdt[MODE == MODE_MIXED ? 1 : kMaxTileElems];
    __shared__ unsigned short scand[MODE == MODE_MIXED ? 1 : kMaxTileElems];
    __shared__ int s_tile, s_ncand;
    __shared__ float s_thr;
    TileQueue q{sched, sched[0]};
    if constexpr (MODE == MODE_MIXED) {
        mixed_tile_loop<ACT, VISC>(descs, tiles, q, parity);
        q.finish();
        return;
    }
    if (threadIdx.x == 0) s_tile = q.claim();
    __syncthreads();
    int t = s_tile;
    while (t < q.n) {
        int next = 0;
        if (threadIdx.x == 0) next = q.claim();
        const Tile tl = tiles[t];
        const Problem &p = descs[tl.solve];
        if (p.ctrl[parity].ran) {
            if (MODE != MODE_MIXED && threadIdx.x == 0) s_ncand = 0;
            const float v32 = tile_elements<MODE, ACT, VISC>(p, tl, parity, sdt);
            const float bmin = block_min_bcast(v32);   // also orders the sdt writes before the reads below
            if (threadIdx.x == 0) {
                // g: the solve's smallest FP32 screen value over the tiles closed
                // so far in this step, this one included.  g >= the step's FP32
                // minimum m, and the exact minimum's screen value is <= m (1 + 2^-8)
                // (screen error below 2^-9 outside slivers), so elements above
                // g (1 + 2^-8) are never the exact minimum: most tiles skip the
                // FP64 recheck, whichever order they close in.
                float g = bmin;
                if (bmin < INFINITY) {
                    const unsigned long long old =
                        atomicMin(p.dtmin + 2 + (parity ^ 1), (unsigned long long)__float_as_uint(bmin));
                    g = old >= kScreenInfBits ? bmin : fminf(__uint_as_float((unsigned)old), bmin);
                }
                s_thr = g * (1.0f + 1.0f / 256.0f);
            }
            __syncthreads();
            const float thr = s_thr;
            if (MODE == MODE_MIXED) {
                // a thread reads back only the entries it wrote itself
                double v = INFINITY;
                for (long long e = tl.begin + threadIdx.x; e < tl.end; e += blockDim.x) {
                    const float d = sdt[e - tl.begin];
                    if (d < 0.0f || d <= thr) v = fmin(v, cfl_dw(p, e));
                }
                if (v >= 0.0 && v < INFINITY)
                    atomicMin(p.dtmin + (parity ^ 1), (unsigned long long)__double_as_longlong(v));
            } else {
                // the tile's candidates are listed first and then recomputed by
                // consecutive threads, so a few candidates take one warp, not several
                for (long long e = tl.begin + threadIdx.x; e < tl.end; e += blockDim.x) {
                    float d = sdt[e - tl.begin];
                    if (d < 0.0f || d <= thr) scand[atomicAdd(&s_ncand, 1)] = (unsigned short)(e - tl.begin);
                }
                __syncthreads();
                const int nc = s_ncand;
                if (nc > 0) {   // uniform across the block
                    double v = INFINITY;
                    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
                        const long long e = tl.begin + scand[c];
                        v = fmin(v, MODE == MODE_DW ? cfl_dw(p, e) : cfl_fp64(p, e));
                    }
                    block_min_to(v, p.dtmin + (parity ^ 1));
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_tile = next;
        __syncthreads();
        t = s_tile;
    }
    q.finish();
}

// ---------------------------------------------------------------------------
// Set-up kernels (reference operation order), built in the exact unit only
// ---------------------------------------------------------------------------
#ifdef MSX_SETUP_KERNELS
// Reference Jacobian of a tet from xyz[i*4 + k] (coordinate i of corner k):
// Jac_ij = 0 + sum_k x_ik natDev_kj in corner order, natDev's entries -1, 0
// and 1 (classLinearTetrahedra.cpp:171-268).  For finite coordinates that sum
// is (0 - x_i0) + x_i(j+1) bit for bit: 0 - x_i0 is never -0, and the products
// with 0 add signed zeros to a partial sum that is never -0, which leaves it
// unchanged.  A non-finite coordinate (x * 0 is NaN) takes the full sum.
__device__ __forceinline__ void ref_jacobian(const double *xyz, double *Jac)
{
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 12; k++) finite &= isfinite(xyz[k]);
    if (finite) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const double y0 = 0.0 - xyz[i * 4];
#pragma unroll
            for (int j = 0; j < 3; j++) Jac[i * 3 + j] = y0 + xyz[i * 4 + j + 1];
        }
    } else {
        const double natDev[12] = {-1.0, -1.0, -1.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) c += xyz[i * 4 + k] * natDev[k * 3 + j];
                Jac[i * 3 + j] = c;
            }
    }
}

// The plain FP64 mode's compressible neo-Hookean element data of element e
// (Problem::Eref, Mg, rdetE) from its corner coordinates pts[k*3 + i], the
// stored gradients g (G's nine entries) and the reference Jacobian's
// determinant.
__device__ __forceinline__ void write_cnh_arrays(const Problem &p, long long e, const double *pts, const double *g,
                                                 double Jref)
{
    const long long ne = p.ne;
    double *Er = const_cast<double *>(p.Eref), *Mw = const_cast<double *>(p.Mg);
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int i = 0; i < 3; i++) Er[(b * 3 + i) * ne + e] = pts[(b + 1) * 3 + i] - pts[i];
    int k = 0;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = a; b < 3; b++, k++)
            Mw[k * ne + e] = g[a * 3] * g[b * 3] + g[a * 3 + 1] * g[b * 3 + 1] + g[a * 3 + 2] * g[b * 3 + 2];
    const_cast<double *>(p.rdetE)[e] = 1.0 / Jref;
}

// classLinearTetrahedra.cpp:171-268 (Jacobian, inverse, dphi), classGPs.cpp:27
// (wJ = 0.166666666667 |J|), classLinearTetrahedra.cpp:129-140 (charLength).
__global__ void setup_elements_kernel(Problem p, const double *X, double *G, double *wJ, double *Lref,
                                      float *G32, float *wJ32, float *Lref32, long long e0, long long e1)
{
    const long long e = e0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;   // elements [e0, e1)
    if (e >= e1) return;
    const long long nn = p.nn, ne = p.ne;
    int4 cn = p.conn[e];
    // an out-of-range node id: the node-list build queued after this kernel
    // rejects the mesh
    if ((unsigned long long)(unsigned)cn.x >= (unsigned long long)nn || (unsigned long long)(unsigned)cn.y >= (unsigned long long)nn ||
        (unsigned long long)(unsigned)cn.z >= (unsigned long long)nn || (unsigned long long)(unsigned)cn.w >= (unsigned long long)nn)
        return;
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double xyz[12], pts[12];
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            xyz[i * 4 + k] = X[i * nn + nd[k]];
            pts[k * 3 + i] = X[i * nn + nd[k]];
        }
    double Jac[9], iJ[9];
    ref_jacobian(xyz, Jac);
    double J = det3_ref(Jac);
    inv3_ref(Jac, iJ);
    double gst[9];   // G as stored
#pragma unroll
    for (int k = 0; k < 9; k++) {
        double g = 0.0 + iJ[k];
        gst[k] = g;
        G[k * ne + e] = g;
        if (G32) G32[k * ne + e] = (float)g;
        if (p.G32lo) const_cast<float *>(p.G32lo)[k * ne + e] = (float)(g - (double)(float)g);
    }
    double w = 0.166666666667 * fabs(J);
    wJ[e] = w;
    if (wJ32) wJ32[e] = (float)w;
    if (p.wJ32lo) const_cast<float *>(p.wJ32lo)[e] = (float)(w - (double)(float)w);
    double v6;   // 6V, signed: the edge determinant of the inscribed-sphere volume
    double L = char_length_ref(pts, &v6);
    Lref[e] = L;
    if (p.Eref) write_cnh_arrays(p, e, pts, gst, J);
    // A reference sliver (6V below 0.063 |e1||e2||e3|) gets a negative FP32
    // length: the FP32 CFL screens then always recompute it in FP64 (the mixed
    // screen rebuilds the reference edges from G in FP32, which loses accuracy
    // on such a tet).  Lref itself is unchanged.
    {
        double e1[3], e2[3], e3[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            e1[i] = pts[3 + i] - pts[i];
            e2[i] = pts[6 + i] - pts[i];
            e3[i] = pts[9 + i] - pts[i];
        }
        const double l1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
        const double l2 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
        const double l3 = e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2];
        const bool sliver = !(v6 * v6 >= 4e-3 * l1 * l2 * l3);
        Lref32[e] = sliver ? -(float)L : (float)L;
    }
}

// The FP32 element arrays of a precision mode that a handle starts using after
// its set-up (a later solver block in another mode), from the FP64 set-up data
// and X: the same conversions setup_elements_kernel makes, so the same bits.
__global__ void mode_arrays_kernel(Problem p, float *G32, float *wJ32, float *G32lo, float *wJ32lo)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const long long ne = p.ne;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const double g = p.G[k * ne + e];
        if (G32) G32[k * ne + e] = (float)g;
        if (G32lo) G32lo[k * ne + e] = (float)(g - (double)(float)g);
    }
    const double w = p.wJ[e];
    if (wJ32) wJ32[e] = (float)w;
    if (wJ32lo) wJ32lo[e] = (float)(w - (double)(float)w);
}

// Problem::Eref, Mg and rdetE of a handle whose FP64 block starts after its
// set-up: the same operations as setup_elements_kernel, from X and the stored G.
__global__ void cnh_arrays_kernel(Problem p)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const long long nn = p.nn, ne = p.ne;
    const int4 cn = p.conn[e];
    const int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double xyz[12], pts[12], g[9], Jac[9];
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            xyz[i * 4 + k] = p.X[i * nn + nd[k]];
            pts[k * 3 + i] = p.X[i * nn + nd[k]];
        }
    ref_jacobian(xyz, Jac);
#pragma unroll
    for (int k = 0; k < 9; k++) g[k] = p.G[k * ne + e];
    write_cnh_arrays(p, e, pts, g, det3_ref(Jac));
}

// Previous-step F diagonal for the bulk viscosity, from displacement u, in the
// reference's order of F (constitutiveManager.cpp:151-164): what the Gauss
// points' previous state holds at the start of a block (the last step's F, or
// I from rest).
__global__ void visc_init_kernel(Problem p, const double *u)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const long long ne = p.ne, nn = p.nn;
    const int4 cn = p.conn[e];
    const int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double dphi[12];
#pragma unroll
    for (int k = 0; k < 9; k++) dphi[3 + k] = p.G[k * ne + e];
#pragma unroll
    for (int j = 0; j < 3; j++) dphi[j] = (-dphi[3 + j] - dphi[6 + j]) - dphi[9 + j];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        double F = 0.;
        F += 1.;
#pragma unroll
        for (int a = 0; a < 4; a++) F += dphi[a * 3 + i] * u[nd[a] + i * nn];
        if (p.visc_f0) p.visc_f0[i * ne + e] = F;
        if (p.visc_h0) p.visc_h0[i * ne + e] = (float)(F - 1.0);
    }
}

// constitutiveAlgorithms.cpp:191-205 (rho wJ phi_a phi_b summed over b) and
// solverExplicit.cpp:429-459 (element-order sum per node).
__global__ void setup_mass_kernel(Problem p, double *mass, double *minv)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nn) return;
    const double phi = -1.0 * 0.25 - 1.0 * 0.25 - 1.0 * 0.25 + 1.0;
    double m = 0;
    const int k1 = p.node_ptr[i + 1];
    // the incidences' loads eight at a time, then their sums in element order
    for (int k = p.node_ptr[i]; k < k1; k += 8) {
        double w[8], r[8];
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (k + j < k1) {
                const long long e = p.node_inc[k + j] >> 2;
                w[j] = p.wJ[e];
                r[j] = mat_of(p, e).rho;
            }
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (k + j < k1) {
                // me = 0 + z + z + z + z over the four corners b, z = ((wJ rho) phi) phi:
                // that sum is (3z) + z bit for bit (0 + z = z and z + z = 2z are exact,
                // 2z + z rounds 3z once); a z of -0 gives -0 instead of +0, which adds
                // to m the same way
                const double z = w[j] * r[j] * phi * phi;
                m += __dadd_rn(__dmul_rn(3.0, z), z);
            }
    }
    mass[i] = m;
    minv[i] = 1.0 / m;
}

// boundaryConditions.cpp:1146-1171 BCsGravity: -w rho |J| g phi_a on the z DOF
// of each corner (|J| as classGPs::getJ keeps it), summed per node in element order.
__global__ void setup_gravity_elem_kernel(Problem p, double g, double *grav_e)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const long long nn = p.nn;
    int4 cn = p.conn[e];
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double M[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) M[i * 3 + j] = p.X[i * nn + nd[j + 1]] - p.X[i * nn + nd[0]];
    const double w = 0.166666666667, phi = -1.0 * 0.25 - 1.0 * 0.25 - 1.0 * 0.25 + 1.0;
    grav_e[e] = -w * mat_of(p, e).rho * fabs(det3_ref(M)) * g * phi;
}

__global__ void setup_gravity_node_kernel(Problem p, const double *grav_e, double *grav_n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nn) return;
    double s = 0;
    for (int k = p.node_ptr[i]; k < p.node_ptr[i + 1]; k++) s += grav_e[p.node_inc[k] >> 2];
    grav_n[i] = s;
}

// Contributions of the traction and pressure faces for the step whose control
// slot `parity` the node kernel just wrote, at that step's time and
// displacement, in the reference's operation order (boundaryConditions.cpp:
// 218-275 BCsTractionInst/Ramp, :370-505 BCsPressureRamp/Inst; amounts from
// classNeumannBCs.h:57-181).  Pressure follows the face: n = F^-T n0 with F of
// the bulk tet by classSpatialPoint::getF (classSpatialPoint.cpp:41-66):
// F_ij = 0 + sum_a dphi_aj u_ai (corner order) + delta_ij.
__global__ void face_load_kernel(Problem p, int parity, bool mixed)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= p.nfaces) return;
    const Ctrl c = p.ctrl[parity];
    if (!c.ran) return;
    const double t = c.t;
    const FaceLoad L = p.faces[f];
    const bool ramp = L.kind == MSX_LOAD_TRACTION_RAMP || L.kind == MSX_LOAD_PRESSURE_RAMP;
    const bool pressure = L.kind == MSX_LOAD_PRESSURE_INST || L.kind == MSX_LOAD_PRESSURE_RAMP;
    double amount[3] = {0.0, 0.0, 0.0};
    if (t >= L.t0 && t <= L.tf)
        for (int i = 0; i < (pressure ? 1 : 3); i++) amount[i] = ramp ? L.value[i] / (L.tf - L.t0) * (t - L.t0) : L.value[i];
    double *out = p.fcon + (long long)L.con * 3;
    if (!pressure) {
        for (int a = 0; a < 3; a++)
            for (int i = 0; i < 3; i++) out[a * 3 + i] = L.wabsJ * L.phi[a] * amount[i];
        return;
    }
    const long long nn = p.nn, ne = p.ne, e = L.tet;
    const int4 cn = p.conn[e];
    const int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double dphi[12];
    for (int a = 1; a < 4; a++)
        for (int j = 0; j < 3; j++) dphi[a * 3 + j] = p.G[((a - 1) * 3 + j) * ne + e];
    for (int j = 0; j < 3; j++) dphi[j] = ((-dphi[3 + j]) - dphi[6 + j]) - dphi[9 + j];
    double F[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < 4; a++) {
        double disp[3];
        for (int i = 0; i < 3; i++) {
            const long long dof = nd[a] + i * nn;
            disp[i] = mixed ? (double)p.uhl[dof].x + (double)p.uhl[dof].y : p.u[dof];
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) F[i * 3 + j] += dphi[a * 3 + j] * disp[i];
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) F[i * 3 + j] += (i == j ? 1.0 : 0.0);
    double Fi[9], n[3];
    const double Jac = det3_ref(F);
    inv3_ref(F, Fi);
    for (int i = 0; i < 3; i++) {
        n[i] = 0;
        for (int j = 0; j < 3; j++) n[i] += Fi[j * 3 + i] * L.n0[j];
    }
    if (L.kind == MSX_LOAD_PRESSURE_RAMP) {
        // the bulk tet's shape function of its first node at natural coordinates 0 is 1
        for (int i = 0; i < 3; i++) out[i] = L.wabsJ * 1.0 * Jac * amount[0] * n[i];
    } else {
        for (int a = 0; a < 3; a++)
            for (int i = 0; i < 3; i++) out[a * 3 + i] = L.wabsJ * L.phi[a] * Jac * amount[0] * n[i];
    }
}

// Node data extraction (dataExtraction.cpp:778-840): the displacement, the
// external force of the last step at its time t, or the internal force summed
// from zero in element order (computeInternalForce, solverExplicit.cpp:363-379)
// from the corner forces the last element kernel left: element order in the
// reference-order mode, the node's CSR slots (also element order) otherwise.
__global__ void node_values_kernel(Problem p, int mode, int field, int comp, const int *nodes, long long n, double t,
                                   double *out)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const long long i = nodes[j], dof = i + comp * p.nn;
    double v = 0.0;
    if (field == MSX_FIELD_DISPLACEMENT) {
        v = p.u[dof];
    } else if (field == MSX_FIELD_EXTERNAL_FORCE) {
        if (p.ext_ptr) v = ext_force_dof(p, dof, t);
    } else {
        for (int k = p.node_ptr[i]; k < p.node_ptr[i + 1]; k++) {
            if (mode == MODE_EXACT) v += p.fe[(long long)p.node_inc[k] * 3 + comp];
            else if (mode == MODE_MIXED) v += (double)p.fe32[(long long)k * 4 + comp];
            else if (mode == MODE_DW) {
                const float2 w = reinterpret_cast<const float2 *>(p.fe)[(long long)k * 3 + comp];
                v += (double)w.x + (double)w.y;
            } else v += p.fe[(long long)k * 3 + comp];
        }
    }
    out[j] = v;
}

// solvers.cpp:276-287 (uK == nullptr) and :296-320: element min into dtmin[slot]
__global__ void __launch_bounds__(kElemBlock) initial_cfl_kernel(Problem p, const double *uK, int slot)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = INFINITY;
    if (e < p.ne) {
        const MatParams &m = mat_of(p, e);
        if (!uK) {
            v = p.Lref[e] / m.c;
        } else {
            int4 cn = p.conn[e];
            int nd[4] = {cn.x, cn.y, cn.z, cn.w};
            double x[12];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    x[a * 3 + k] = p.X[k * p.nn + nd[a]];
                    x[a * 3 + k] += uK[p.nn * k + nd[a]];
                }
            double dist = char_length_ref(x);
            double Lr = p.Lref[e];
            v = ((dist < Lr) ? dist : Lr) / m.c;
        }
    }
    block_min_to(v, p.dtmin + slot);
}

// Output fields of one element from the current u, in the reference's order:
// Cauchy (NH: the law's sigma, hyperElasticNeoHookean.cpp:113-124; other laws
// P F^T / J, maths.cpp:1250-1254), Green-Lagrange E (maths.cpp:1227-1243) and
// von Mises (maths.cpp:1261-1271).
__global__ void element_fields_kernel(Problem p, double t, double *cauchy, double *gl, double *vms)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    if (elem_dead(p, e, t)) {   // never updated: the Gauss point's initial, zero state
#pragma unroll
        for (int k = 0; k < 9; k++) {
            if (cauchy) cauchy[e * 9 + k] = 0.0;
            if (gl) gl[e * 9 + k] = 0.0;
        }
        if (vms) vms[e] = 0.0;
        return;
    }
    const long long ne = p.ne, nn = p.nn;
    int4 cn = p.conn[e];
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double dphi[12];
#pragma unroll
    for (int k = 0; k < 9; k++) dphi[3 + k] = p.G[k * ne + e];
#pragma unroll
    for (int j = 0; j < 3; j++) dphi[j] = (-dphi[3 + j] - dphi[6 + j]) - dphi[9 + j];
    double F[9], P[9], S[9], E[9];
#pragma unroll
    for (int i = 0; i < 9; i++) F[i] = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        F[i * 3 + i] += 1.;
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int j = 0; j < 3; j++) F[i * 3 + j] += dphi[a * 3 + j] * p.u[nd[a] + i * nn];
    }
    const MatParams &m = mat_of(p, e);
    if (m.law == 0) {
        double B[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += F[i * 3 + k] * F[j * 3 + k];
                B[i * 3 + j] = c;
            }
        double J = det3_ref(F);
        double trB = 0;
#pragma unroll
        for (int i = 0; i < 3; i++) trB += B[i * 3 + i];
        double fact1 = pow(J, 5.0 / 3.0);
        double fact2 = m.mu / fact1;
#pragma unroll
        for (int i = 0; i < 9; i++) S[i] = 0 + fact2 * B[i];
        double fact3 = -(m.mu / 3.0) * trB / fact1 + m.K1 * (J - 1.0);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) S[i * 3 + j] += fact3 * (i == j ? 1.0 : 0.0);
    } else {
        stress_ref(m, F, P);
        double detJinv = 1. / det3_ref(F);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double c = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) c += P[i * 3 + k] * F[j * 3 + k];
                S[i * 3 + j] = c;
            }
#pragma unroll
        for (int i = 0; i < 9; i++) S[i] = S[i] * detJinv;
    }
    // the compressible neo-Hookean law never updates its Green-Lagrange strain
    // (hyperElasticNeoHookean.cpp:221-289), so the reference reports zero; the
    // linear-elastic law stores its small strain there (linearElastic.cpp:71-76)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            double c = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) c += F[k * 3 + i] * F[k * 3 + j];
            E[i * 3 + j] = m.law == 1 ? 0.0
                         : m.law == 3 ? 0.5 * (F[i * 3 + j] + F[j * 3 + i] - 2. * (i == j ? 1. : 0.))
                                      : 0.5 * (c - (i == j ? 1.0 : 0.0));
        }
    if (cauchy)
#pragma unroll
        for (int k = 0; k < 9; k++) cauchy[e * 9 + k] = S[k];
    if (gl)
#pragma unroll
        for (int k = 0; k < 9; k++) gl[e * 9 + k] = E[k];
    if (vms)
        vms[e] = sqrt(0.5 * ((S[0] - S[4]) * (S[0] - S[4]) + (S[4] - S[8]) * (S[4] - S[8]) +
                             (S[8] - S[0]) * (S[8] - S[0]) + 6 * (S[1] * S[1] + S[2] * S[2] + S[5] * S[5])));
}

// One Gauss point's element-extraction value (msx_element_quantity) at the
// current u, v, in the reference's operation order: getValueAtGP
// (dataExtraction.cpp:508-563; Cauchy = P F^T / det F, classStates.cpp:309-316),
// the laws' defoEnergy (hyperElasticNeoHookean.cpp:291-304,
// hyperElasticStVenantKirchhoff.cpp:251-274; the Neo-Hookean law keeps the
// zero default, constitutiveModels.h:91-94), kineticEnergy's density at the
// centroid, where every shape function is 0.25 (dataExtraction.cpp:626-688),
// and volume's wJ det F (:690-748).  The internal variables read zero: no law
// here has more than one (getValueAtGP wants more than k for INVAR k).
__device__ double element_quantity_ref(const Problem &p, int q, long long e, double t)
{
    if (elem_dead(p, e, t)) return 0.0;   // dataExtraction.cpp:510
    if (q >= MSX_ELEM_INVAR1 && q <= MSX_ELEM_INVAR6) return 0.0;
    const long long ne = p.ne, nn = p.nn;
    const int4 cn = p.conn[e];
    const int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    const MatParams &m = mat_of(p, e);
    if (q == MSX_ELEM_KIN_ENERGY) {
        double vel[3] = {0., 0., 0.}, val = 0;
        for (int a = 0; a < 4; a++)
            for (int j = 0; j < 3; j++) vel[j] += 0.25 * p.v[nd[a] + j * nn];
        for (int j = 0; j < 3; j++) val += 0.5 * m.rho * vel[j] * vel[j];
        return val;
    }
    if (q == MSX_ELEM_DEFO_ENERGY && m.law == 0) return 0.0;
    double dphi[12];
    for (int k = 0; k < 9; k++) dphi[3 + k] = p.G[k * ne + e];
    for (int j = 0; j < 3; j++) dphi[j] = (-dphi[3 + j] - dphi[6 + j]) - dphi[9 + j];
    double F[9];
    for (int i = 0; i < 9; i++) F[i] = 0.;
    for (int i = 0; i < 3; i++) {
        F[i * 3 + i] += 1.;
        for (int a = 0; a < 4; a++)
            for (int j = 0; j < 3; j++) F[i * 3 + j] += dphi[a * 3 + j] * p.u[nd[a] + i * nn];
    }
    if (q >= MSX_ELEM_FXX && q <= MSX_ELEM_FZZ) return F[q - MSX_ELEM_FXX];
    if (q == MSX_ELEM_VOLUME) return p.wJ[e] * det3_ref(F);
    if (q == MSX_ELEM_DEFO_ENERGY && m.law == 3) {
        // linearElastic.cpp:88-101: 0.5 (P:F - P:I), contractions summed from 0
        double P[9], a = 0, b = 0;
        stress_ref(m, F, P);
        for (int i = 0; i < 9; i++) a += P[i] * F[i];
        for (int i = 0; i < 9; i++) b += P[i] * ((i % 4) == 0 ? 1. : 0.);
        return 0.5 * (a - b);
    }
    if (q == MSX_ELEM_DEFO_ENERGY) {
        double C[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += F[k * 3 + i] * F[k * 3 + j];
                C[i * 3 + j] = c;
            }
        if (m.law == 1) {
            const double J = det3_ref(F);
            double tr = 0;
            for (int i = 0; i < 3; i++) tr += C[i * 3 + i];
            return 0.5 * m.lambda * log(J) * log(J) - m.mu * log(J) + 0.5 * m.mu * tr;
        }
        double E[9], S[9], trE = 0, w = 0;
        for (int i = 0; i < 9; i++) E[i] = 0.5 * (C[i] - ((i % 4) == 0 ? 1.0 : 0.0));
        for (int i = 0; i < 3; i++) trE += E[i * 3 + i];
        for (int i = 0; i < 9; i++) S[i] = E[i] * m.mu2;
        for (int i = 0; i < 3; i++) S[i * 3 + i] += m.lam_stvk * trE;
        for (int i = 0; i < 9; i++) w += S[i] * E[i];
        return 0.5 * w;
    }
    double P[9];
    stress_ref(m, F, P);
    if (q >= MSX_ELEM_PXX && q <= MSX_ELEM_PZZ) return P[q - MSX_ELEM_PXX];
    // SVM, KVM
    const double detF = det3_ref(F), detJinv = 1. / detF;
    double S[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double c = 0;
            for (int k = 0; k < 3; k++) c += P[i * 3 + k] * F[j * 3 + k];
            S[i * 3 + j] = c;
        }
    for (int i = 0; i < 9; i++) S[i] = S[i] * detJinv;
    const double svm = sqrt(0.5 * ((S[0] - S[4]) * (S[0] - S[4]) + (S[4] - S[8]) * (S[4] - S[8]) +
                                   (S[8] - S[0]) * (S[8] - S[0]) + 6 * (S[1] * S[1] + S[2] * S[2] + S[5] * S[5])));
    return q == MSX_ELEM_KVM ? svm * detF : svm;
}

__global__ void element_values_kernel(Problem p, int q, const int *elems, long long n, double t, double *out)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] = element_quantity_ref(p, q, elems ? elems[j] : j, t);
}

// The element-extraction reduction in two fixed-shape passes, so the result
// does not depend on the GPU or the run: kReduceBlocks blocks each take a
// grid-stride share in index order and fold it in a shared-memory tree into
// part[2b] (the weighted sum, or the extreme) and part[2b+1] (the sum of dV);
// one block then folds the partials the same way.
constexpr int kReduceBlocks = 512, kReduceThreads = 256;

__device__ __forceinline__ void fold_pair(int op, double &s, double &w, double s2, double w2)
{
    if (op == MSX_OP_MAX) s = s2 > s ? s2 : s;
    else if (op == MSX_OP_MIN) s = s2 < s ? s2 : s;
    else s += s2;
    w += w2;
}

__device__ __forceinline__ void block_fold(int op, double &s, double &w)
{
    __shared__ double ss[kReduceThreads], ws[kReduceThreads];
    ss[threadIdx.x] = s;
    ws[threadIdx.x] = w;
    __syncthreads();
    for (int h = kReduceThreads / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            double a = ss[threadIdx.x], b = ws[threadIdx.x];
            fold_pair(op, a, b, ss[threadIdx.x + h], ws[threadIdx.x + h]);
            ss[threadIdx.x] = a;
            ws[threadIdx.x] = b;
        }
        __syncthreads();
    }
    s = ss[0];
    w = ws[0];
}

__device__ __forceinline__ double reduce_identity(int op)
{
    return op == MSX_OP_MAX ? -INFINITY : (op == MSX_OP_MIN ? INFINITY : 0.0);
}

__global__ void __launch_bounds__(kReduceThreads) element_reduce_kernel(Problem p, int q, int op, const int *elems,
                                                                        long long n, double t, double *part)
{
    double s = reduce_identity(op), w = 0.0;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        if (q == MSX_ELEM_EXTERNAL_ENERGY) {
            s += p.u[j] * (p.ext_ptr ? ext_force_dof(p, j, t) : 0.0);
            continue;
        }
        const long long e = elems ? elems[j] : j;
        // the energies and the volume skip dead Gauss points altogether (:577-578, 644-645, 706-707)
        if ((q == MSX_ELEM_DEFO_ENERGY || q == MSX_ELEM_KIN_ENERGY || q == MSX_ELEM_VOLUME) && elem_dead(p, e, t))
            continue;
        const double v = element_quantity_ref(p, q, e, t), dV = p.wJ[e];
        fold_pair(op, s, w, q == MSX_ELEM_VOLUME || op == MSX_OP_MAX || op == MSX_OP_MIN ? v : v * dV, dV);
    }
    block_fold(op, s, w);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s;
        part[2 * blockIdx.x + 1] = w;
    }
}

__global__ void __launch_bounds__(kReduceThreads) element_reduce_finish_kernel(int q, int op, const double *part,
                                                                               double *out)
{
    double s = reduce_identity(op), w = 0.0;
    for (int b = threadIdx.x; b < kReduceBlocks; b += blockDim.x) fold_pair(op, s, w, part[2 * b], part[2 * b + 1]);
    block_fold(op, s, w);
    if (threadIdx.x == 0) *out = op == MSX_OP_MEAN ? s / w : s;
}

#endif  // MSX_SETUP_KERNELS

// f_int gather for the test hook: fint[node + c*nn] in element order
template <int MODE>
__global__ void gather_kernel(Problem p, double *fint)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nn) return;
    double s[3] = {0, 0, 0};
    for (int k = p.node_ptr[i]; k < p.node_ptr[i + 1]; k++) {
        // reference-order corner forces are in element order, the others in CSR slots
        long long inc = MODE == MODE_EXACT ? p.node_inc[k] : k;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (MODE == MODE_MIXED) {
                s[c] += (double)p.fe32[inc * 4 + c];
            } else if (MODE == MODE_DW) {
                const float2 w = reinterpret_cast<const float2 *>(p.fe)[inc * 3 + c];
                s[c] += (double)w.x + (double)w.y;
            } else {
                s[c] += p.fe[inc * 3 + c];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) fint[i + c * p.nn] = s[c];
}

inline unsigned grid_for(long long n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace msx
