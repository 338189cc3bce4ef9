// msx_internal.h -- device-side data layout shared by the kernels and the
// host runtime of the explicit C3D4 step.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/msx.h"

namespace msx {

constexpr int kMaxMats = 16;
constexpr int kElemBlock = 256;   // element-kernel CTA (one element per thread)
constexpr int kNodeBlock = 256;   // node-kernel CTA (one node per thread)

enum Mode { MODE_FP64 = 0, MODE_EXACT = 1, MODE_MIXED = 2, MODE_DW = 3 };

// Material constants, derived on the host the way the reference's law
// constructors do (hyperElasticNeoHookean.cpp:23-33,203-215,
// hyperElasticStVenantKirchhoff.cpp:23-31,64-70).
struct MatParams {
    int law;
    double young, nu, rho;
    double lambda, mu, K1;        // NH / compressible NH
    double mu2, lam_stvk;         // StVK: E/(1+nu), E nu/((1+nu)(1-2nu))
    double c;                     // sound speed used by the CFL
    float lambda_f, mu_f, K1_f, mu2_f, lam_stvk_f, inv_c_f, rho_f;
    float2 lambda_w, mu_w, K1_w, mu2_w, lam_stvk_w, mu3_w;   // double-word copies (mu3 = mu/3)
};

// One Dirichlet entry; `val` is what classDirichlet stores
// (classNodes.cpp:58-74): U/(tf-t0) for RAMP, U for INST, Vmax for VEL_RAMP.
struct BCEntry {
    int mode;
    int ramp_steps;
    double val;
};

// One nodal-force DOF of *BOUNDARY, TYPE=FORCE: f(t) = m t for t0 <= t <= tf
// (classNeumann::getTracAmount, classNodes.h:101-109), m = value / (tf - t0).
struct ForceEntry {
    double m, t0, tf;
};

// One face of a traction or pressure block (boundaryConditions.cpp:218-505):
// face S of bulk tet `tet`, its one-point rule (w |J|, phi) and unit normal n0
// from the reference geometry, and the block's amount.  Its contributions
// fcon[(con + a)*3 + i] go to node[a]: the three face nodes, or for a ramped
// pressure only the tet's first node (phi = 1, the reference's evaluation of
// the bulk shape functions at natural coordinates 0).
struct FaceLoad {
    int kind;                 // MSX_LOAD_TRACTION_INST .. MSX_LOAD_PRESSURE_RAMP
    int tet;
    int node[3];
    int con;
    double wabsJ, phi[3], n0[3];
    double t0, tf, value[3];
};

// Terms of the external-force lists: kind in the top 4 bits, index below.
enum : unsigned { EXT_FORCE = 0u, EXT_GRAV_ELEM = 1u, EXT_GRAV_NODE = 2u, EXT_FACE = 3u };
constexpr unsigned kExtIndexBits = 28;

// Step control, double-buffered by step parity.  The node kernel of step n
// reads slot (n-1)&1 and writes slot n&1; every thread derives the same
// values, so no thread waits for another.
struct Ctrl {
    double t;            // time after the last time advance
    double dt;           // dt of the last executed step (dt_init before any)
    long long step;      // steps executed in this solver block
    long long limit;     // stop once step reaches this count
    int ran;             // 1: the last node kernel started a step (its post is pending)
    int stop;            // 1: block finished (tf reached, limit hit or error)
    int status;          // msx_status
    int pad;
    unsigned long long pending;  // CFL min for the next step, saved when a block stops
};

struct Problem {
    long long nn, ne;
    // elements (SoA)
    const int4 *conn;
    const double *G;          // 9*ne: G[k*ne + e] = invJ[k/3][k%3] = dphi of node k/3+1
    const double *wJ;
    const double *Lref;
    const float *G32, *wJ32, *Lref32;       // FP32 copies (mixed mode)
    const float *G32lo, *wJ32lo;  // low words: G32 + G32lo and wJ32 + wJ32lo as double-words (double-word mode)
    const unsigned char *mat; // per-element material id, or nullptr
    const double *act_t;      // per-element activation time under *ACTIVATION, or nullptr
    int nmat;
    MatParams mats[kMaxMats];
    // nodes (SoA, dof = node + c*nn)
    const double *X;
    double *u, *v, *a;
    // plain FP64 mode: a node-major copy of u, one 32-byte record per node
    // (x, y, z, zero pad), kept by the node kernel beside u; the element
    // kernel gathers a node with two loads of one sector instead of three
    // 8-byte loads from three rows.  Null in the other modes.
    double *u4;
    // plain FP64 mode, compressible neo-Hookean elements: the reference edges
    // X_b - X_0 (9*ne: Eref[(3(b-1) + i)*ne + e], b = 1..3), the metric
    // M_ab = g_a . g_b of the shape-function gradients g_1..g_3 (6*ne, in the
    // order 11 12 13 22 23 33) and 1/det of the reference Jacobian (ne).  The
    // element kernel then takes F g_a = sum_b M_ab e_b and cof(F) g_a from the
    // cross products of the deformed edges e_b, without forming F.  Null in the
    // other modes and in pooled solves.
    const double *Eref, *Mg, *rdetE;
    const double *mass;       // lumped mass per node
    const double *minv;       // 1/mass per node
    // mixed mode: u, v, a as FP32 (hi, lo) pairs (value hi + lo) while a block
    // runs; u, v, a above hold the state between calls (state_merge)
    float2 *uhl, *vhl, *ahl;  // 3*nn each (the mixed mode keeps a as one FP32 per DOF: mixed_a32)
    const float2 *minv2;      // 1/mass as an (hi, lo) pair
    // corner forces.  Reference-order mode: fe[(e*4 + a)*3 + i] (element
    // order).  FP64 and mixed modes: in the node's CSR slot k = slot[e].a,
    // fe[k*3 + i] and fe32[k*4 + i] (16-byte slots), so a node's corner forces
    // are contiguous.  Double-word mode: fe's bytes hold float2 (hi, lo) pairs,
    // ((float2 *)fe)[k*3 + i].
    double *fe;
    float *fe32;
    // node -> (element, corner) incidences sorted by element id
    const int *node_ptr;
    const int *node_inc;      // e*4 + a
    const int4 *slot;         // per element: CSR positions k of its four corners
    // Dirichlet data
    const int *node_bc;       // per node: -1 or record index
    const int2 *bc_rec;       // per record, per comp: (first entry, count)
    const BCEntry *bcs;
    // Neumann loads (ext_ptr == nullptr without loads).  The external force of
    // DOF d is the sum, in deck order starting from 0, of its terms
    // ext_term[ext_ptr[d] .. ext_ptr[d+1]): EXT_FORCE i = nodal-force entry
    // nfs[i]; EXT_GRAV_ELEM i = grav_e[i] (gravity block b, element e:
    // i = b ne + e); EXT_GRAV_NODE i = grav_n[i] (block b, node: b nn + node;
    // the block's element terms of the node summed in element order, used only
    // as a DOF's first term); EXT_FACE i = fcon[i] (filled each step by the
    // face kernel from that step's u and t).
    const int *ext_ptr;
    const unsigned *ext_term;
    const ForceEntry *nfs;
    const double *grav_e, *grav_n;
    double *fcon;
    const FaceLoad *faces;
    int nfaces;
    // Artificial bulk viscosity (*Bulk viscosity with a nonzero element size;
    // solverExplicit.cpp:381-421, 514-541).  visc != 0: the element kernels add
    // the viscous stress qBV cof(F), qBV = rho/J h (c1^2 h |trD| min(0, trD) +
    // cl c0 trD), trD = tr(F - F_prev)/dt, and roll each element's F_prev
    // diagonal: visc_f0 (3*ne, F_ii, FP64, exact and double-word modes) or
    // visc_h0 (3*ne, H_ii = F_ii - 1, mixed mode), SoA by component.
    int visc;
    double *visc_f0;
    float *visc_h0;
    double visc_h, visc_c1, visc_cl, visc_c0;
    float visc_hf, visc_c1sq_hf, visc_clc0f;   // h, c1^2 h and cl c0 in FP32 (mixed mode)
    // control
    Ctrl *ctrl;                       // [2]
    unsigned long long *dtmin;        // [4]: [0..1] bit patterns of positive doubles (the CFL
                                      // minimum by step parity); [2..3] FP32 bit patterns of the
                                      // running minimum of the elements' FP32 CFL screen
    int *flags;                       // [2] NaN flag raised by the element kernel
    double sf, tf;
};

// A contiguous element (or node) range [begin, end) of one solve.  The step
// kernels of the FP64 and mixed modes take tiles from a list, so one solve and
// many pooled solves run the same kernels.
struct Tile {
    int solve;
    int begin, end;
};

constexpr int kStepThreads = 256;   // upper bound on the CTA size of the tiled step kernels
constexpr int kMaxTileElems = 4096; // upper bound on the elements of one tile

// Tiled step kernels (one instantiation in msx_fast.cu, used by msx_run and
// the pool).  `counts` is kTileSched ints of device memory: element-tile
// count, claim counter, blocks done, then the same three for the node tiles;
// the counters start at zero and every launch leaves them at zero.
constexpr int kTileSched = 6;
void launch_tiled_node(const Problem *descs, const Tile *ntiles, int *counts, int mode, int parity, int grid,
                       int threads, cudaStream_t s);
// tile_elems: the largest tile of etiles (unused: every kernel's shared memory
// is static); act: the instantiation with element birth
// (Problem::act_t set); visc: the one with bulk viscosity (Problem::visc set)
void launch_tiled_elem(const Problem *descs, const Tile *etiles, int *counts, int mode, int parity, int grid,
                       int threads, int tile_elems, cudaStream_t s, bool act = false, bool visc = false);
// CTAs of the tiled element kernel (node kernel when `node` is true) that fit on one SM
int tiled_ctas_per_sm(int mode, int threads, bool node = false);
// Mixed-mode state conversions: u, v, a (FP64) -> uhl, vhl, ahl, and back
// (hi + lo, exact unless the pair spans more than 53 bits); minv -> minv2.
void launch_state_split(const Problem &p, bool mixed, cudaStream_t s);
void launch_state_merge(const Problem &p, bool mixed, cudaStream_t s);
void launch_minv_split(const double *minv, float2 *minv2, long long nn, cudaStream_t s);
// u (SoA) -> the plain FP64 mode's node-major copy u4
void launch_u4_from_u(const double *u, double *u4, long long nn, cudaStream_t s);

// records the message returned by msx_last_error() on this host thread
void msx_set_error(const char *msg);

// launchers (one translation unit per numeric mode)
void launch_node_exact(const Problem &p, int parity, cudaStream_t s);
void launch_elem_exact(const Problem &p, int parity, cudaStream_t s);

// set-up (exact operation order)
// the element set-up of elements [e0, e1) (e1 < 0: to the last element)
void launch_setup_elements(const Problem &p, const double *X, cudaStream_t s, long long e0 = 0, long long e1 = -1);
void launch_setup_mass(const Problem &p, double *mass, double *minv, cudaStream_t s);
// a precision mode's FP32 element arrays (any pointer may be null) from G, wJ and X
void launch_mode_arrays(const Problem &p, float *G32, float *wJ32, float *G32lo, float *wJ32lo, cudaStream_t s);
// Problem::Eref, Mg and rdetE from X and G (the same values the set-up writes)
void launch_cnh_arrays(const Problem &p, cudaStream_t s);
// bulk viscosity: the elements' previous-step F diagonal from displacement u
void launch_visc_init(const Problem &p, const double *u, cudaStream_t s);
// min over elements of Lref/c (undeformed) or min(Lref, L(X+u))/c, into dtmin[slot]
void launch_initial_cfl(const Problem &p, const double *uK, int slot, cudaStream_t s);
// gravity terms per element and their per-node sums (reference order)
void launch_setup_gravity(const Problem &p, double g, double *grav_e, double *grav_n, cudaStream_t s);
// Face contributions of the step whose control slot `parity` the node kernel
// just wrote (its time and displacement); mixed mode reads u as (hi, lo) pairs.
void launch_face_loads(const Problem &p, int parity, bool mixed, cudaStream_t s);
// Values of one field component at n nodes for the current state (node data
// extraction): field as msx_node_field, t = time of the last step, mode = the
// corner-force layout in use (MODE_*).
void launch_node_values(const Problem &p, int mode, int field, int comp, const int *nodes, long long n, double t,
                        double *out, cudaStream_t s);
// Cauchy, Green-Lagrange (9 per element, row-major) and von Mises of the current u
void launch_element_fields(const Problem &p, double t, double *cauchy, double *gl, double *vms, cudaStream_t s);
// Element data extraction: per-element values of a msx_element_quantity, and
// the reduction one extraction row writes (quantity, op as in msx.h), from the
// current u, v and, for the external energy, the loads at time t.  part holds
// element_reduce_scratch() - 1 doubles of partials, out one.
void launch_element_values(const Problem &p, int quantity, const int *elems, long long n, double t, double *out,
                           cudaStream_t s);
void launch_element_reduce(const Problem &p, int quantity, int op, const int *elems, long long n, double t,
                           double *part, double *out, cudaStream_t s);
long long element_reduce_scratch();
// one element pass + gather for f_int(u) (test hook); writes fint[3*nn]
void launch_internal_force_exact(const Problem &p, double *fint, cudaStream_t s);
void launch_internal_force_fp64(const Problem &p, double *fint, cudaStream_t s);
void launch_internal_force_mixed(const Problem &p, double *fint, cudaStream_t s);
void launch_internal_force_dw(const Problem &p, double *fint, cudaStream_t s);
// Law parameters of one material, FP64 and the FP32 / double-word copies; false if invalid.
bool material_params(const msx_material &m, MatParams &o);

// The double-word mode holds values as FP32 (hi, lo) pairs, whose low word
// needs FP32's normal range: material constants and nonzero coordinates must
// lie within [2^-100, 2^100] (a margin for the products the kernels form).
constexpr int kDwExpLimit = 100;
bool dw_in_range(double x);   // x == 0 or 2^-100 <= |x| <= 2^100
bool dw_material_ok(const MatParams &m);
// min nonzero |x| and max |x| over x[0..n) on the device, as the bit patterns
// of non-negative doubles in mm[0], mm[1] (device memory, set here)
void launch_abs_range(const double *x, long long n, unsigned long long *mm, cudaStream_t s);

// Node -> (element, corner) lists in element order (node_ptr[nn + 1],
// node_inc[4 ne], slot[ne]) built on the device from the uploaded conn;
// synchronises s once.  MSX_ERR_ARG (message in err) when a node id is out of
// range; lists with a node in more than kCsrMaxDegree elements are built on the
// host from conn_host instead.
constexpr int kCsrMaxDegree = 1024;
msx_status build_node_csr(const int4 *conn, const int *conn_host, long long ne, long long nn, int *node_ptr,
                          int *node_inc, int4 *slot, cudaStream_t s, std::string &err);

// The Dirichlet tables of one solve, built on the host in O(nbc log nbc)
// (nothing per node): `nodes` holds (node, record) for each node with an
// entry, ascending by node; `rec` three (first entry, count) records per such
// node, one per component; `ent` the entries grouped by DOF, each DOF's in
// input order (the order the reference applies them in).  MSX_ERR_ARG with
// the reason in err for a bad entry.
struct BCTables {
    std::vector<int2> nodes, rec;
    std::vector<BCEntry> ent;
};
msx_status build_bc_tables(long long nn, const msx_bc *bcs, long long nbc, double t0, double tf, BCTables &t,
                           std::string &err);
// node_bc[nn] = -1 except node_bc[nodes[k].x] = nodes[k].y (device arrays)
void launch_node_bc_scatter(int *node_bc, long long nn, const int2 *nodes, long long n, cudaStream_t s);

}  // namespace msx
