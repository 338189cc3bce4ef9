/*
 * msx_oracle.h -- CPU restatement of MuPhiSim v1.1's explicit C3D4 step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA path is checked
 * against; nothing in the product links or calls it.  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg load it.
 *
 * Parity pin: the oracle is validated against the reference itself, built
 * from its own sources behind a small PETSc/MPI shim (oracle/Makefile,
 * oracle/ref_harness.cpp), on the golden decks in tests/golden/.
 *
 * Every routine follows the reference's arithmetic in the same operation
 * order (compile with -ffp-contract=off), so on a host without implicit FMA
 * contraction it reproduces the reference bit for bit.
 */
#ifndef MSX_ORACLE_H
#define MSX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Constitutive laws, named as in the reference's *HyperElastic keyword. */
enum { ORC_NEO_HOOKEAN = 0,          /* "Neo-Hookean" (Belytschko form)      */
       ORC_COMPRESSIBLE_NH = 1,      /* "3D-Compressible-Neo-Hookean"        */
       ORC_STVK = 2,                 /* "St-Venant-Kirchhoff" (3D isotropic)  */
       ORC_LINEAR_ELASTIC = 3 };     /* *Linear-Elastic (small strain, 3D)     */

/* Dirichlet modes: reference *BOUNDARY, TYPE=DISPLACEMENT RAMP / INST, plus
 * the step-ramped velocity extension (no reference counterpart). */
enum { ORC_BC_RAMP = 0, ORC_BC_INST = 1, ORC_BC_VEL_RAMP = 2 };

typedef struct { int32_t law; double young, nu, rho; } orc_material;
/* one nodal force DOF of *BOUNDARY, TYPE=FORCE: value = F_k * Ff over [t0, tf] */
typedef struct { int64_t dof; double t0, tf, value; } orc_force;
typedef struct { int64_t dof; int32_t mode; int32_t ramp_steps; double value; } orc_bc;

/* One Neumann block of the deck (src/solvers/boundaryConditions.cpp:75-138). */
enum { ORC_LOAD_FORCE = 0, ORC_LOAD_GRAVITY = 1, ORC_LOAD_TRACTION_INST = 2, ORC_LOAD_TRACTION_RAMP = 3,
       ORC_LOAD_PRESSURE_INST = 4, ORC_LOAD_PRESSURE_RAMP = 5 };
typedef struct {
    int32_t kind;
    int32_t face;                 /* surface loads: face S (1..4) of every listed tet        */
    double t0, tf;                /* surface loads: active for t0 <= t <= tf                  */
    double value[3];              /* traction (Tx, Ty, Tz); pressure P or gravity g: value[0] */
    const int32_t *elems; int64_t nelems;      /* surface loads: bulk tets, 0-based, deck order */
    const orc_force *forces; int64_t nforces;  /* FORCE block: its entries, deck order          */
} orc_load;

typedef struct {
    int64_t nn, ne;
    const double *X;          /* 3*nn, X[c*nn + node]                        */
    const int32_t *conn;      /* 4*ne, 0-based                               */
    const int32_t *elem_mat;  /* ne material ids, or NULL (all 0)            */
    const orc_material *mats; int32_t nmat;
    const orc_bc *bcs; int64_t nbc;
    double t0, tf, scale_factor;
    int64_t max_steps;        /* 0: run to tf as the reference does          */
    int32_t first_step_zero_uK; /* 1: the reference's chained-solver quirk   */
    int32_t nthreads;
    const orc_force *forces; int64_t nforces;  /* nodal forces, input order   */
    double gravity;           /* *GRAVITY g (0: none), applied on the z DOFs  */
    int32_t gravity_first;    /* 1: *GRAVITY precedes *BOUNDARY, TYPE=FORCE   */
    const orc_load *loads; int64_t nloads;     /* when nloads > 0: all Neumann blocks in deck
                                                  order; forces/gravity above are then unused */
    const double *act_time;   /* ne activation times (first internal variable), or NULL  */
    int32_t activation;       /* 1: the block's *ACTIVATION option (element birth)       */
    double time;              /* element extraction: the time the element states are at */
    /* Artificial viscosity of the explicit solver (solverExplicit.cpp:381-421, 469-541):
     * 0 none, 1 *Bulk viscosity, 2 *Dev viscosity; c1, cl as the keyword reads them
     * (inputFile.cpp:2462-2511).  visc_h and visc_c0 stand for solvers::_elementSize and
     * _c0 (solvers.h:53-54), which the reference never assigns (0 in its builds). */
    int32_t viscosity;
    double visc_c1, visc_cl, visc_h, visc_c0;
    double *F_prev;           /* 9*ne: each element's F at the previous step (the Gauss
                                 point's previous state), in/out; needed with viscosity */
} orc_problem;

typedef struct { int64_t steps; double t, dt_last, dt_init; int32_t status; double loop_seconds; } orc_result;

/* status codes */
enum { ORC_OK = 0, ORC_ERR_NEG_JACOBIAN = 1, ORC_ERR_NAN = 2, ORC_ERR_ARG = 3 };

/* Element set-up: dphi[12*ne] (node-major a*3+j), wJ[ne], Lref[ne]. */
int orc_precompute(int64_t nn, int64_t ne, const double *X, const int32_t *conn,
                   double *dphi, double *wJ, double *Lref);
/* Lumped mass per node (identical for the three components). */
int orc_lumped_mass(int64_t nn, int64_t ne, const int32_t *conn, const double *wJ,
                    const int32_t *elem_mat, const orc_material *mats, double *mass);
/* First Piola stress P(F), row-major 3x3. */
void orc_stress(const orc_material *m, const double *F, double *P);
/* Sound speed of a law. */
double orc_sound_speed(const orc_material *m);
/* Characteristic length (inscribed-sphere diameter) of one tet; x[a*3+c]. */
double orc_char_length(const double *x);
/* Internal force of displacement u: fint[3*nn] (reference scatter order). */
int orc_internal_force(int64_t nn, int64_t ne, const int32_t *conn, const double *dphi,
                       const double *wJ, const int32_t *elem_mat, const orc_material *mats,
                       const double *u, double *fint, double *F_out, double *P_out, int nthreads);
/* Element output fields of displacement u: Cauchy and Green-Lagrange (9 per
 * element) and von Mises (1 per element), as the reference's laws store them. */
int orc_element_fields(int64_t nn, int64_t ne, const int32_t *conn, const double *dphi, const int32_t *elem_mat,
                       const orc_material *mats, const double *u, double *cauchy, double *gl, double *vms);
/* Element data extraction (*EXTRACTION, ELEMENT) at the state u, v: the
 * per-element value of quantity q (numbered as the reference's
 * ExtractData::ElementDataType, 1..30) for the listed elements (elems NULL:
 * all), and the value one extraction row holds for operation op (1 Mean,
 * 2 Min, 3 Max, 4 Sum) over them; fext (3*nn) serves q = 28, the external
 * energy, only.  The problem's X, conn, elem_mat and mats are used. */
int orc_element_values(const orc_problem *p, const double *u, const double *v, int32_t q, const int32_t *elems,
                       int64_t n, double *out);
int orc_element_reduce(const orc_problem *p, const double *u, const double *v, const double *fext, int32_t q,
                       int32_t op, const int32_t *elems, int64_t n, double *value);
/* Full explicit solve; u,v,a (3*nn each) in = initial, out = final.
 * dt_hist (optional) receives one dt per executed step (max_hist entries). */
int orc_run(const orc_problem *p, double *u, double *v, double *a,
            double *dt_hist, int64_t max_hist, orc_result *res);
/* Seeded cube generator: (n+1)^3 nodes, 6 n^3 tets (hex -> 6 tets). */
/* External force of all Neumann blocks at displacement u and time t (3*nn). */
int orc_external_force(const orc_problem *p, const double *u, double t, double *fext);
int orc_cube_mesh(int32_t n, uint64_t seed, double jitter, double *X, int32_t *conn);

#ifdef __cplusplus
}
#endif
#endif
