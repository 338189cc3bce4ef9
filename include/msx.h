/*
 * msx.h -- C ABI of the GB300-native explicit solid-mechanics step.
 *
 * Drop-in for MuPhiSim v1.1's explicit solver path: C3D4 linear tets with one
 * Gauss point, "Neo-Hookean", "3D-Compressible-Neo-Hookean" and
 * "St-Venant-Kirchhoff" laws, lumped mass, central differences, Dirichlet
 * ramp/instantaneous BCs and the CFL stable time step.
 *
 * Conventions (as in the reference):
 *   - nodal fields are SoA float64, entry [dof] with dof = node + comp*num_nodes
 *     (src/spatialDiscretisation/classGPs.cpp:37-67 getLocalDofs);
 *   - connectivity is 0-based int32, 4 nodes per element;
 *   - a solver block runs from t0 to tf with dt = scale_factor * CFL dt
 *     recomputed every step (src/solvers/solverExplicit.cpp:217-276).
 * All functions return an msx_status; none exits the process.  The library
 * owns device memory; the caller owns host buffers.  A handle is used by one
 * host thread at a time; the pool API is thread-safe.
 */
#ifndef MSX_H
#define MSX_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MSX_OK = 0,
    MSX_ERR_ARG = 1,           /* invalid argument (sizes, ids, pointers)            */
    MSX_ERR_CUDA = 2,          /* CUDA runtime failure; see msx_last_error()          */
    MSX_ERR_NEG_JACOBIAN = 3,  /* dt < 1e-20 ("Negative jacobian", solverExplicit.cpp:270-273) */
    MSX_ERR_NAN = 4,           /* non-finite displacement (solverExplicit.cpp:306-308) */
    MSX_ERR_OOM = 5,           /* device memory exhausted / admission refused         */
    MSX_ERR_STATE = 6,         /* call not valid in the handle's current state        */
    MSX_ERR_NO_DEVICE = 7,     /* no CUDA device or not an sm_103 device              */
    MSX_ERR_TIMEOUT = 8,       /* a bounded device-side wait ran out                  */
    MSX_ERR_BUSY = 9           /* pool full: try again after a poll                   */
} msx_status;

enum { MSX_LAW_NEO_HOOKEAN = 0,             /* *HyperElastic, Neo-Hookean                 */
       MSX_LAW_COMPRESSIBLE_NEO_HOOKEAN = 1, /* *HyperElastic, 3D-Compressible-Neo-Hookean */
       MSX_LAW_STVK = 2,                     /* *HyperElastic, St-Venant-Kirchhoff          */
       MSX_LAW_LINEAR_ELASTIC = 3 };         /* *Linear-Elastic (small strain; 3D isotropic) */

enum { MSX_BC_RAMP = 0,      /* *BOUNDARY, TYPE=DISPLACEMENT RAMP: value reached at tf         */
       MSX_BC_INST = 1,      /* *BOUNDARY, TYPE=DISPLACEMENT INST: value applied at first step */
       MSX_BC_VEL_RAMP = 2,  /* extension: velocity ramped linearly to `value` over ramp_steps */
       MSX_BC_RAMP_RATE = 3 };/* a ramp given by its rate U/(tf - t0), the value a ramped
                                 classDirichlet stores (getUU(), classNodes.cpp:66-73)     */

enum { MSX_PREC_FP64 = 0,        /* plain FP64, FMA-contracted, algebraically simplified laws */
       MSX_PREC_FP64_EXACT = 1,  /* FP64 in the reference's operation order, no contraction   */
       MSX_PREC_MIXED = 2,       /* FP32 element kinematics, stress, B^T P, J-1 and ln J (trace
                                    summed exactly); nodal u, v as double-word FP32 pairs
                                    (~48 bits), a in FP32; the stable dt is the FP64 CFL
                                    minimum (FP32 screen, FP64 recheck of the near-minimum
                                    elements)                                                  */
       MSX_PREC_DOUBLE_WORD = 3  /* MSX_PREC_FP64's algebra in double-word (FP32 pair, ~48-bit)
                                    arithmetic on the FP32 pipe, state and corner forces too;
                                    FP64 CFL check.  Values must stay inside FP32's exponent
                                    range: msx_create, msx_next_solver and msx_pool_submit
                                    refuse (MSX_ERR_ARG) material constants or nonzero
                                    coordinates outside [2^-100, 2^100] for this mode. */ };

typedef struct {
    int64_t num_nodes, num_elems;
    const double *X;              /* 3*num_nodes coordinates, X[c*num_nodes + node]        */
    const int32_t *conn;          /* 4*num_elems node ids                                  */
    const int32_t *elem_material; /* num_elems material ids, or NULL for material 0       */
} msx_mesh;

typedef struct {
    int32_t law;
    int32_t reserved;
    double young, nu, rho;        /* *HyperElastic "E, nu" and *Density                   */
} msx_material;

typedef struct {
    int64_t dof;                  /* node + comp*num_nodes (deck line "node, comp, value") */
    int32_t mode;                 /* MSX_BC_*                                              */
    int32_t ramp_steps;           /* MSX_BC_VEL_RAMP only                                  */
    double value;
} msx_bc;

typedef struct {
    double t0, tf, scale_factor;  /* *Time t0, tf and *Scale Factor                        */
    int64_t max_steps;            /* 0: run to tf like the reference; >0: stop after N     */
    int32_t precision;            /* MSX_PREC_*                                            */
    int32_t steps_per_graph;      /* steps per full CUDA-graph chunk; 0 = default (64)     */
} msx_solver_opts;

typedef struct {
    int64_t steps;                /* steps executed by this call                           */
    int64_t total_steps;          /* steps executed in this solver block so far            */
    double t, dt, dt_init;        /* time reached, last dt, initial dt of the block        */
    int32_t status;               /* msx_status of the run                                 */
    int32_t reserved;
    double device_ms;             /* device time of the call (CUDA events)                 */
    int64_t kernel_launches;      /* step kernels launched by the call (incl. no-op tail)   */
} msx_run_report;

typedef struct {
    double element_ms, node_ms;   /* mean duration of one element / node kernel launch     */
    int64_t element_launches, node_launches;
    double element_alg_bytes, node_alg_bytes; /* algorithmic bytes per launch              */
} msx_profile_report;

typedef struct msx_handle msx_handle;

/* Mesh, materials, BCs and the first solver block: uploads the mesh, builds
 * the per-element shape-function gradients, wJ, reference characteristic
 * lengths, lumped mass and node->corner CSR on the device.
 * Replaces the set-up of classSolverExplicit::calculate
 * (src/solvers/solverExplicit.cpp:63-215) fed by the input deck readers
 * (src/IO/inputFile.cpp:20-323, 838-1029, 2253-2831, 2960-3218). */
msx_status msx_create(const msx_mesh *mesh, const msx_material *mats, int32_t num_mats,
                      const msx_bc *bcs, int64_t num_bcs, const msx_solver_opts *opts,
                      msx_handle **out);

/* Advance the current solver block to tf (or opts.max_steps, or the extra
 * cap max_steps > 0 of this call).  Replaces the time loop of
 * classSolverExplicit::calculate (src/solvers/solverExplicit.cpp:217-338). */
msx_status msx_run(msx_handle *h, int64_t max_steps, msx_run_report *report);

/* Final nodal fields, host buffers of 3*num_nodes doubles each (any may be
 * NULL).  Replaces solvers::getFinalValues (src/solvers/solvers.h:171-187). */
msx_status msx_get_state(msx_handle *h, double *u, double *v, double *a);

/* Initial nodal fields.  Replaces solvers::initValues (src/solvers/solvers.h:171-187). */
msx_status msx_set_state(msx_handle *h, const double *u, const double *v, const double *a);

/* Start the next *SOLVER, EXPLICIT block with the current state, as the
 * reference's solver chain does (src/main.cpp:162-181). */
msx_status msx_next_solver(msx_handle *h, const msx_bc *bcs, int64_t num_bcs,
                           const msx_solver_opts *opts);

/* One nodal-force DOF of *BOUNDARY, TYPE=FORCE (deck block "t0, tf, Ff" then
 * "node, Fx, Fy, Fz" lines): value = F_comp * Ff; the force at time t is
 * value/(tf - t0) * t for t0 <= t <= tf and 0 outside, as
 * classNeumann::getTracAmount computes it (spatialDiscretisation/classNodes.h:101-109). */
typedef struct {
    int64_t dof;
    double t0, tf, value;
} msx_nodal_force;

/* Neumann loads of the explicit path (solvers/boundaryConditions.cpp:75-138):
 * nodal forces in deck order and *GRAVITY g (force -w rho |J| g phi on the z
 * DOFs, :1146-1171; 0 for none).  gravity_first = 1 when *GRAVITY comes before
 * the force blocks in the deck (the summation order of the reference).
 * Replaces any loads set before; takes effect from the next step. */
msx_status msx_set_loads(msx_handle *h, const msx_nodal_force *forces, int64_t num_forces, double gravity,
                         int32_t gravity_first);

/* One Neumann block of the deck, for msx_set_load_blocks.  Replaces the
 * reference's classNeumannBCs list (solvers/classNeumannBCs.h:32-181) as built
 * by NeumannCommonManagement (IO/inputFile.cpp:4705-4760) and applied by
 * NeumannBCManagement (solvers/boundaryConditions.cpp:75-138). */
typedef enum {
    MSX_LOAD_FORCE = 0,          /* *BOUNDARY, TYPE=FORCE: `forces` (value = F_k * Ff)        */
    MSX_LOAD_GRAVITY = 1,        /* *GRAVITY g = value[0]                                      */
    MSX_LOAD_TRACTION_INST = 2,  /* *BOUNDARY, TYPE=TRACTION INST: t0, tf, Tx, Ty, Tz, S       */
    MSX_LOAD_TRACTION_RAMP = 3,  /* *BOUNDARY, TYPE=TRACTION RAMP: T (t - t0)/(tf - t0)        */
    MSX_LOAD_PRESSURE_INST = 4,  /* *BOUNDARY, TYPE=PRESSURE INST: t0, tf, P, S; follower load */
    MSX_LOAD_PRESSURE_RAMP = 5   /* *BOUNDARY, TYPE=PRESSURE RAMP: P (t - t0)/(tf - t0)        */
} msx_load_kind;

typedef struct {
    int32_t kind;                       /* msx_load_kind */
    int32_t face;                       /* traction/pressure: face S (1..4) of every listed tet */
    double t0, tf;                      /* traction/pressure: active for t0 <= t <= tf          */
    double value[3];                    /* traction (Tx, Ty, Tz); pressure P, gravity g: [0]    */
    const int32_t *elems;               /* traction/pressure: bulk tets, 0-based, deck order    */
    int64_t num_elems;
    const msx_nodal_force *forces;      /* FORCE: entries, deck order                           */
    int64_t num_forces;
} msx_load_block;

/* All Neumann loads as blocks in deck order: each DOF's external force is
 * summed block by block in that order, as the reference sums it.  Pressure
 * follows the deformation (J F^-T n0 of the face's tet at the step's u);
 * a ramped pressure loads the tet's first node, as the reference does
 * (boundaryConditions.cpp:370-452).  Replaces any loads set before (by either
 * call); takes effect from the next step. */
msx_status msx_set_load_blocks(msx_handle *h, const msx_load_block *blocks, int64_t num_blocks);

/* The Neumann blocks of an input deck, read from the file by the library:
 * one msx_load_block per *BOUNDARY, TYPE=FORCE | TRACTION INST|RAMP |
 * PRESSURE INST|RAMP and *GRAVITY block, in file order, as
 * NeumannCommonManagement (IO/inputFile.cpp:4705-4760) scans the whole file
 * and builds one classNeumannBCs per block.  For a solver plugin inside the
 * reference, which holds the deck's path (GeneralOptions::getInputFilePath)
 * but whose load objects keep their t0, tf and amounts private.  Force
 * entries: dof = node + comp * num_nodes, value = F_comp * Ff; surface loads:
 * 0-based bulk tets.  The blocks stay valid until msx_deck_loads_free. */
typedef struct msx_deck_loads msx_deck_loads;
msx_status msx_deck_read_loads(const char *path, int64_t num_nodes, msx_deck_loads **out);
msx_status msx_deck_loads_blocks(const msx_deck_loads *loads, const msx_load_block **blocks, int64_t *num_blocks);
msx_status msx_deck_loads_free(msx_deck_loads *loads);

/* Element birth: the reference's *ACTIVATION option of a solver block
 * (solvers.cpp:403-433, called each step at solverExplicit.cpp:259-264) with the
 * activation times *INITINTVARS sets as the first internal variable of
 * St-Venant-Kirchhoff and linear-elastic elements (IO/inputFile.cpp:2055-2111;
 * elements without one have 0).  activation_time: num_elems values, or NULL to
 * keep the current ones; enabled: 1 for blocks with *ACTIVATION (applies from
 * the next step of the current block on, and to later blocks until changed).
 * While enabled, such an element whose activation time is above the step's time
 * is dead: it adds no internal force (solverExplicit.cpp:370-371), its output
 * fields are zero and element extraction skips or zeroes it as the reference
 * does; the neo-Hookean laws have no activation time and are always alive.  The
 * lumped mass and the stable time step include every element, as there.  Not
 * available in msx_pool_*. */
msx_status msx_set_activation(msx_handle *h, const double *activation_time, int32_t enabled);

/* Artificial viscosity of the explicit solver: *Bulk viscosity (kind
 * MSX_VISC_BULK) and *Dev viscosity (MSX_VISC_DEV) with the "c1, cl" the
 * deck gives (defaults 0.06, 1.2 and 1, 0.5: IO/inputFile.cpp:2462-2511), the
 * second pass of classSolverExplicit::computeInternalForce
 * (solverExplicit.cpp:381-421).  Bulk: per element trD = tr(F - F_prev)/dt
 * (F_prev: the element's F at the previous step, the handed-over state's at a
 * block start), qBV = rho/J h (c1^2 h |trD| min(0, trD) + cl c0 trD) and the
 * viscous Piola stress J qBV F^-T, integrated as wJ B^T P (bulkViscosity,
 * :514-541).  h and c0 are the reference's solvers::_elementSize and _c0
 * (solvers.h:53-54), which it never assigns: its builds run with 0, which
 * makes the viscous force zero, and element_size = 0 here does the same
 * (results bit for bit those without viscosity).  A nonzero element_size
 * applies the formula with the given h and c0.  Deviatoric: the reference
 * scales the deviatoric rate but maps the still-zero Cauchy tensor to P
 * (:469-502), so it adds nothing, whatever its parameters; here too.
 * MSX_VISC_NONE turns it off.  Applies from the next step, also to later
 * solver blocks (the reference's flag stays set); msx_internal_force leaves it
 * out.  Not together with element birth, not in msx_pool_*. */
enum { MSX_VISC_NONE = 0, MSX_VISC_BULK = 1, MSX_VISC_DEV = 2 };
msx_status msx_set_viscosity(msx_handle *h, int32_t kind, double c1, double cl, double element_size, double c0);

/* Nodal values of the current state for the reference's node data extraction
 * (*EXTRACTION, NODE: solvers/dataExtraction.cpp:778-840, written every step by
 * classSolverExplicit::calculate, solverExplicit.cpp:325).  field: displacement
 * ("Unknown"), external force or internal force of the last step; component
 * comp (0..2) of the n listed nodes (0-based) into out[n].  The internal force
 * is summed from zero in element order, as computeInternalForce scatters it. */
typedef enum { MSX_FIELD_DISPLACEMENT = 0, MSX_FIELD_EXTERNAL_FORCE = 1, MSX_FIELD_INTERNAL_FORCE = 2 } msx_node_field;
msx_status msx_node_values(msx_handle *h, int32_t field, int32_t comp, const int32_t *nodes, int64_t n, double *out);

/* Element data extraction (*EXTRACTION, ELEMENT: classElementData and
 * classExtractData, solvers/dataExtraction.cpp:304-470 and 508-890, written
 * every step by solverExplicit.cpp:325).  The quantities carry the numbers of
 * the reference's ExtractData::ElementDataType and the operations those of
 * ExtractData::Operation (solvers/dataExtraction.h:23-29), so a caller casts
 * them across.  Values are taken at the state of the last step: F = I + grad u,
 * the law's first Piola-Kirchhoff P, von Mises of P F^T / det F (SVM), SVM det F
 * (KVM), the internal variables (none of the three laws has more than one, so
 * INVAR1..6 read zero, dataExtraction.cpp:552-557), the law's strain energy
 * density (DEFO_ENERGY; zero for the Neo-Hookean law, which keeps the default),
 * the kinetic energy density 0.5 rho |v(centroid)|^2 (KIN_ENERGY) and the
 * current volume wJ det F (VOLUME). */
typedef enum {
    MSX_ELEM_FXX = 1, MSX_ELEM_FXY, MSX_ELEM_FXZ, MSX_ELEM_FYX, MSX_ELEM_FYY, MSX_ELEM_FYZ, MSX_ELEM_FZX,
    MSX_ELEM_FZY, MSX_ELEM_FZZ,
    MSX_ELEM_PXX = 10, MSX_ELEM_PXY, MSX_ELEM_PXZ, MSX_ELEM_PYX, MSX_ELEM_PYY, MSX_ELEM_PYZ, MSX_ELEM_PZX,
    MSX_ELEM_PZY, MSX_ELEM_PZZ,
    MSX_ELEM_SVM = 19, MSX_ELEM_KVM = 20,
    MSX_ELEM_INVAR1 = 21, MSX_ELEM_INVAR2, MSX_ELEM_INVAR3, MSX_ELEM_INVAR4, MSX_ELEM_INVAR5, MSX_ELEM_INVAR6,
    MSX_ELEM_DEFO_ENERGY = 27, MSX_ELEM_EXTERNAL_ENERGY = 28, MSX_ELEM_KIN_ENERGY = 29, MSX_ELEM_VOLUME = 30
} msx_element_quantity;
typedef enum { MSX_OP_MEAN = 1, MSX_OP_MIN = 2, MSX_OP_MAX = 3, MSX_OP_SUM = 4 } msx_element_op;

/* Per-element value of `quantity` for the n listed elements (0-based; elems
 * NULL means all, n then ignored) into out[n] (all: out[num_elems]), in list
 * order.  EXTERNAL_ENERGY is not per element and is refused. */
msx_status msx_element_values(msx_handle *h, int32_t quantity, const int32_t *elems, int64_t n, double *out);

/* The number the reference writes in one row of an element extraction over
 * the listed elements (elems NULL: all), reduced on the device.  Each listed
 * element counts once, whatever its order or repeats, as the reference selects
 * the Gauss points of the listed elements (classElementData::initialise, :441-464).
 *   F..INVAR6  Mean sum(v dV)/V, Sum sum(v dV), Max, Min of v, with dV = wJ
 *              and V = sum(dV) (classElementData::getValue, :338-378);
 *   DEFO_ENERGY, KIN_ENERGY  Mean sum(w dV)/V, Sum sum(w dV), Max, Min of the
 *              density w (defoEnergy, kineticEnergy :569-688);
 *   VOLUME     Sum, Max, Min of wJ det F (volume :690-748; its Mean returns no
 *              value in the reference and is refused here);
 *   EXTERNAL_ENERGY  u . f_ext over every DOF whatever op and list (:853-861).
 * Sums run in a fixed tree order, so a result differs from the reference's
 * element-order sum by rounding only and repeats bit for bit from run to run.
 * An empty list is refused (the reference builds no extraction for it). */
msx_status msx_element_reduce(msx_handle *h, int32_t quantity, int32_t op, const int32_t *elems, int64_t n,
                              double *value);

msx_status msx_destroy(msx_handle *h);

/* Message of the last failing call on this host thread. */
const char *msx_last_error(void);

/* Internal force f_int(u) for host u (3*num_nodes), host fint out: one element
 * pass plus the CSR gather (classSolverExplicit::computeInternalForce,
 * src/solvers/solverExplicit.cpp:363-379; the elastic part: artificial
 * viscosity depends on the previous step and is left out).  Leaves the solver
 * state untouched. */
msx_status msx_internal_force(msx_handle *h, const double *u, double *fint);

/* Per-element set-up data and per-node lumped mass: G[9*num_elems] (rows of
 * the inverse reference Jacobian = dphi of local nodes 1..3), wJ, Lref
 * [num_elems], mass[num_nodes] (classLinearTetrahedra.cpp:129-268,
 * solverExplicit.cpp:429-459).  Any pointer may be NULL. */
msx_status msx_get_element_data(msx_handle *h, double *G, double *wJ, double *Lref, double *mass);

/* Initial dt of the current solver block (the undeformed CFL times the scale
 * factor, solverExplicit.cpp:165-166); sets the block up without stepping.
 * The reference derives its output cadence from it (solverExplicit.cpp:171-174). */
msx_status msx_initial_dt(msx_handle *h, double *dt_init);

/* Element output fields of the current state, host buffers: Cauchy stress and
 * Green-Lagrange strain (9 doubles per element, row-major) and von Mises
 * stress (1 per element), in the reference's operation order
 * (maths.cpp:1227-1271; the Neo-Hookean law's own sigma; zero strain for the
 * compressible neo-Hookean law, which never updates it).  Any may be NULL.
 * Computed on the device only when called, i.e. at output steps. */
msx_status msx_element_fields(msx_handle *h, double *cauchy, double *green_lagrange, double *von_mises);

/* Run `steps` steps launching each kernel separately with CUDA events around
 * it on the library's stream, and report the mean kernel durations. */
msx_status msx_profile(msx_handle *h, int64_t steps, msx_profile_report *report);

/* Seeded unit-cube mesh: (n+1)^3 nodes, 6 n^3 tets (each hex split into six
 * around its N1-N7 diagonal as applications/tools/Hex2Tet-Parallel/
 * Hex2Tet-Partitioning.py:87-110 does), interior nodes jittered by
 * jitter*h*(2r-1), r from splitmix64(seed) in node order. */
msx_status msx_mesh_cube(int32_t n, uint64_t seed, double jitter, double *X, int32_t *conn);

/* The library's CUDA stream (cudaStream_t) for callers that time it. */
void *msx_stream(msx_handle *h);

/* Select the CUDA device used by later msx_create calls on this host thread
 * (one process per GPU: pass the local rank). */
msx_status msx_set_device(int32_t device);

/* Largest element count msx_internal_force_noalloc accepts (its scratch holds
 * 12 corner-force doubles per element: 6 MiB per GPU). */
#define MSX_NOALLOC_MAX_ELEMS 65536

/* No counterpart in the reference: an allocation-free variant of
 * msx_internal_force for callers that cannot call cudaMalloc (for example a
 * host application that owns all device memory through its own allocator,
 * code that must not trigger the device synchronisation cudaMalloc/cudaFree
 * can cause, or work enqueued while a stream is being captured into a graph).
 * It computes f_int(u) for one material (any of the four laws) in the
 * reference's operation order, bit-identical to msx_internal_force on an
 * MSX_PREC_FP64_EXACT handle.
 * Every array is DEVICE memory owned by the caller: X[3*num_nodes] (SoA),
 * conn[4*num_elems], node_ptr[num_nodes+1] and node_inc[4*num_elems] (for
 * each node, e*4+corner of its incident elements in increasing element order),
 * u[3*num_nodes] in, fint[3*num_nodes] out.  conn must be 16-byte aligned,
 * X, u and fint 8-byte aligned, node_ptr and node_inc 4-byte aligned; other
 * pointers are rejected with MSX_ERR_ARG.  Work is enqueued on `stream` (a
 * cudaStream_t, NULL for the default stream) and is not waited for.  The
 * corner forces go to a fixed scratch array inside the library, so num_elems
 * above MSX_NOALLOC_MAX_ELEMS is rejected with MSX_ERR_ARG.  Each call looks
 * up that array's device address (cudaGetSymbolAddress) with the device
 * current, so a device reset between calls is harmless; the first call on a
 * device may load the library's device code, so make it before capturing a
 * stream.  All calls share the one array, which keeps the last call's
 * contents; each call writes every entry it reads, but calls whose work
 * overlaps on the GPU race on it. */
msx_status msx_internal_force_noalloc(const double *X, const int32_t *conn, int64_t num_nodes,
                                      int64_t num_elems, const int32_t *node_ptr,
                                      const int32_t *node_inc, const msx_material *material,
                                      const double *u, double *fint, void *stream);

/* ------------------------------------------------------------------------
 * Batched / serving pool: many independent solves resident on the device,
 * stepped together by one persistent, graph-captured step kernel pair.
 * Each solve is one mesh + material + BCs + solver block (tf or max_steps).
 * ------------------------------------------------------------------------ */
typedef struct msx_pool msx_pool;

typedef struct {
    int64_t hbm_budget_bytes;     /* admission limit for resident solves (0 = 80% free) */
    int32_t max_slots;            /* concurrent solves                                   */
    int32_t precision;            /* MSX_PREC_FP64, MSX_PREC_MIXED or MSX_PREC_DOUBLE_WORD */
    int32_t elems_per_block;      /* element-kernel CTA size; 0 = autotuned             */
    int32_t steps_per_launch;     /* steps per graph replay; 0 = default                */
    const char *tune_cache;       /* autotuner cache file, or NULL                       */
} msx_pool_opts;

typedef struct {
    int64_t ticket;
    int32_t status;               /* msx_status of the solve                            */
    int32_t reserved;
    int64_t steps;
    double t;
    double submit_to_done_ms;     /* wall latency from submit to completion            */
} msx_pool_result;

msx_status msx_pool_create(const msx_pool_opts *opts, msx_pool **out);
/* Admit a solve (copies host inputs); MSX_ERR_BUSY if slots/HBM are full
 * (a finished solve frees its slot at once, its HBM when it is fetched). */
msx_status msx_pool_submit(msx_pool *p, const msx_mesh *mesh, const msx_material *mat,
                           const msx_bc *bcs, int64_t num_bcs, const msx_solver_opts *opts,
                           int64_t *ticket);
/* Advance every resident solve by up to `steps` steps (graph replays of
 * steps_per_launch steps).  Keeps one replay in flight: waits for the previous
 * one, collects its finished solves, launches the next and returns without
 * waiting for it, so the caller's next admissions overlap it.
 * MSX_ERR_STATE while the pool is serving. */
msx_status msx_pool_step(msx_pool *p, int64_t steps);
/* Serving mode on (enabled != 0) or off.  On: a thread of the library launches
 * replays back to back while any solve is resident and sleeps while none is;
 * msx_pool_submit admits new solves between replays, msx_pool_poll returns the
 * finished ones, msx_pool_wait blocks until a ticket is done.  Admissions build
 * their tables and upload their data without holding the pool's lock, so they
 * overlap the running replays.  Off: waits for the replay in flight and stops
 * the thread; msx_pool_step drives the pool again.  A CUDA failure in the
 * serving thread stops the stepping and is returned by the next poll or wait
 * (and by turning serving off).  Results are the same as with msx_pool_step:
 * only the host-side driving differs. */
msx_status msx_pool_serve(msx_pool *p, int32_t enabled);
/* Finished solves collected so far (never waits; takes in the replay in flight
 * if it has completed): fills up to max results, returns the count in *n.
 * u, v, a of a solve are copied out by msx_pool_fetch. */
msx_status msx_pool_poll(msx_pool *p, msx_pool_result *results, int32_t max, int32_t *n);
/* Copy a finished solve's u, v, a (host buffers of 3*num_nodes doubles, any
 * may be NULL; page-locked buffers copy fastest) and release its device memory.
 * The result stays on the device until then, counted against the HBM budget.
 * The copies run on a stream of their own without the pool's lock, so the
 * replays, admissions and polls of other threads go on meanwhile. */
msx_status msx_pool_fetch(msx_pool *p, int64_t ticket, double *u, double *v, double *a);
/* Step the pool until solve `ticket` has finished and fill its result (the
 * other resident solves advance too; their results are kept for poll/fetch).
 * MSX_ERR_ARG if the ticket is unknown or already fetched. */
msx_status msx_pool_wait(msx_pool *p, int64_t ticket, msx_pool_result *result);
msx_status msx_pool_destroy(msx_pool *p);

typedef struct {
    int32_t active, finished_unfetched;   /* resident solves; results awaiting fetch      */
    int32_t threads, tile_elems;          /* schedule in use (after autotuning)            */
    int32_t ctas_per_sm, steps_per_launch;
    int64_t element_steps;                /* sum over all solves of elements x steps done  */
    int64_t used_bytes, budget_bytes;     /* HBM held by resident solves / admission limit */
} msx_pool_stats;

/* Counters of the pool (reads the device control table). */
msx_status msx_pool_stats_get(msx_pool *p, msx_pool_stats *stats);

/* Fault injection for tests of the admission path (no counterpart in the
 * reference): the next `count` calls of msx_pool_submit fail their device
 * allocation as if cudaMallocAsync had run out of memory, after the slot and
 * its HBM were reserved, so they take the same release path as a real
 * failure and return MSX_ERR_OOM.  Resident solves are not touched.
 * count = 0 disarms it. */
msx_status msx_pool_inject_alloc_failures(msx_pool *p, int32_t count);

#ifdef __cplusplus
}
#endif
#endif
