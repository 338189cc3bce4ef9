// solverExplicitGPU.h -- the reference-side binding of the explicit C3D4 step:
// a `solvers` plugin (src/solvers/solvers.h:98-101) that hands one
// *SOLVER, EXPLICIT block of MuPhiSim to libmsx (include/msx.h) in place of
// classSolverExplicit::calculate (src/solvers/solverExplicit.cpp:63-361).
//
// A maintainer adds this header to src/solvers/, includes it from
// solversList.h, constructs classSolverExplicitGPU in solverManagement
// (src/IO/inputFile.cpp:2312-2327, 2727-2738) for `*SOLVER, EXPLICIT GPU` with
// the arguments classSolverExplicit gets plus a precision (MSX_PREC_*), and
// links with -lmsx.  It covers decks of C3D4 elements with the Neo-Hookean,
// compressible Neo-Hookean, St-Venant-Kirchhoff and linear-elastic laws,
// Dirichlet BCs, element birth (*ACTIVATION), artificial viscosity (the
// factory's flag_AV and para_AV, as classSolverExplicit gets them) and the Neumann loads of the
// explicit path (nodal forces, gravity, traction and pressure, instantaneous
// and ramped).  The reference's load classes keep their t0, tf and amounts
// private, so the loads are read from the deck file itself by the library
// (msx_deck_read_loads on GeneralOptions::getInputFilePath()), and each block
// is checked against the reference's own load object through its public
// getters (class, node ids, element count, amount at the block's tf): a deck
// that does not match the loaded model stops the block with an error.
// The state hand-off is the reference's own: initValues() before calculate,
// getFinalValues() after, through the protected _u, _v, _a.
//
// Errors follow the reference's convention at this boundary: ERROR(...) and
// exit(-1) (configuration.h:111-113).
#pragma once
#include <cstdint>
#include <cstdlib>
#include <map>
#include <string>
#include <typeinfo>
#include <vector>

#include "classElements.h"
#include "classGPs.h"
#include "classNeumannBCs.h"
#include "classNodes.h"
#include "commandLine.h"
#include "configuration.h"
#include "hyperElasticNeoHookean.h"
#include "hyperElasticStVenantKirchhoff.h"
#include "linearElastic.h"
#include "msx.h"
#include "solvers.h"

namespace msx_binding {

// E and nu of a law object.  The reference keeps them protected, without
// getters; a member pointer named through a derived class reads them without
// changing the reference (a maintainer may add getters instead).
template <class Law>
struct LawParams : Law {
    static double young(const Law &m) { return m.*(&LawParams::_Young); }
    static double nu(const Law &m) { return m.*(&LawParams::_nu); }
};

template <class Law>
inline void fill(const constitutiveModels &law, int32_t id, msx_material &m)
{
    const Law &c = static_cast<const Law &>(law);
    m.law = id;
    m.young = LawParams<Law>::young(c);
    m.nu = LawParams<Law>::nu(c);
}

// The msx_material of one of the four laws on the path; the class must match
// exactly (the stochastic and thermal variants are other laws).  False for
// any other law.
inline bool material_of(const constitutiveModels &law, msx_material &m)
{
    m = msx_material{};
    m.rho = law.getRho();
    const std::type_info &t = typeid(law);
    if (t == typeid(classHyperElasticNeoHookean))
        fill<classHyperElasticNeoHookean>(law, MSX_LAW_NEO_HOOKEAN, m);
    else if (t == typeid(classHyperElastic3DCompressibleNeoHookean))
        fill<classHyperElastic3DCompressibleNeoHookean>(law, MSX_LAW_COMPRESSIBLE_NEO_HOOKEAN, m);
    else if (t == typeid(classHyperElasticStVenantKirchhoff))
        fill<classHyperElasticStVenantKirchhoff>(law, MSX_LAW_STVK, m);
    else if (t == typeid(linearElastic))
        fill<linearElastic>(law, MSX_LAW_LINEAR_ELASTIC, m);
    else
        return false;
    return true;
}

// One classDirichlet as an msx_bc.  getMe() is node + direction * Nn and
// getUU() what the constructor stored (classNodes.cpp:58-74): U for an
// instantaneous BC (flag 1), U / duration for a ramp (flag -1), which goes to
// the library as that rate so that no division is redone; flag 0 (an
// instantaneous BC already applied) adds nothing and holds v and a at zero,
// which a ramp of rate 0 does (solverExplicit.cpp:545-575).
inline msx_bc bc_of(const classDirichlet &d)
{
    msx_bc b{};
    b.dof = d.getMe();
    b.ramp_steps = 0;
    const int flag = d.getflagDiri();
    b.mode = flag == 1 ? MSX_BC_INST : MSX_BC_RAMP_RATE;
    b.value = flag == 0 ? 0.0 : d.getUU();
    return b;
}

// Whether block B (read from the deck by the library) is the reference's load
// object L, as far as L's public getters show: the class for the kind, then
// the node ids and the amount at B's tf computed as L computes it
// (classNodes.h:101-109 for nodal forces: F / (tf - t0) * t; classNeumannBCs.h
// for tractions and pressures), the number of faces of a surface load (one
// per listed tet in a serial run) and g.  Empty when they agree, else why not.
inline std::string load_mismatch(const msx_load_block &B, classNeumannBCs *L, int64_t nn)
{
    const std::type_info &t = typeid(*L);
    const double tf = B.tf, dt = 0.0;
    switch (B.kind) {
    case MSX_LOAD_FORCE: {
        if (t != typeid(classNodalForces)) return "a nodal-force block where the model has " + L->getType();
        vector<classNeumann *> &nodes = static_cast<classNodalForces *>(L)->getListOfNodes();
        if ((int64_t)nodes.size() * 3 != B.num_forces) return "a different number of force nodes";
        for (size_t i = 0; i < nodes.size(); i++) {
            const msx_nodal_force *f = B.forces + 3 * i;
            if (f[0].dof != nodes[i]->getMe()) return "a different force node";
            const vector<double> F = nodes[i]->getTracAmount(f[0].tf, dt);
            for (int c = 0; c < 3; c++)
                if (F[c] != f[c].value / (f[c].tf - f[c].t0) * f[c].tf) return "a different nodal force";
        }
        return "";
    }
    case MSX_LOAD_GRAVITY:
        if (t != typeid(classGravity)) return "a gravity block where the model has " + L->getType();
        return static_cast<classGravity *>(L)->getGravity() == B.value[0] ? "" : "a different g";
    case MSX_LOAD_TRACTION_INST:
    case MSX_LOAD_TRACTION_RAMP: {
        const bool ramp = B.kind == MSX_LOAD_TRACTION_RAMP;
        double T[3] = {0, 0, 0};
        size_t faces = 0;
        if (!ramp && t == typeid(classTractionInst)) {
            auto *x = static_cast<classTractionInst *>(L);
            x->getTraction(tf, dt, T[0], T[1], T[2]);
            faces = x->getListOfElements().size();
        } else if (ramp && t == typeid(classTractionRamp)) {
            auto *x = static_cast<classTractionRamp *>(L);
            x->getTraction(tf, dt, T[0], T[1], T[2]);
            faces = x->getListOfElements().size();
        } else {
            return std::string("a traction block where the model has ") + L->getType();
        }
        if ((int64_t)faces != B.num_elems) return "a different number of traction faces";
        for (int c = 0; c < 3; c++) {
            const double want = ramp ? B.value[c] / (B.tf - B.t0) * (tf - B.t0) : B.value[c];
            if (T[c] != want) return "a different traction";
        }
        return "";
    }
    case MSX_LOAD_PRESSURE_INST:
    case MSX_LOAD_PRESSURE_RAMP: {
        const bool ramp = B.kind == MSX_LOAD_PRESSURE_RAMP;
        double P = 0;
        size_t faces = 0;
        if (!ramp && t == typeid(classPressureInst)) {
            auto *x = static_cast<classPressureInst *>(L);
            P = x->getPressure(tf, dt);
            faces = x->getListOfElements().size();
        } else if (ramp && t == typeid(classPressureRamp)) {
            auto *x = static_cast<classPressureRamp *>(L);
            P = x->getPressure(tf, dt);
            faces = x->getListOfElements().size();
        } else {
            return std::string("a pressure block where the model has ") + L->getType();
        }
        if ((int64_t)faces != B.num_elems) return "a different number of pressure faces";
        const double want = ramp ? B.value[0] / (B.tf - B.t0) * (tf - B.t0) : B.value[0];
        return P == want ? "" : "a different pressure";
    }
    default:
        return "an unknown load kind";
    }
}

// The model's Neumann loads as msx_load_blocks read from the deck file, each
// checked against the reference's object; `keep` owns the blocks.
inline std::string loads_of(const std::string &deck, vector<classNeumannBCs *> &NeumannBCs, int64_t nn,
                            msx_deck_loads *&keep, const msx_load_block *&blocks, int64_t &nblocks)
{
    keep = nullptr;
    if (msx_deck_read_loads(deck.c_str(), nn, &keep) != MSX_OK || msx_deck_loads_blocks(keep, &blocks, &nblocks) != MSX_OK)
        return msx_last_error();
    if (nblocks != (int64_t)NeumannBCs.size())
        return "the deck " + deck + " has " + std::to_string(nblocks) + " Neumann blocks, the model " +
               std::to_string(NeumannBCs.size());
    for (int64_t k = 0; k < nblocks; k++) {
        const std::string why = load_mismatch(blocks[k], NeumannBCs[k], nn);
        if (!why.empty()) return "Neumann block " + std::to_string(k + 1) + " of " + deck + ": " + why;
    }
    return "";
}

}  // namespace msx_binding

class classSolverExplicitGPU : public solvers {
  public:
    // The arguments of classSolverExplicit's constructor (solverExplicit.h), with
    // flag_AV and para_AV = {c1, cl} of *Bulk viscosity (1) / *Dev viscosity (2),
    // plus the precision.
    classSolverExplicitGPU(vector<classNodes *> &nod, int ndim, int numDof, vector<classDirichlet *> &DNod,
                           double scaleFactor, classOutputs *&outputs, double t0, double tf, string solverType,
                           const vector<int> &activeDofMapLocal, const vector<int> &nActiveDof,
                           const vector<int> &ISactiveDof, int flag_AV, const vector<double> &para_AV,
                           classPrintForces *&forceOutputs, bool flagActivation, string &petsc_solver,
                           string &petsc_precon, bool flagFSI, int precision)
        : solvers(nod, ndim, numDof, DNod, scaleFactor, outputs, t0, tf, solverType, activeDofMapLocal, nActiveDof,
                  ISactiveDof, forceOutputs, flagActivation, petsc_solver, petsc_precon, flagFSI),
          _precision(precision), _flagAV(flag_AV), _c1(para_AV.size() > 0 ? para_AV[0] : 0.0),
          _cl(para_AV.size() > 1 ? para_AV[1] : 0.0)
    {
    }

    void calculate(vector<classNeumannBCs *> &NeumannBCs, vector<classGPs *> &GPs, int sim, vector<classNodes *> &nod,
                   vector<classElements *> &elem, const vector<int> &nodFEM, const vector<int> &nodMM,
                   const vector<int> &nodShare, const vector<int> &elemFEM, const vector<int> &elemMM,
                   vector<classElements *> &geoShape, vector<constitutiveModels *> &consMod,
                   const vector<int> &nodLocal, int nNodGlobal, int nNodLocal) override
    {
        const int64_t nn = (int64_t)nod.size(), ne = (int64_t)elem.size();
        if (_ndim != 3 || (int64_t)_u.size() != 3 * nn || (int64_t)_v.size() != 3 * nn ||
            (int64_t)_a.size() != 3 * nn)
            stop("EXPLICIT GPU: 3D mechanics only (3 DOFs per node, no extra fields)");
        // mesh: X[c*Nn + node], conn[4e + a], one material id per element
        std::vector<double> X(3 * nn);
        for (int64_t i = 0; i < nn; i++)
            for (int c = 0; c < 3; c++) X[c * nn + i] = nod[i]->getXYZ()[c];
        std::vector<int32_t> conn(4 * ne), emat(ne);
        std::vector<msx_material> mats;
        std::map<const constitutiveModels *, int32_t> ids;
        std::vector<double> act(ne, 0.0);
        for (int64_t e = 0; e < ne; e++) {
            const vector<int> &n = elem[e]->getMyNodes();
            if (n.size() != 4 || elem[e]->getConsModel().empty()) stop("EXPLICIT GPU: C3D4 elements only");
            for (int a = 0; a < 4; a++) conn[4 * e + a] = n[a];
            const constitutiveModels *law = elem[e]->getConsModel()[0];
            auto it = ids.find(law);
            if (it == ids.end()) {
                msx_material m;
                if (!msx_binding::material_of(*law, m))
                    stop("EXPLICIT GPU: constitutive law not on the GPU path: " + law->getName());
                it = ids.emplace(law, (int32_t)mats.size()).first;
                mats.push_back(m);
            }
            emat[e] = it->second;
            // *INITINTVARS: the activation time is the GP's first internal variable
            // (hyperElasticStVenantKirchhoff.cpp:185-194, linearElastic alike)
            const vector<int> &gp = elem[e]->getMyGPs();
            if (_flagActivation && !gp.empty()) {
                const vector<double> &iv = GPs[gp[0]]->getCurrentState().getInternalVariables();
                if (!iv.empty()) act[e] = iv[0];
            }
        }
        std::vector<msx_bc> bcs;
        bcs.reserve(_DNod.size());
        for (const classDirichlet *d : _DNod) bcs.push_back(msx_binding::bc_of(*d));

        const msx_mesh mesh{nn, ne, X.data(), conn.data(), emat.data()};
        const msx_solver_opts o{_t0, _tf, _scaleFactor, 0, _precision, 0};
        msx_handle *h = nullptr;
        check(msx_create(&mesh, mats.data(), (int32_t)mats.size(), bcs.data(), (int64_t)bcs.size(), &o, &h), h);
        check(msx_set_state(h, _u.data(), _v.data(), _a.data()), h);
        if (!NeumannBCs.empty()) {
            msx_deck_loads *loads = nullptr;
            const msx_load_block *blocks = nullptr;
            int64_t nblocks = 0;
            const std::string why =
                msx_binding::loads_of(GeneralOptions::getInputFilePath(), NeumannBCs, nn, loads, blocks, nblocks);
            if (!why.empty()) {
                msx_deck_loads_free(loads);
                msx_destroy(h);
                stop("EXPLICIT GPU: " + why);
            }
            const msx_status st = msx_set_load_blocks(h, blocks, nblocks);
            msx_deck_loads_free(loads);
            check(st, h);
        }
        if (_flagActivation) check(msx_set_activation(h, act.data(), 1), h);
        // artificial viscosity with the element size and c0 the reference computes with: it
        // never assigns solvers::_elementSize and _c0 (0 in its builds), so pass 0
        if (_flagAV == 1 || _flagAV == 2)
            check(msx_set_viscosity(h, _flagAV == 1 ? MSX_VISC_BULK : MSX_VISC_DEV, _c1, _cl, 0.0, 0.0), h);
        msx_run_report r{};
        check(msx_run(h, 0, &r), h);
        check(msx_get_state(h, _u.data(), _v.data(), _a.data()), h);   // read back by getFinalValues()
        msx_destroy(h);
        INFO("EXPLICIT GPU: %lld steps, t = %g, dt = %g", (long long)r.total_steps, r.t, r.dt);
    }

  private:
    int _precision;
    int _flagAV;
    double _c1, _cl;

    static void stop(const std::string &msg)
    {
        ERROR("%s", msg.c_str());
        exit(-1);
    }
    static void check(msx_status st, msx_handle *h)
    {
        if (st == MSX_OK) return;
        ERROR("EXPLICIT GPU: %s (status %d)", msx_last_error(), (int)st);
        if (h) msx_destroy(h);
        exit(-1);
    }
};
