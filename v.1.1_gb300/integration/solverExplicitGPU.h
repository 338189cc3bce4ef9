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
// Dirichlet BCs and element birth (*ACTIVATION).  Neumann loads need getters
// the reference's load classes do not have (their t0, tf and amounts are
// private): with loads present the block stops with an error naming them.
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

}  // namespace msx_binding

class classSolverExplicitGPU : public solvers {
  public:
    classSolverExplicitGPU(vector<classNodes *> &nod, int ndim, int numDof, vector<classDirichlet *> &DNod,
                           double scaleFactor, classOutputs *&outputs, double t0, double tf, string solverType,
                           const vector<int> &activeDofMapLocal, const vector<int> &nActiveDof,
                           const vector<int> &ISactiveDof, classPrintForces *&forceOutputs, bool flagActivation,
                           string &petsc_solver, string &petsc_precon, bool flagFSI, int precision)
        : solvers(nod, ndim, numDof, DNod, scaleFactor, outputs, t0, tf, solverType, activeDofMapLocal, nActiveDof,
                  ISactiveDof, forceOutputs, flagActivation, petsc_solver, petsc_precon, flagFSI),
          _precision(precision)
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
        if (!NeumannBCs.empty())
            stop("EXPLICIT GPU: Neumann loads need getters for their t0, tf and amounts "
                 "(classNodalForces, classGravity, classTractionInst/Ramp, classPressureInst/Ramp)");
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
        if (_flagActivation) check(msx_set_activation(h, act.data(), 1), h);
        msx_run_report r{};
        check(msx_run(h, 0, &r), h);
        check(msx_get_state(h, _u.data(), _v.data(), _a.data()), h);   // read back by getFinalValues()
        msx_destroy(h);
        INFO("EXPLICIT GPU: %lld steps, t = %g, dt = %g", (long long)r.total_steps, r.t, r.dt);
    }

  private:
    int _precision;

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
