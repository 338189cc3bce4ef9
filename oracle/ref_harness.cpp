/*
 * ref_harness.cpp -- driver for the reference MuPhiSim build used as the
 * oracle's pin.  TEST INFRASTRUCTURE.
 *
 * It walks the same sequence as the reference's src/main.cpp:37-217
 * (options, input deck, Gauss points, internal variables, solver chain with
 * getFinalValues/initValues hand-off) by calling the reference's own
 * functions, then writes the final u, v, a of the last solver as raw
 * little-endian float64 to the file given by `-dump <path>` (the reference's
 * VTK output has 6 significant digits only), plus the solve wall time in
 * seconds as a fourth record when `-timing <path>` is given.
 */
#include "configuration.h"
#include "commandLine.h"
#include "init.h"
#include "solvers.h"
#include "constitutiveModels.h"
#include "classGPs.h"
#include "classNeumannBCs.h"
#include "dataExtraction.h"
#include "boundaryConditions.h"
#include <chrono>
#include <cstdio>

int main(int argc, char **argv)
{
    const char *dump = nullptr, *timing = nullptr;
    for (int i = 1; i + 1 < argc; i++) {
        if (strcmp(argv[i], "-dump") == 0) dump = argv[i + 1];
        if (strcmp(argv[i], "-timing") == 0) timing = argv[i + 1];
    }
    GeneralOptions::initialise(argc, argv);
    vector<classNodes *> nod;
    vector<classElements *> elem, geoShape;
    vector<classGPs *> GPs;
    vector<classNeumannBCs *> NeumannBCs;
    vector<int> nodFEM, nodMM, nodShare, elemFEM, elemMM, npartShare, nodLocal, elemLocal, npart, epart;
    vector<constitutiveModels *> consMod;
    vector<solvers *> solver;
    vector<double> iniValueExtraDof;
    int ndim = 0;
    inputManagement(nod, elem, NeumannBCs, ndim, nodFEM, nodMM, nodShare, elemFEM, elemMM, geoShape, consMod,
                    epart, npartShare, nodLocal, elemLocal, npart, solver, iniValueExtraDof);
    int nNodGlobal = nod.size();
    int sim = nodMM.empty() ? 2 : (nodFEM.empty() ? 1 : 3);
    if (sim != 2) { fprintf(stderr, "harness: only FEM decks are supported\n"); return 2; }
    initGPsDefinition(GPs, nod, elem, ndim, sim, nodFEM, nodMM, nodShare, elemFEM, elemMM, consMod);
    int nmulti = 0;
    for (size_t i = 1; i < consMod.size(); i++) nmulti += consMod[i]->getNbrDofConsMod();
    int nNod = nod.size();
    int nDof = nNod * consMod[0]->getNbrDofConsMod();
    initInternalVariables(GPs, elem);
    vector<double> u(nDof, 0), v(nDof, 0), a(nDof, 0), vv(nNod * nmulti, 0), extF(nDof, 0);
    solver[0]->initValues(u, v, a, vv, extF);
    auto t0 = std::chrono::steady_clock::now();
    for (size_t i = 0; i < solver.size(); i++) {
        solver[i]->calculate(NeumannBCs, GPs, sim, nod, elem, nodFEM, nodMM, nodShare, elemFEM, elemMM, geoShape,
                             consMod, nodLocal, nNodGlobal, nNod);
        solver[i]->getFinalValues(u, v, a, vv, extF);
        if (i + 1 < solver.size()) solver[i + 1]->initValues(u, v, a, vv, extF);
    }
    double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (dump) {
        FILE *f = fopen(dump, "wb");
        if (!f) return 3;
        fwrite(u.data(), sizeof(double), u.size(), f);
        fwrite(v.data(), sizeof(double), v.size(), f);
        fwrite(a.data(), sizeof(double), a.size(), f);
        fclose(f);
    }
    if (timing) {
        FILE *f = fopen(timing, "w");
        if (f) { fprintf(f, "%.9f\n", wall); fclose(f); }
    }
    return 0;
}
