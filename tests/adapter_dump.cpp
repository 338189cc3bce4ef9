/*
 * adapter_dump.cpp -- TEST INFRASTRUCTURE.  Reads a deck with the reference's
 * own readers (the sequence of src/main.cpp:37-160, as oracle/ref_harness.cpp)
 * and prints, instead of running the solvers, what the GPU solver plugin
 * (v.1.1_gb300/integration/solverExplicitGPU.h) would hand to msx_create for
 * it: coordinates, connectivity, each element's msx_material, its activation
 * time, each solver block's msx_bc entries, and the Neumann blocks the plugin
 * reads from the deck file and checks against the reference's load objects.
 * Numbers as %.17g.  With -drop-last-load the last of the reference's load
 * objects is left out before that check (which must then refuse the deck).
 */
#include "solverExplicitGPU.h"
#include "commandLine.h"
#include "init.h"
#include "dataExtraction.h"
#include "boundaryConditions.h"
#include <cstdio>

int main(int argc, char **argv)
{
    bool drop_last_load = false;
    std::vector<char *> args;
    for (int k = 0; k < argc; k++) {
        if (std::string(argv[k]) == "-drop-last-load") drop_last_load = true;
        else args.push_back(argv[k]);
    }
    argc = (int)args.size();
    argv = args.data();
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
    int sim = nodMM.empty() ? 2 : (nodFEM.empty() ? 1 : 3);
    if (sim != 2) return 2;
    initGPsDefinition(GPs, nod, elem, ndim, sim, nodFEM, nodMM, nodShare, elemFEM, elemMM, consMod);
    initInternalVariables(GPs, elem);
    const long long nn = nod.size(), ne = elem.size();
    printf("N %lld %lld %zu\n", nn, ne, solver.size());
    for (long long i = 0; i < nn; i++) {
        const vector<double> &x = nod[i]->getXYZ();
        printf("X %lld %.17g %.17g %.17g\n", i, x[0], x[1], x[2]);
    }
    for (long long e = 0; e < ne; e++) {
        const vector<int> &n = elem[e]->getMyNodes();
        printf("C %lld %d %d %d %d\n", e, n[0], n[1], n[2], n[3]);
        msx_material m;
        if (!msx_binding::material_of(*elem[e]->getConsModel()[0], m)) return 3;
        printf("M %lld %d %.17g %.17g %.17g\n", e, m.law, m.young, m.nu, m.rho);
        const vector<int> &gp = elem[e]->getMyGPs();
        const vector<double> &iv = GPs[gp[0]]->getCurrentState().getInternalVariables();
        printf("A %lld %.17g\n", e, iv.empty() ? 0.0 : iv[0]);
    }
    for (size_t k = 0; k < solver.size(); k++) {
        vector<classDirichlet *> &d = solver[k]->getDirBCs();
        printf("S %zu %.17g %.17g %.17g %zu\n", k, solver[k]->getT0(), solver[k]->getTf(), solver[k]->getSf(),
               d.size());
        for (const classDirichlet *b : d) {
            const msx_bc c = msx_binding::bc_of(*b);
            printf("B %zu %lld %d %.17g\n", k, (long long)c.dof, c.mode, c.value);
        }
    }
    if (!NeumannBCs.empty()) {
        if (drop_last_load) NeumannBCs.pop_back();
        msx_deck_loads *keep = nullptr;
        const msx_load_block *blocks = nullptr;
        int64_t nb = 0;
        const std::string why =
            msx_binding::loads_of(GeneralOptions::getInputFilePath(), NeumannBCs, nn, keep, blocks, nb);
        if (!why.empty()) {
            printf("LX %s\n", why.c_str());
            msx_deck_loads_free(keep);
            return 4;
        }
        for (int64_t k = 0; k < nb; k++) {
            const msx_load_block &b = blocks[k];
            printf("L %lld %d %d %.17g %.17g %.17g %.17g %.17g %lld %lld\n", (long long)k, b.kind, b.face, b.t0,
                   b.tf, b.value[0], b.value[1], b.value[2], (long long)b.num_elems, (long long)b.num_forces);
            for (int64_t e = 0; e < b.num_elems; e++) printf("LE %lld %d\n", (long long)k, b.elems[e]);
            for (int64_t f = 0; f < b.num_forces; f++)
                printf("LF %lld %lld %.17g %.17g %.17g\n", (long long)k, (long long)b.forces[f].dof, b.forces[f].t0,
                       b.forces[f].tf, b.forces[f].value);
        }
        msx_deck_loads_free(keep);
    }
    return 0;
}
