// msx_deck.cpp -- input-deck front end: runs an explicit C3D4 deck through
// the C ABI, as `MuPhiSim -input <deck>` runs it through the reference's
// solver chain (src/main.cpp:37-217).
//
//   msx_deck -input deck.inp [-inputDir d] [-outputDir o] [-precision fp64|exact|mixed|dword]
//            [-dump final.bin] [-csv final.csv] [-parse-only]
//
// -inputDir defaults to "input" and the extraction and *Forces files go to
// -outputDir, by default "output", as in the reference (IO/commandLine.cpp).
// With -outputDir given, VTK files MuPhiSimOutputs_0_.<k>.vtk and the series index
// allOutputs_0.vtk.series are written at the reference's *Outputs cadence
// (solverExplicit.cpp:171-174, 310-321): at t0 when t0 < 1e-12, then every
// long(long((tf - t0)/dt0)/outputs) steps and when the block ends at tf; the
// element fields (Cauchy, Green-Lagrange, von Mises) are computed on the
// device only at those steps.  Values are written at full precision.
//
// Keyword subset (src/IO/inputFile.cpp): *Node (:20-108), *Element, type=C3D4
// (:118-323), *FEM Nodes / *FEM Elements, *MATERIAL with *Density,
// *HyperElastic {Neo-Hookean | 3D-Compressible-Neo-Hookean |
// St-Venant-Kirchhoff}, *Linear-Elastic, *INITINTVARS and *List of Elements
// (:838-1029, 2010-2111), *SOLVER, EXPLICIT ... *END SOLVER with *ACTIVATION,
// *Scale Factor, *Outputs, *Time, *Forces and *BOUNDARY, TYPE=DISPLACEMENT
// RAMP|INST and *Bulk viscosity / *Dev viscosity (:2253-2831, 2960-3218,
// 4830-4886), the Neumann blocks *BOUNDARY,
// TYPE=FORCE | TRACTION INST|RAMP | PRESSURE INST|RAMP and *GRAVITY
// (:4705-4760, 2841-2945), and *EXTRACTION, NODE | ELEMENT (:4950-5111).
// Other keywords belong to paths this library does not implement and are
// refused.
// As in the reference, a RAMP BC stores U/(tf - t0) with the *Time read so
// far, and once an INST block has been read every later displacement block
// is instantaneous (the flag is not reset between solvers).
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/msx.h"

namespace {

struct SolverBlock {
    double sf = 1, t0 = 0, tf = 0;
    int outputs = -1;
    std::vector<msx_bc> bcs;
    // *Forces (IO/inputFile.cpp:2537-2541, 4830-4886): output frequency and
    // the (node, direction) pairs whose internal force is written
    double force_freq = 0;
    std::vector<std::pair<int32_t, int>> force_out;
    bool activation = false;          // *ACTIVATION (element birth)
    // *Bulk viscosity / *Dev viscosity (IO/inputFile.cpp:2462-2511): kind and "c1, cl";
    // once read, later blocks keep it (the reader never resets its flag)
    int visc = MSX_VISC_NONE;
    double visc_c1 = 0, visc_cl = 0;
};

struct Deck {
    std::vector<double> xyz;          // node-major while reading
    bool has_loads = false;           // Neumann blocks present (read by msx_deck_read_loads)
    // *EXTRACTION, NODE blocks (IO/inputFile.cpp:4950-5026): "name, type, operation, comp";
    // *EXTRACTION, ELEMENT blocks (:5028-5111): "name,type,operation", then All or elements
    struct Extraction {
        std::string name;             // the output file's stem: <name>_<Type><comp>_<Operation> (node),
                                      // <name>_<TYPE>_<Operation> or All_<TYPE>_<Operation> (element)
        bool element = false;
        int field = 0, comp = 0;      // node: msx_node_field
        int quantity = 0;             // element: msx_element_quantity
        std::string op;               // Mean, Min, Max, Sum, Rough
        bool all = false;             // element: every element
        std::vector<int32_t> nodes;   // node: the nodes; element: the listed elements (0-based)
        double last_time = 0;
        FILE *file = nullptr;
    };
    std::vector<Extraction> extractions;
    std::vector<int32_t> conn;
    std::vector<msx_material> mats;
    std::vector<double> act_time;     // *INITINTVARS position 1 per element (0 without), if any
    std::vector<int32_t> elem_mat;    // -1 until assigned
    std::vector<SolverBlock> solvers;
};

std::string trim(const std::string &s)
{
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

bool starts(const std::string &s, const char *p) { return s.compare(0, strlen(p), p) == 0; }

std::vector<std::string> split(const std::string &s)
{
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ',')) out.push_back(trim(item));
    return out;
}

[[noreturn]] void die(const std::string &msg, int line)
{
    fprintf(stderr, "msx_deck: %s (line %d)\n", msg.c_str(), line);
    exit(2);
}

// The reference keeps the first extraction of a file name and drops later
// ones (classExtractData::addClassNodeDataToSave / addClassElementDataToSave,
// solvers/dataExtraction.cpp:469-488).
void add_extraction(Deck &d, const Deck::Extraction &E)
{
    for (const auto &x : d.extractions)
        if (x.name == E.name) return;
    d.extractions.push_back(E);
}

Deck parse(const std::string &path)
{
    std::ifstream in(path);
    if (!in) die("cannot open " + path, 0);
    std::vector<std::string> lines;
    for (std::string l; std::getline(in, l);) lines.push_back(trim(l));
    Deck d;
    bool instantaneous = false;
    int visc = MSX_VISC_NONE;         // the artificial viscosity read so far (kept across blocks)
    double visc_c1 = 0, visc_cl = 0;
    const size_t n = lines.size();
    size_t i = 0;
    auto data_line = [&](size_t k) { return k < n && !lines[k].empty() && lines[k][0] != '*'; };
    while (i < n) {
        const std::string &L = lines[i];
        int ln = (int)i + 1;
        if (L.empty() || starts(L, "**")) {
            i++;
        } else if (starts(L, "*Node")) {
            for (i++; data_line(i); i++) {
                auto f = split(lines[i]);
                if (f.size() != 4) die("a 3D node line has id, x, y, z", (int)i + 1);
                if (atoi(f[0].c_str()) != (int)d.xyz.size() / 3 + 1) die("node ids must be 1..N in order", (int)i + 1);
                for (int c = 1; c < 4; c++) d.xyz.push_back(atof(f[c].c_str()));
            }
        } else if (starts(L, "*Element")) {
            if (L.find("C3D4") == std::string::npos) die("only *Element, type=C3D4 is supported", ln);
            for (i++; data_line(i); i++) {
                auto f = split(lines[i]);
                if (f.size() != 5) die("a C3D4 line has id and 4 nodes", (int)i + 1);
                for (int c = 1; c < 5; c++) d.conn.push_back(atoi(f[c].c_str()) - 1);
            }
        } else if (starts(L, "*BOUNDARY, TYPE=FORCE") || starts(L, "*BOUNDARY, TYPE=TRACTION RAMP") ||
                   starts(L, "*BOUNDARY, TYPE=TRACTION INST") || starts(L, "*BOUNDARY, TYPE=PRESSURE RAMP") ||
                   starts(L, "*BOUNDARY, TYPE=PRESSURE INST")) {
            // Neumann blocks: read by the library (msx_deck_read_loads); skipped here
            for (i += 2; data_line(i); i++) {
            }
            d.has_loads = true;
        } else if (starts(L, "*GRAVITY")) {
            i += 2;
            d.has_loads = true;
        } else if (starts(L, "*EXTRACTION, NODE")) {
            // data extraction of nodal values written every step (solvers/dataExtraction.cpp)
            auto h = split(lines[i + 1]);
            if (h.size() != 4) die("a node extraction starts with name, type, operation, comp", (int)i + 2);
            Deck::Extraction E;
            static const char *types[] = {"Unknown", "ExternalForce", "InternalForce"};
            E.field = -1;
            for (int t = 0; t < 3; t++)
                if (h[1] == types[t]) E.field = t;
            if (E.field < 0) die("node datatype " + h[1] + " has not defined", (int)i + 2);
            E.op = h[2];
            if (E.op != "Mean" && E.op != "Min" && E.op != "Max" && E.op != "Sum" && E.op != "Rough")
                die("operation " + E.op + " has not defined", (int)i + 2);
            E.comp = (int)atof(h[3].c_str());
            if (E.comp < 0 || E.comp > 2) die("node extraction component must be 0..2", (int)i + 2);
            E.name = h[0] + "_" + types[E.field] + std::to_string(E.comp) + "_" + E.op;
            for (i += 2; data_line(i); i++) {
                long long node = atoll(lines[i].c_str()) - 1;
                if (node < 0 || node >= (long long)d.xyz.size() / 3) die("extraction node out of range", (int)i + 1);
                E.nodes.push_back((int32_t)node);
            }
            if (!E.nodes.empty()) add_extraction(d, E);
        } else if (starts(L, "*EXTRACTION, ELEMENT")) {
            // element data written every step (solvers/dataExtraction.cpp:304-470, 841-889)
            auto h = split(lines[i + 1]);
            if (h.size() != 3) die("an element extraction starts with name, type, operation", (int)i + 2);
            Deck::Extraction E;
            E.element = true;
            static const char *qn[] = {"FXX", "FXY", "FXZ", "FYX", "FYY", "FYZ", "FZX", "FZY", "FZZ",
                                       "PXX", "PXY", "PXZ", "PYX", "PYY", "PYZ", "PZX", "PZY", "PZZ",
                                       "SVM", "KVM", "INVAR1", "INVAR2", "INVAR3", "INVAR4", "INVAR5", "INVAR6",
                                       "DEFO_ENERGY", "EXTERNAL_ENERGY", "KIN_ENERGY", "VOLUME"};
            for (int q = 0; q < 30; q++)
                if (h[1] == qn[q]) E.quantity = MSX_ELEM_FXX + q;
            if (E.quantity == 0) die("element datatype " + h[1] + " has not defined", (int)i + 2);
            E.op = h[2];
            if (E.op == "Rough") die("Rough data is not implemented for element extraction", (int)i + 2);
            if (E.op != "Mean" && E.op != "Min" && E.op != "Max" && E.op != "Sum")
                die("operation " + E.op + " has not defined", (int)i + 2);
            if (E.quantity == MSX_ELEM_VOLUME && E.op == "Mean")
                die("VOLUME has no Mean (the reference's volume() returns no value for it)", (int)i + 2);
            bool all = false;
            for (i += 2; data_line(i); i++) {
                if (starts(lines[i], "All")) {
                    all = true;
                    continue;
                }
                long long e = atoll(lines[i].c_str()) - 1;
                if (e < 0 || e >= (long long)d.conn.size() / 4) die("extraction element out of range", (int)i + 1);
                E.nodes.push_back((int32_t)e);
            }
            // "All" and a list make two extractions, the All one first (:5100-5111)
            if (all) {
                Deck::Extraction A = E;
                A.all = true;
                A.nodes.clear();
                A.name = std::string("All_") + h[1] + "_" + E.op;
                add_extraction(d, A);
            }
            E.name = h[0] + "_" + h[1] + "_" + E.op;
            if (!E.nodes.empty()) add_extraction(d, E);
        } else if (starts(L, "*FEM Nodes") || starts(L, "*FEM Elements")) {
            if (i + 1 >= n || !starts(lines[i + 1], "All")) die("only 'All' FEM sets are supported", ln);
            i += 2;
        } else if (starts(L, "*MATERIAL")) {
            msx_material m{};
            m.law = -1;
            bool have_rho = false;
            int id = (int)d.mats.size();
            // the reference reads extraction blocks wherever they stand in the file
            for (i++; i < n && !starts(lines[i], "*MATERIAL") && !starts(lines[i], "*END") && !starts(lines[i], "*SOLVER") &&
                      !starts(lines[i], "*EXTRACTION");) {
                const std::string &K = lines[i];
                if (starts(K, "*Density")) {
                    m.rho = atof(lines[i + 1].c_str());
                    have_rho = true;
                    i += 2;
                } else if (starts(K, "*HyperElastic")) {
                    std::string law = trim(K.substr(K.find(',') + 1));
                    if (law == "Neo-Hookean") m.law = MSX_LAW_NEO_HOOKEAN;
                    else if (law == "3D-Compressible-Neo-Hookean") m.law = MSX_LAW_COMPRESSIBLE_NEO_HOOKEAN;
                    else if (law == "St-Venant-Kirchhoff") m.law = MSX_LAW_STVK;
                    else die("unsupported law " + law, (int)i + 1);
                    auto f = split(lines[i + 1]);
                    if (f.size() < 2) die("*HyperElastic needs E, nu", (int)i + 2);
                    m.young = atof(f[0].c_str());
                    m.nu = atof(f[1].c_str());
                    i += 2;
                } else if (starts(K, "*Linear-Elastic")) {
                    // IO/inputFile.cpp:886-925: "E, nu[, PlaneStress|PlaneStrain]"; the
                    // stress state only matters in 2D
                    auto f = split(lines[i + 1]);
                    if (f.size() < 2) die("*Linear-Elastic needs E, nu", (int)i + 2);
                    m.law = MSX_LAW_LINEAR_ELASTIC;
                    m.young = atof(f[0].c_str());
                    m.nu = atof(f[1].c_str());
                    i += 2;
                } else if (starts(K, "*INITINTVARS")) {
                    // IO/inputFile.cpp:2055-2111 and init.cpp:54-80: "element, position, value";
                    // the St-Venant-Kirchhoff and linear-elastic laws have one internal
                    // variable, the activation time; the neo-Hookean laws have none
                    if (m.law != MSX_LAW_STVK && m.law != MSX_LAW_LINEAR_ELASTIC)
                        die("*INITINTVARS needs a St-Venant-Kirchhoff or linear-elastic law before it", (int)i + 1);
                    if (d.act_time.empty()) d.act_time.assign(d.conn.size() / 4, 0.0);
                    for (i++; i < n && !lines[i].empty() && lines[i][0] != '*'; i++) {
                        auto f = split(lines[i]);
                        if (f.size() < 3) die("an *INITINTVARS line has element, position, value", (int)i + 1);
                        long long e = atoll(f[0].c_str()) - 1, pos = atoll(f[1].c_str()) - 1;
                        if (e < 0 || e >= (long long)d.act_time.size()) die("*INITINTVARS element out of range", (int)i + 1);
                        if (pos != 0) die("Position of an internal variable not valid", (int)i + 1);
                        if (!d.elem_mat.empty() && d.elem_mat[e] != id) die("Element on INITINTVARS list not valid", (int)i + 1);
                        d.act_time[e] = atof(f[2].c_str());
                    }
                } else if (starts(K, "*List of Elements")) {
                    if (d.elem_mat.size() != d.conn.size() / 4) d.elem_mat.assign(d.conn.size() / 4, -1);
                    if (starts(lines[i + 1], "All")) {
                        for (auto &e : d.elem_mat) e = id;
                    } else {
                        // the reference reads one element id per keyword
                        int e = atoi(lines[i + 1].c_str()) - 1;
                        if (e < 0 || e >= (int)d.elem_mat.size()) die("element id out of range", (int)i + 2);
                        d.elem_mat[e] = id;
                    }
                    i += 2;
                } else if (K.empty()) {
                    i++;
                } else {
                    die("unsupported material keyword " + K, (int)i + 1);
                }
            }
            if (m.law < 0 || !have_rho) die("material needs *Density and *HyperElastic or *Linear-Elastic", ln);
            d.mats.push_back(m);
        } else if (starts(L, "*SOLVER")) {
            if (trim(L.substr(L.find(',') + 1)) != "EXPLICIT") die("only *SOLVER, EXPLICIT is supported", ln);
            SolverBlock s;
            bool have_time = false;
            for (i++; i < n && !starts(lines[i], "*END SOLVER"); ) {
                const std::string &K = lines[i];
                if (starts(K, "*Scale Factor")) {
                    s.sf = atof(lines[i + 1].c_str());
                    i += 2;
                } else if (starts(K, "*Outputs")) {
                    s.outputs = atoi(lines[i + 1].c_str());
                    i += 2;
                    if (data_line(i)) i++;   // optional variable list
                } else if (starts(K, "*Time")) {
                    auto f = split(lines[i + 1]);
                    if (f.size() != 2) die("*Time needs t0, tf", (int)i + 2);
                    s.t0 = atof(f[0].c_str());
                    s.tf = atof(f[1].c_str());
                    have_time = true;
                    i += 2;
                } else if (starts(K, "*BOUNDARY, TYPE=DISPLACEMENT")) {
                    // the reference divides a ramp by the *Time read before it
                    if (!have_time) die("put *Time before *BOUNDARY in a solver block", (int)i + 1);
                    if (K.find("INST") != std::string::npos) instantaneous = true;
                    else if (K.find("RAMP") == std::string::npos) die("unknown displacement BC type", (int)i + 1);
                    for (i++; data_line(i); i++) {
                        auto f = split(lines[i]);
                        if (f.size() != 3) die("a BC line has node, direction, value", (int)i + 1);
                        msx_bc b{};
                        long long node = atoll(f[0].c_str()) - 1, dir = atoll(f[1].c_str());
                        long long nn = (long long)d.xyz.size() / 3;
                        if (node < 0 || node >= nn || dir < 0 || dir > 2) die("BC node/direction out of range", (int)i + 1);
                        b.dof = node + dir * nn;
                        b.mode = instantaneous ? MSX_BC_INST : MSX_BC_RAMP;
                        // a ramp is U/(tf - t0) with the *Time read so far: pass U and
                        // make the library divide by this block's own duration
                        b.value = atof(f[2].c_str());
                        s.bcs.push_back(b);
                    }
                } else if (starts(K, "*ACTIVATION")) {
                    s.activation = true;   // IO/inputFile.cpp:2332-2334
                    i++;
                } else if (starts(K, "*Bulk viscosity") || starts(K, "*Dev viscosity")) {
                    // IO/inputFile.cpp:2462-2511: defaults (0.06, 1.2) and (1, 0.5); the next
                    // line is always consumed and read as "c1, cl": spaces are skipped, each
                    // comma sets c1 from the characters before it, the line's last character
                    // closes cl, and a '*' ends the scan (no parameters)
                    const bool bulk = starts(K, "*Bulk");
                    visc = bulk ? MSX_VISC_BULK : MSX_VISC_DEV;
                    visc_c1 = bulk ? 0.06 : 1.0;
                    visc_cl = bulk ? 1.2 : 0.5;
                    if (i + 1 < n) {
                        const std::string &T = lines[i + 1];
                        std::string tok;
                        for (size_t c = 0; c < T.size(); c++) {
                            if (T[c] == '*') break;
                            if (T[c] == ' ') continue;
                            if (T[c] == ',') {
                                visc_c1 = atof(tok.c_str());
                                tok.clear();
                            } else {
                                tok += T[c];
                                if (c == T.size() - 1) visc_cl = atof(tok.c_str());
                            }
                        }
                    }
                    i += 2;
                } else if (starts(K, "*Forces")) {
                    if (i + 1 >= n) die("*Forces needs a frequency", (int)i + 1);
                    s.force_freq = atof(lines[i + 1].c_str());
                    if (!(s.force_freq > 0)) die("*Forces frequency must be > 0", (int)i + 2);
                    for (i += 2; data_line(i); i++) {
                        auto f = split(lines[i]);
                        if (f.size() < 2) die("a *Forces line has node, direction", (int)i + 1);
                        long long node = atoll(f[0].c_str()) - 1, dir = atoll(f[1].c_str());
                        if (node < 0 || node >= (long long)d.xyz.size() / 3) die("*Forces node out of range", (int)i + 1);
                        // directions are 0..2 (output.cpp:121-124 refuses dir >= ndim)
                        if (dir < 0 || dir > 2) die("*Forces direction must be 0, 1 or 2", (int)i + 1);
                        s.force_out.push_back({(int32_t)node, (int)dir});
                    }
                } else if (K.empty()) {
                    i++;
                } else {
                    die("unsupported solver keyword " + K, (int)i + 1);
                }
            }
            if (s.outputs < 0) die("*Outputs is required in an explicit solver block", ln);
            s.visc = visc;
            s.visc_c1 = visc_c1;
            s.visc_cl = visc_cl;
            d.solvers.push_back(s);
            i++;
        } else if (starts(L, "*END")) {
            break;
        } else {
            die("unsupported keyword " + L, ln);
        }
    }
    if (d.xyz.size() < 12 || d.conn.empty()) die("deck needs nodes and C3D4 elements", 0);
    if (d.mats.empty() || d.solvers.empty()) die("deck needs a material and a solver block", 0);
    if (!d.elem_mat.empty())
        for (int32_t m : d.elem_mat)
            if (m < 0) die("an element has no material", 0);
    return d;
}

// One output file in the reference's VTK layout (src/IO/output.cpp:296-700):
// undeformed points, C3D4 cells, nodal displacement / velocity /
// acceleration, element Cauchy, Green-Lagrange and von Mises.
bool write_vtk(const std::string &dir, int index, const std::vector<double> &X, const std::vector<int32_t> &conn,
               msx_handle *h)
{
    const long long nn = (long long)X.size() / 3, ne = (long long)conn.size() / 4;
    std::vector<double> u(3 * nn), v(3 * nn), a(3 * nn), cau(9 * ne), gl(9 * ne), vms(ne);
    if (msx_get_state(h, u.data(), v.data(), a.data()) != MSX_OK ||
        msx_element_fields(h, cau.data(), gl.data(), vms.data()) != MSX_OK)
        return false;
    std::string name = "MuPhiSimOutputs_0_." + std::to_string(index) + ".vtk";
    FILE *f = fopen((dir + "/" + name).c_str(), "w");
    if (!f) return false;
    fprintf(f, "# vtk DataFile Version 1.0\n3D Unstructured Grid of C3D4 elements\nASCII\n\n");
    fprintf(f, "DATASET UNSTRUCTURED_GRID\nPOINTS %lld float\n", nn);
    for (long long i = 0; i < nn; i++) fprintf(f, "%.17g %.17g %.17g\n", X[i], X[nn + i], X[2 * nn + i]);
    fprintf(f, "\nCELLS %lld %lld\n", ne, 5 * ne);
    for (long long e = 0; e < ne; e++)
        fprintf(f, "4 %d %d %d %d\n", conn[4 * e], conn[4 * e + 1], conn[4 * e + 2], conn[4 * e + 3]);
    fprintf(f, "\nCELL_TYPES %lld\n", ne);
    for (long long e = 0; e < ne; e++) fprintf(f, "10\n");
    fprintf(f, "\nPOINT_DATA %lld\n", nn);
    const char *names[3] = {"Displacement", "Velocity", "Acceleration"};
    const std::vector<double> *fields[3] = {&u, &v, &a};
    for (int k = 0; k < 3; k++) {
        fprintf(f, "VECTORS %s float\n", names[k]);
        const std::vector<double> &w = *fields[k];
        for (long long i = 0; i < nn; i++) fprintf(f, "%.17g %.17g %.17g\n", w[i], w[nn + i], w[2 * nn + i]);
        fprintf(f, "\n");
    }
    fprintf(f, "CELL_DATA %lld\n", ne);
    const char *tnames[2] = {"Cauchy", "E"};
    const std::vector<double> *tens[2] = {&cau, &gl};
    for (int k = 0; k < 2; k++) {
        fprintf(f, "TENSORS %s float\n", tnames[k]);
        const std::vector<double> &w = *tens[k];
        for (long long e = 0; e < ne; e++)
            for (int r = 0; r < 3; r++)
                fprintf(f, "%.17g %.17g %.17g\n", w[9 * e + 3 * r], w[9 * e + 3 * r + 1], w[9 * e + 3 * r + 2]);
        fprintf(f, "\n");
    }
    fprintf(f, "SCALARS VMS float\nLOOKUP_TABLE default\n");
    for (long long e = 0; e < ne; e++) fprintf(f, "%.17g\n", vms[e]);
    fclose(f);
    return true;
}

// allOutputs_0.vtk.series (ParaView file-series JSON), rewritten after each output
void write_series(const std::string &dir, const std::vector<std::pair<std::string, double>> &files)
{
    FILE *f = fopen((dir + "/allOutputs_0.vtk.series").c_str(), "w");
    if (!f) return;
    fprintf(f, "{\n\"file-series-version\" : \"1.0\",\n\"files\" : [\n");
    for (size_t k = 0; k < files.size(); k++)
        fprintf(f, "{ \"name\" : \"%s\", \"time\" :%.17g}%s\n", files[k].first.c_str(), files[k].second,
                k + 1 < files.size() ? "," : "");
    fprintf(f, "]\n}\n");
    fclose(f);
}

}  // namespace

// One row of an extraction (solvers/dataExtraction.cpp:190-300 node data,
// :386-400 element data): written only when the time has advanced; the file
// <dir>/<name>.csv is opened at the first row with the reference's header; the
// time and either every value (Rough) or the operation over them (node data:
// Mean, Sum sum from 0 in node order, Max, Min the first extreme; element data:
// msx_element_reduce), at %.16g.
static bool write_extraction(Deck::Extraction &E, const std::string &dir, msx_handle *h, double t)
{
    if (!(t > E.last_time)) return true;
    E.last_time = t;
    if (E.element) {
        const int op = E.op == "Mean" ? MSX_OP_MEAN : E.op == "Min" ? MSX_OP_MIN : E.op == "Max" ? MSX_OP_MAX : MSX_OP_SUM;
        double val = 0;
        if (msx_element_reduce(h, E.quantity, op, E.all ? nullptr : E.nodes.data(), (int64_t)E.nodes.size(), &val) !=
            MSX_OK)
            return false;
        if (!E.file) {
            E.file = fopen((dir + "/" + E.name + ".csv").c_str(), "w");
            if (!E.file) return false;
            fprintf(E.file, "Time,Value\n");
        }
        fprintf(E.file, "%.16g,%.16g\n", t, val);
        fflush(E.file);
        return true;
    }
    std::vector<double> v(E.nodes.size());
    if (msx_node_values(h, E.field, E.comp, E.nodes.data(), (int64_t)v.size(), v.data()) != MSX_OK) return false;
    if (!E.file) {
        E.file = fopen((dir + "/" + E.name + ".csv").c_str(), "w");
        if (!E.file) return false;
        if (E.op == "Rough") {
            fprintf(E.file, "Time");
            for (int32_t nd : E.nodes) fprintf(E.file, ",Node%dComp%d", nd + 1, E.comp);
            fprintf(E.file, "\n");
        } else {
            fprintf(E.file, "Time,Value\n");
        }
    }
    if (E.op == "Rough") {
        fprintf(E.file, "%.16g", t);
        for (double x : v) fprintf(E.file, ",%.16g", x);
        fprintf(E.file, "\n");
    } else {
        double val = 0;
        if (E.op == "Mean" || E.op == "Sum") {
            for (double x : v) val += x;
            if (E.op == "Mean") val /= (double)v.size();
        } else if (E.op == "Max") {
            val = *std::max_element(v.begin(), v.end());
        } else {
            val = *std::min_element(v.begin(), v.end());
        }
        fprintf(E.file, "%.16g,%.16g\n", t, val);
    }
    fflush(E.file);
    return true;
}

// *Forces output of one solver block (IO/output.cpp:107-133 writeExternalForces,
// :153-279 printForcesOut, called every step at solverExplicit.cpp:304): when
// t >= k * max(1/frequency, dt) + t0 (k = rows written so far), one line per
// listed (node, direction) with the internal force of the step (the inertia
// term the reference adds is zero: computeInertialForce is not called,
// solverExplicit.cpp:611), in <dir>/externalForces<t0>-<tf>.csv, numbers
// formatted as std::to_string does.
struct ForcePrinter {
    const SolverBlock &s;
    std::string path;
    long long done = 0;
    ForcePrinter(const SolverBlock &b, const std::string &dir)
        : s(b), path(dir + "/externalForces" + std::to_string(b.t0) + "-" + std::to_string(b.tf) + ".csv") {}
    bool step(msx_handle *h, double t, double dt)
    {
        double period = 1.0 / s.force_freq;
        if (period < dt) period = dt;
        if (!(t >= done * period + s.t0)) return true;
        FILE *f = fopen(path.c_str(), done == 0 ? "w" : "a");
        if (!f) return false;
        if (done == 0) fprintf(f, "Node,Direction,Force,Time,\n");
        for (const auto &nd : s.force_out) {
            double v = 0;
            if (msx_node_values(h, MSX_FIELD_INTERNAL_FORCE, nd.second, &nd.first, 1, &v) != MSX_OK) {
                fclose(f);
                return false;
            }
            fprintf(f, "%s,%s,%s,%s,\n", std::to_string(nd.first + 1).c_str(), std::to_string(nd.second).c_str(),
                    std::to_string(v).c_str(), std::to_string(t).c_str());
        }
        fclose(f);
        done++;
        return true;
    }
};

int main(int argc, char **argv)
{
    std::string input, dir = "input", dump, csv, outdir;
    int precision = MSX_PREC_FP64;
    bool parse_only = false;
    for (int k = 1; k < argc; k++) {
        std::string a = argv[k];
        auto next = [&]() { return k + 1 < argc ? std::string(argv[++k]) : std::string(); };
        if (a == "-input") input = next();
        else if (a == "-inputDir") dir = next();
        else if (a == "-dump") dump = next();
        else if (a == "-outputDir") outdir = next();
        else if (a == "-csv") csv = next();
        else if (a == "-parse-only") parse_only = true;
        else if (a == "-precision") {
            std::string p = next();
            precision = p == "exact" ? MSX_PREC_FP64_EXACT
                        : p == "mixed" ? MSX_PREC_MIXED
                        : p == "dword" ? MSX_PREC_DOUBLE_WORD : MSX_PREC_FP64;
        }
    }
    if (input.empty()) {
        fprintf(stderr, "usage: msx_deck -input deck.inp [-inputDir d] [-outputDir o] "
                        "[-precision fp64|exact|mixed|dword] [-dump f.bin] [-csv f.csv] [-parse-only]\n");
        return 2;
    }
    Deck d = parse(dir + "/" + input);
    const long long nn = (long long)d.xyz.size() / 3, ne = (long long)d.conn.size() / 4;
    // the Neumann blocks, as the library reads them for any caller
    msx_deck_loads *loads = nullptr;
    const msx_load_block *blocks = nullptr;
    int64_t nblocks = 0;
    if (d.has_loads && (msx_deck_read_loads((dir + "/" + input).c_str(), nn, &loads) != MSX_OK ||
                        msx_deck_loads_blocks(loads, &blocks, &nblocks) != MSX_OK)) {
        fprintf(stderr, "msx_deck: %s\n", msx_last_error());
        return 2;
    }
    std::vector<double> X(3 * nn);
    for (long long i = 0; i < nn; i++)
        for (int c = 0; c < 3; c++) X[c * nn + i] = d.xyz[3 * i + c];
    if (parse_only) {
        size_t nbc = 0;
        for (auto &s : d.solvers) nbc += s.bcs.size();
        printf("{\"nodes\": %lld, \"elements\": %lld, \"materials\": %zu, \"solvers\": %zu, \"bcs\": %zu",
               nn, ne, d.mats.size(), d.solvers.size(), nbc);
        size_t nforces = 0;
        double gravity = 0;
        int gravity_first = 0;
        for (int64_t k = 0; k < nblocks; k++) {
            const msx_load_block &B = blocks[k];
            if (B.kind == MSX_LOAD_FORCE) nforces += (size_t)B.num_forces;
            if (B.kind == MSX_LOAD_GRAVITY) {
                if (nforces == 0 && gravity == 0) gravity_first = 1;
                gravity = B.value[0];
            }
        }
        printf(", \"forces\": %zu, \"gravity\": %.17g, \"gravity_first\": %d", nforces, gravity, gravity_first);
        static const char *names[] = {"FORCE", "GRAVITY", "TRACTION INST", "TRACTION RAMP", "PRESSURE INST",
                                      "PRESSURE RAMP"};
        printf(", \"extractions\": [");
        for (size_t k = 0; k < d.extractions.size(); k++) {
            const auto &E = d.extractions[k];
            if (E.element && E.all)
                printf("%s{\"name\": \"%s\", \"elements\": \"All\"}", k ? ", " : "", E.name.c_str());
            else
                printf("%s{\"name\": \"%s\", \"%s\": %zu}", k ? ", " : "", E.name.c_str(),
                       E.element ? "elements" : "nodes", E.nodes.size());
        }
        printf("]");
        printf(", \"loads\": [");
        for (int64_t k = 0; k < nblocks; k++)
            printf("%s{\"kind\": \"%s\", \"face\": %d, \"elements\": %lld, \"entries\": %lld}", k ? ", " : "",
                   names[blocks[k].kind], blocks[k].face, (long long)blocks[k].num_elems,
                   (long long)blocks[k].num_forces);
        printf("]");
        printf(", \"blocks\": [");
        for (size_t k = 0; k < d.solvers.size(); k++)
            printf("%s{\"t0\": %.17g, \"tf\": %.17g, \"sf\": %.17g, \"bcs\": %zu, \"inst\": %d, "
                   "\"force_freq\": %.17g, \"force_out\": %zu, \"visc\": %d, \"visc_c1\": %.17g, "
                   "\"visc_cl\": %.17g}", k ? ", " : "",
                   d.solvers[k].t0, d.solvers[k].tf, d.solvers[k].sf, d.solvers[k].bcs.size(),
                   d.solvers[k].bcs.empty() ? 0 : d.solvers[k].bcs[0].mode == MSX_BC_INST, d.solvers[k].force_freq,
                   d.solvers[k].force_out.size(), d.solvers[k].visc, d.solvers[k].visc_c1, d.solvers[k].visc_cl);
        printf("]}\n");
        return 0;
    }
    msx_mesh mesh{nn, ne, X.data(), d.conn.data(), d.elem_mat.empty() ? nullptr : d.elem_mat.data()};
    // extraction files go to the output directory, by default ./output (IO/commandLine.cpp:20, 165-170)
    const std::string xdir = outdir.empty() ? "output" : outdir;
    bool any_forces = false;
    for (const auto &s : d.solvers) any_forces |= s.force_freq > 0;
    if (!d.extractions.empty() || any_forces) mkdir(xdir.c_str(), 0755);
    msx_handle *h = nullptr;
    long long total = 0;
    std::vector<std::pair<std::string, double>> outputs;
    for (size_t k = 0; k < d.solvers.size(); k++) {
        const SolverBlock &s = d.solvers[k];
        // with extraction or *Forces the block advances one step per call: two-step graphs
        const bool stepwise = !d.extractions.empty() || s.force_freq > 0;
        msx_solver_opts o{s.t0, s.tf, s.sf, 0, precision, stepwise ? 2 : 0};
        msx_status st;
        if (k == 0) {
            st = msx_create(&mesh, d.mats.data(), (int32_t)d.mats.size(), s.bcs.data(), (int64_t)s.bcs.size(), &o, &h);
            if (st == MSX_OK && nblocks > 0) st = msx_set_load_blocks(h, blocks, nblocks);
        } else {
            // src/main.cpp:171-179: time continuity between solvers
            if (s.t0 - d.solvers[k - 1].tf > 1E-12) {
                fprintf(stderr, "msx_deck: This is not continuity in time between solvers\n");
                return 1;
            }
            st = msx_next_solver(h, s.bcs.data(), (int64_t)s.bcs.size(), &o);
        }
        // artificial viscosity with the element size and c0 the reference runs with: 0
        // (solvers.h:53-54 are never assigned), which makes its force zero
        if (st == MSX_OK) st = msx_set_viscosity(h, s.visc, s.visc_c1, s.visc_cl, 0.0, 0.0);
        // element birth: the activation times once, the block's *ACTIVATION flag each block
        if (st == MSX_OK && !d.act_time.empty())
            st = msx_set_activation(h, k == 0 ? d.act_time.data() : nullptr, s.activation ? 1 : 0);
        if (st != MSX_OK) {
            fprintf(stderr, "msx_deck: %s\n", msx_last_error());
            return 1;
        }
        msx_run_report r{};
        ForcePrinter fp{s, xdir};
        if (outdir.empty() && !stepwise) {
            st = msx_run(h, 0, &r);
            total += r.steps;
            printf("solver %zu: %lld steps, t = %.9g, dt = %.6g, device %.3f ms\n", k, (long long)r.steps, r.t, r.dt,
                   r.device_ms);
        } else {
            // the reference's output cadence (solverExplicit.cpp:171-174, 176-187, 310-321)
            // and, with node extraction, a row per step (:325)
            double dt0 = 0;
            if ((st = msx_initial_dt(h, &dt0)) != MSX_OK) {
                fprintf(stderr, "msx_deck: %s\n", msx_last_error());
                return 1;
            }
            long long numStepsT = (long long)((s.tf - s.t0) / dt0);
            long long sampler = s.outputs > 0 ? numStepsT / s.outputs : numStepsT;
            const long long every = sampler > 0 ? sampler : 1;
            auto emit = [&](double t) {
                if (!write_vtk(outdir, (int)outputs.size(), X, d.conn, h)) return false;
                outputs.push_back({"MuPhiSimOutputs_0_." + std::to_string(outputs.size()) + ".vtk", t});
                write_series(outdir, outputs);
                return true;
            };
            if (!outdir.empty() && s.t0 < 1E-12 && !emit(s.t0)) {
                fprintf(stderr, "msx_deck: cannot write output\n");
                return 1;
            }
            long long steps = 0, since = 0;
            for (;;) {
                const long long chunk = stepwise ? 1 : every;
                st = msx_run(h, chunk, &r);
                if (st != MSX_OK) break;
                steps += r.steps;
                since += r.steps;
                if (r.steps == 0) break;
                if (s.force_freq > 0 && !fp.step(h, r.t, r.dt)) {
                    fprintf(stderr, "msx_deck: cannot write %s\n", fp.path.c_str());
                    return 1;
                }
                for (auto &E : d.extractions)
                    if (!write_extraction(E, xdir, h, r.t)) {
                        fprintf(stderr, "msx_deck: cannot write %s/%s.csv\n", xdir.c_str(), E.name.c_str());
                        return 1;
                    }
                if (!outdir.empty() && (since >= every || r.t == s.tf)) {
                    if (!emit(r.t)) {
                        fprintf(stderr, "msx_deck: cannot write output\n");
                        return 1;
                    }
                    since = 0;
                }
                if (r.steps < chunk || r.t >= s.tf - 1E-12) break;
            }
            total += steps;
            printf("solver %zu: %lld steps, t = %.9g, dt = %.6g, %zu outputs so far\n", k, steps, r.t, r.dt,
                   outputs.size());
        }
        if (st != MSX_OK) {
            fprintf(stderr, "msx_deck: %s\n", msx_last_error());
            return 1;
        }
    }
    std::vector<double> u(3 * nn), v(3 * nn), a(3 * nn);
    msx_get_state(h, u.data(), v.data(), a.data());
    if (!dump.empty()) {
        FILE *f = fopen(dump.c_str(), "wb");
        if (!f) return 3;
        fwrite(u.data(), sizeof(double), u.size(), f);
        fwrite(v.data(), sizeof(double), v.size(), f);
        fwrite(a.data(), sizeof(double), a.size(), f);
        fclose(f);
    }
    if (!csv.empty()) {
        // full precision, as the reference's node extraction writes (dataExtraction.cpp:282-300)
        FILE *f = fopen(csv.c_str(), "w");
        if (!f) return 3;
        fprintf(f, "node,ux,uy,uz,vx,vy,vz\n");
        for (long long i = 0; i < nn; i++)
            fprintf(f, "%lld,%.16g,%.16g,%.16g,%.16g,%.16g,%.16g\n", i + 1, u[i], u[nn + i], u[2 * nn + i], v[i],
                    v[nn + i], v[2 * nn + i]);
        fclose(f);
    }
    printf("total %lld steps\n", total);
    for (auto &E : d.extractions)
        if (E.file) fclose(E.file);
    msx_destroy(h);
    msx_deck_loads_free(loads);
    return 0;
}
