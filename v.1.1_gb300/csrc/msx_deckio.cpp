// msx_deckio.cpp -- the Neumann blocks of an input deck, read by the library.
//
// The reference keeps each load's parameters (t0, tf, amounts) private in its
// load classes (solvers/classNeumannBCs.h:32-506), so a solver plugin that is
// handed the reference's NeumannBCs list cannot read them.  This reader gives
// that plugin, and the msx_deck front end, the same blocks from the deck file
// itself: one msx_load_block per block, in file order, as
// NeumannCommonManagement (IO/inputFile.cpp:4705-4760) scans the whole file
// and builds one classNeumannBCs per block.
//
// Block formats (IO/inputFile.cpp): *BOUNDARY, TYPE=FORCE "t0, tf, Ff" then
// "node, Fx, Fy, Fz" lines (:2841-2945; entry value F_k * Ff); *BOUNDARY,
// TYPE=TRACTION INST|RAMP "t0, tf, Tx, Ty, Tz, S" and *BOUNDARY,
// TYPE=PRESSURE INST|RAMP "t0, tf, P, S", then one bulk tet per line
// (:3229-3780); *GRAVITY then g (:4723-4735).  Node and element ids are
// 1-based in the file and 0-based here.
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/msx.h"
#include "msx_internal.h"

struct msx_deck_loads {
    std::vector<msx_load_block> blocks;
    std::vector<std::vector<msx_nodal_force>> forces;   // per block
    std::vector<std::vector<int32_t>> elems;            // per block
};

namespace {

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

msx_status bad(const std::string &path, size_t line, const std::string &msg)
{
    msx::msx_set_error(("msx_deck_read_loads: " + msg + " (" + path + " line " + std::to_string(line) + ")").c_str());
    return MSX_ERR_ARG;
}

}  // namespace

extern "C" msx_status msx_deck_read_loads(const char *path, int64_t num_nodes, msx_deck_loads **out)
{
    if (!path || !out || num_nodes < 1) {
        msx::msx_set_error("msx_deck_read_loads: NULL path or output, or no nodes");
        return MSX_ERR_ARG;
    }
    *out = nullptr;
    std::ifstream in(path);
    if (!in) {
        msx::msx_set_error((std::string("msx_deck_read_loads: cannot open ") + path).c_str());
        return MSX_ERR_ARG;
    }
    std::vector<std::string> lines;
    for (std::string l; std::getline(in, l);) lines.push_back(trim(l));
    const size_t n = lines.size();
    auto data_line = [&](size_t k) { return k < n && !lines[k].empty() && lines[k][0] != '*'; };
    msx_deck_loads *d = new msx_deck_loads();
    auto fail = [&](size_t line, const std::string &msg) {
        delete d;
        return bad(path, line, msg);
    };
    for (size_t i = 0; i < n; i++) {
        const std::string &L = lines[i];
        msx_load_block B{};
        std::vector<msx_nodal_force> forces;
        std::vector<int32_t> elems;
        if (starts(L, "*BOUNDARY, TYPE=FORCE")) {
            if (i + 1 >= n) return fail(i + 1, "a force block starts with t0, tf, Ff");
            auto h = split(lines[i + 1]);
            if (h.size() != 3) return fail(i + 2, "a force block starts with t0, tf, Ff");
            const double t0 = atof(h[0].c_str()), tf = atof(h[1].c_str()), Ff = atof(h[2].c_str());
            B.kind = MSX_LOAD_FORCE;
            size_t k = i + 2;
            for (; data_line(k); k++) {
                auto f = split(lines[k]);
                if (f.size() != 4) return fail(k + 1, "a force line has node, Fx, Fy, Fz");
                const long long node = atoll(f[0].c_str()) - 1;
                if (node < 0 || node >= num_nodes) return fail(k + 1, "force node out of range");
                for (int c = 0; c < 3; c++) forces.push_back({node + c * num_nodes, t0, tf, atof(f[c + 1].c_str()) * Ff});
            }
            i = k - 1;
        } else if (starts(L, "*BOUNDARY, TYPE=TRACTION RAMP") || starts(L, "*BOUNDARY, TYPE=TRACTION INST") ||
                   starts(L, "*BOUNDARY, TYPE=PRESSURE RAMP") || starts(L, "*BOUNDARY, TYPE=PRESSURE INST")) {
            const bool pressure = L.find("PRESSURE") != std::string::npos, ramp = L.find("RAMP") != std::string::npos;
            B.kind = pressure ? (ramp ? MSX_LOAD_PRESSURE_RAMP : MSX_LOAD_PRESSURE_INST)
                              : (ramp ? MSX_LOAD_TRACTION_RAMP : MSX_LOAD_TRACTION_INST);
            const size_t nv = pressure ? 1 : 3;
            auto h = i + 1 < n ? split(lines[i + 1]) : std::vector<std::string>();
            if (h.size() != nv + 3)
                return fail(i + 2, pressure ? "a pressure block starts with t0, tf, P, S"
                                            : "a traction block starts with t0, tf, Tx, Ty, Tz, S");
            B.t0 = atof(h[0].c_str());
            B.tf = atof(h[1].c_str());
            for (size_t k = 0; k < nv; k++) B.value[k] = atof(h[2 + k].c_str());
            B.face = (int32_t)atof(h[2 + nv].c_str());
            if (B.face < 1 || B.face > 4) return fail(i + 2, "the face of a C3D4 surface load is 1..4");
            size_t k = i + 2;
            for (; data_line(k); k++) elems.push_back(atoi(lines[k].c_str()) - 1);
            i = k - 1;
        } else if (starts(L, "*GRAVITY")) {
            if (i + 1 >= n) return fail(i + 1, "*GRAVITY needs g");
            B.kind = MSX_LOAD_GRAVITY;
            B.value[0] = atof(lines[i + 1].c_str());
            i++;
        } else {
            continue;
        }
        d->blocks.push_back(B);
        d->forces.push_back(std::move(forces));
        d->elems.push_back(std::move(elems));
    }
    // point the blocks at their entry arrays only now: the vectors no longer move
    for (size_t k = 0; k < d->blocks.size(); k++) {
        msx_load_block &B = d->blocks[k];
        B.forces = d->forces[k].empty() ? nullptr : d->forces[k].data();
        B.num_forces = (int64_t)d->forces[k].size();
        B.elems = d->elems[k].empty() ? nullptr : d->elems[k].data();
        B.num_elems = (int64_t)d->elems[k].size();
    }
    *out = d;
    return MSX_OK;
}

extern "C" msx_status msx_deck_loads_blocks(const msx_deck_loads *d, const msx_load_block **blocks, int64_t *num_blocks)
{
    if (!d || !blocks || !num_blocks) {
        msx::msx_set_error("msx_deck_loads_blocks: NULL argument");
        return MSX_ERR_ARG;
    }
    *blocks = d->blocks.empty() ? nullptr : d->blocks.data();
    *num_blocks = (int64_t)d->blocks.size();
    return MSX_OK;
}

extern "C" msx_status msx_deck_loads_free(msx_deck_loads *d)
{
    delete d;
    return MSX_OK;
}
