// Basis facade over the FP64 basis module; see Basis.h.
#include "Basis.h"

#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include <unistd.h>

#include <cstdio>

#include "BCParam.h"
#include "dg3d.h"

// cppsrc/BCParam.cpp:24
extern const BCParam BCParamDefault = {{false, false, false}, {10, 10, 10, 10, 10, 10}, -1.0, false, false, false,
                                       -1.0, -1.0, -1.0, -1.0, -1.0, -1.0, -1.0, -1.0};

namespace {

double hex2double(const std::string& s)
{
    uint64_t b = 0;
    for (char c : s) {
        int d = (c >= '0' && c <= '9') ? c - '0' : (c >= 'a' && c <= 'f') ? c - 'a' + 10 : (c >= 'A' && c <= 'F') ? c - 'A' + 10 : 0;
        b = (b << 4) | (uint64_t)d;
    }
    double v;
    std::memcpy(&v, &b, 8);
    return v;
}

void require_open(const string& f)
{
    std::ifstream in(f);
    if (!in.is_open())
        throw std::runtime_error("Opening file '" + f + "' failed, it either doesn't exist or is not accessible.\n");
}

}  // namespace

Basis::Basis(string filename, string filename2) : mCoeffFile(filename)
{
    load(filename, filename2);
}

void Basis::load(const string& filename, const string& filename2)
{
    require_open(filename);
    require_open(filename2);
    std::ifstream f(filename);
    string line;
    int phase = 0, npts = 0;
    while (std::getline(f, line)) {
        if (phase == 0) {
            npts = std::atoi(line.c_str() + 2);
        } else {
            std::istringstream iss(line);
            vector<double> v;
            string tok;
            for (int i = 0; i < npts && (iss >> tok); i++) v.push_back(hex2double(tok));
            (phase == 1 ? mZeros : mWeights).push_back(v);
        }
        phase = (phase + 1) % 3;
    }
    std::ifstream f2(filename2);
    vector<vector<double>> grid;
    bool first = true;
    npts = 0;
    while (std::getline(f2, line)) {
        if (line.compare(0, 1, "p") == 0) {
            if (!first) {
                mDPsi.push_back(grid);
                mPsi.push_back(grid);
            }
            first = false;
            npts = std::atoi(line.c_str() + 2);
            grid.clear();
        } else {
            std::istringstream iss(line);
            vector<double> row;
            string tok;
            for (int i = 0; i < npts && (iss >> tok); i++) row.push_back(hex2double(tok));
            grid.push_back(row);
        }
    }
    mDPsi.push_back(grid);
    mPsi.push_back(grid);
}

namespace {
string generated_dir(int kmax)
{
    char tmpl[] = "/tmp/dg3d_basis_XXXXXX";
    char* d = mkdtemp(tmpl);
    if (!d) throw std::runtime_error("cannot create a temporary directory for the basis files");
    if (dg_write_basis_files(d, kmax, 0) != DG_OK) throw std::runtime_error(dg_last_error());
    return d;
}
}  // namespace

// Generated tables: written through the C ABI in the reference's formats,
// then read back exactly as the file constructor reads them.
Basis::Basis(int kmax)
{
    const string d = generated_dir(kmax);
    load(d + "/hardcoded_coeff.txt", d + "/hardcoded_coeff2.txt");
    for (const char* f : {"hardcoded_coeff.txt", "hardcoded_coeff2.txt", "matrices.txt"}) std::remove((d + "/" + f).c_str());
    rmdir(d.c_str());
}
