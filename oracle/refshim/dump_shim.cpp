/* Stand-in for the reference's HDF5 output (cppsrc/HDF5Functions.cpp), used
 * only when the reference sources are compiled as a CPU oracle; this machine
 * has no libhdf5.  Test infrastructure: never linked into the product.
 *
 * It implements the two functions the reference's driver calls
 * (cppsrc/HDF5Functions.h:19-20) with the same node-duplicated gather as the
 * original (cppsrc/HDF5Functions.cpp:34-247: X = E_x*(N+1), element index +1 to
 * skip the halo ring) and writes each dataset as a flat little-endian file:
 *   char magic[8] = "DGRAW01"; int32 ndim; int32 pad; int64 dims[ndim];
 *   double time; double data[prod(dims)]   (row-major, same order as the HDF5
 *   dataset: [X][Y][Z] for scalars, [3][X][Y][Z] for vectors)
 * File names follow the original with ".bin" for ".h5".
 */
#include <cstdio>
#include <cstdint>
#include <string>
#include <vector>
#include <cmath>
#include <iostream>
#include "HDF5Functions.h"
#include "Grid.h"
#include "Block.h"

namespace {

int write_raw(const std::string& path, const std::vector<int64_t>& dims, double t,
              const std::vector<double>& data)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return -1;
    char magic[8] = {'D', 'G', 'R', 'A', 'W', '0', '1', 0};
    int32_t nd = (int32_t)dims.size(), pad = 0;
    std::fwrite(magic, 1, 8, f);
    std::fwrite(&nd, 4, 1, f);
    std::fwrite(&pad, 4, 1, f);
    std::fwrite(dims.data(), 8, dims.size(), f);
    std::fwrite(&t, 8, 1, f);
    std::fwrite(data.data(), 8, data.size(), f);
    std::fclose(f);
    return 0;
}

struct Gather {
    int X, Y, Z, order;
    Grid* g;
    Gather(Grid* grid) : g(grid)
    {
        order = g->getOrder();
        int nb = g->getNumBlocks()[0] * g->getNumBlocks()[1] * g->getNumBlocks()[2];
        int m[3] = {1, 1, 1};
        if (nb == 1) for (int a = 0; a < 3; a++) m[a] = g->getNumBlocks()[a];
        X = m[0] * g->getNumElements()[0] * (order + 1);
        Y = m[1] * g->getNumElements()[1] * (order + 1);
        Z = m[2] * g->getNumElements()[2] * (order + 1);
    }
    Element& at(int ii, int jj, int kk, int nod[3])
    {
        const int K = order + 1;
        int* ne = g->getNumElements();
        int nb = g->getNumBlocks()[0] * g->getNumBlocks()[1] * g->getNumBlocks()[2];
        Block* b;
        int ele[3];
        if (nb == 1) {
            b = &g->mBlocks[ii / ne[0] / K][jj / ne[1] / K][kk / ne[2] / K];
            ele[0] = (ii / K) % ne[0] + 1;
            ele[1] = (jj / K) % ne[1] + 1;
            ele[2] = (kk / K) % ne[2] + 1;
        } else {
            b = &g->mBlock;
            ele[0] = ii / K + 1;
            ele[1] = jj / K + 1;
            ele[2] = kk / K + 1;
        }
        nod[0] = ii % K;
        nod[1] = jj % K;
        nod[2] = kk % K;
        return b->mElements[ele[0]][ele[1]][ele[2]];
    }
};

std::string rawname(const std::string& folder, const char* stem, int rank, int ts)
{
    return folder + "/raw/" + stem + "_" + std::to_string(rank) + "_" + std::to_string(ts) + ".bin";
}

}  // namespace

int dumpGridToHDF5File(string outputFolder, Grid* myGrid, int timestep, float time, int rank)
{
    Gather G(myGrid);
    size_t n = (size_t)G.X * G.Y * G.Z;
    std::vector<double> coords(3 * n), c0(n), rho0(n), ba(n), diff(n);
    for (int i = 0; i < G.X; i++)
        for (int j = 0; j < G.Y; j++)
            for (int k = 0; k < G.Z; k++) {
                int nod[3];
                Element& e = G.at(i, j, k, nod);
                size_t p = ((size_t)i * G.Y + j) * G.Z + k;
                for (int a = 0; a < 3; a++) coords[a * n + p] = e.getOutputCoords(nod)[a];
                c0[p] = e.getC0();
                rho0[p] = e.getRho0();
                ba[p] = e.getBoverA();
                diff[p] = e.getDiffusionConstant();
            }
    std::vector<int64_t> d3 = {G.X, G.Y, G.Z}, d4 = {3, G.X, G.Y, G.Z};
    int rc = 0;
    rc |= write_raw(rawname(outputFolder, "coords", rank, timestep), d4, time, coords);
    rc |= write_raw(rawname(outputFolder, "ba", rank, timestep), d3, time, ba);
    rc |= write_raw(rawname(outputFolder, "diff", rank, timestep), d3, time, diff);
    rc |= write_raw(rawname(outputFolder, "rho0", rank, timestep), d3, time, rho0);
    rc |= write_raw(rawname(outputFolder, "c0", rank, timestep), d3, time, c0);
    return rc ? -1 : 0;
}

int dumpToHDF5File(string outputFolder, Grid* myGrid, int timestep, float time, int rank)
{
    Gather G(myGrid);
    size_t n = (size_t)G.X * G.Y * G.Z;
    std::vector<double> rho(n), vel(3 * n);
    double maxDRho = 0.0;
    for (int i = 0; i < G.X; i++)
        for (int j = 0; j < G.Y; j++)
            for (int k = 0; k < G.Z; k++) {
                int nod[3];
                Element& e = G.at(i, j, k, nod);
                size_t p = ((size_t)i * G.Y + j) * G.Z + k;
                rho[p] = e.getOutputRho(nod);
                if (std::abs(rho[p]) > maxDRho || std::isnan(rho[p])) maxDRho = std::abs(rho[p]);
                for (int a = 0; a < 3; a++) vel[a * n + p] = e.getOutputVelocity(nod)[a];
            }
    std::cout << " - Printing to " << rawname(outputFolder, "dRho", rank, timestep)
              << "; Max dRho=" << maxDRho << "\n";
    std::vector<int64_t> d3 = {G.X, G.Y, G.Z}, d4 = {3, G.X, G.Y, G.Z};
    int rc = 0;
    rc |= write_raw(rawname(outputFolder, "dRho", rank, timestep), d3, time, rho);
    rc |= write_raw(rawname(outputFolder, "vel", rank, timestep), d4, time, vel);
    return rc ? -1 : 0;
}
