// HDF5 output functions of the reference over the C ABI; see HDF5Functions.h.
#include "HDF5Functions.h"

#include <cmath>
#include <iostream>

namespace {

int code_of(int rc)
{
    // DG_ERR_* values that are not the reference's HDF5 codes become -1
    // (FileIException), the code of every file-level failure there.
    return (rc >= -4 && rc <= -1) ? rc : -1;
}

}  // namespace

int dumpGridToHDF5File(string outputFolder, Grid* myGrid, int timestep, double time, int rank)
{
    (void)time;
    (void)rank;  // one process writes every block's files
    std::cout << " - Printing to " << outputFolder << "/raw/coords_0_" << timestep << ".h5\n";
    int rc = dg_write_snapshot(myGrid->handle(), outputFolder.c_str(), timestep, 2);
    if (rc != DG_OK) {
        std::cout << "HDF5 FileIException error\n";
        return code_of(rc);
    }
    return 0;
}

int dumpToHDF5File(string outputFolder, Grid* myGrid, int timestep, double time, int rank)
{
    (void)time;
    (void)rank;
    int X, Y, Z;
    dg_dims(myGrid->handle(), &X, &Y, &Z);
    vector<double> rho((size_t)X * Y * Z);
    double maxDRho = 0.0;
    if (dg_get_state(myGrid->handle(), rho.data(), nullptr) == DG_OK)
        for (double v : rho)
            if (std::abs(v) > maxDRho || std::isnan(v)) maxDRho = std::abs(v);
    std::cout << " - Printing to " << outputFolder << "/raw/dRho_0_" << timestep << ".h5; Max dRho=" << maxDRho
              << "\n";
    int rc = dg_write_snapshot(myGrid->handle(), outputFolder.c_str(), timestep, 0);
    if (rc != DG_OK) {
        std::cout << "HDF5 FileIException error\n";
        return code_of(rc);
    }
    return 0;
}

int hdf5outputVector(const vector<vector<vector<vector<double>>>>& data4D, string outputFilename, string Datasetname,
                     int Dimx, int Dimy, int Dimz, double time)
{
    // data4D[i][j][k][h] -> dataset [3][X][Y][Z] (cppsrc/HDF5Functions.cpp:268-273)
    vector<double> flat((size_t)3 * Dimx * Dimy * Dimz);
    for (int h = 0; h < 3; h++)
        for (int i = 0; i < Dimx; i++)
            for (int j = 0; j < Dimy; j++)
                for (int k = 0; k < Dimz; k++)
                    flat[(((size_t)h * Dimx + i) * Dimy + j) * Dimz + k] = data4D[i][j][k][h];
    const long long dims[4] = {3, Dimx, Dimy, Dimz};
    return code_of(dg_hdf5_write(outputFilename.c_str(), Datasetname.c_str(), 4, dims, flat.data(), time));
}

int hdf5outputScalar(const vector<vector<vector<double>>>& data3D, string outputFilename, string Datasetname,
                     int Dimx, int Dimy, int Dimz, double time)
{
    vector<double> flat((size_t)Dimx * Dimy * Dimz);
    for (int i = 0; i < Dimx; i++)
        for (int j = 0; j < Dimy; j++)
            for (int k = 0; k < Dimz; k++) flat[((size_t)i * Dimy + j) * Dimz + k] = data3D[i][j][k];
    const long long dims[3] = {Dimx, Dimy, Dimz};
    return code_of(dg_hdf5_write(outputFilename.c_str(), Datasetname.c_str(), 3, dims, flat.data(), time));
}

int hdf5input(vector<vector<vector<double>>>& data3D, string inputFilename, string Datasetname, int Dimx, int Dimy,
              int Dimz)
{
    static const char* const kind[5] = {"", "File", "DataSet", "DataSpace", "DataType"};
    long long dims[32];
    int nd = 0, cls = -1;
    int rc = dg_hdf5_read(inputFilename.c_str(), Datasetname.c_str(), 32, dims, &nd, nullptr, 0, &cls);
    long long n = 1;
    for (int i = 0; i < nd && rc == 0; i++) n *= dims[i];
    if (rc == 0 && n != (long long)Dimx * Dimy * Dimz) rc = -3;
    std::vector<double> flat;
    if (rc == 0) {
        std::cout << cls << "\n";
        flat.resize((size_t)n);
        rc = dg_hdf5_read(inputFilename.c_str(), Datasetname.c_str(), 0, nullptr, nullptr, flat.data(), n, nullptr);
    }
    if (rc != 0) {
        rc = code_of(rc);
        std::cout << "HDF5 " << kind[-rc] << "IException error\n";
        return rc;
    }
    for (int z = 0; z < Dimz; z++)
        for (int y = 0; y < Dimy; y++)
            for (int x = 0; x < Dimx; x++) data3D[x][y][z] = flat[((size_t)z * Dimy + y) * Dimx + x];
    return 0;
}
