// The reference's HDF5 output functions (cppsrc/HDF5Functions.h:19-26) over
// the C ABI's library-free HDF5 writer.  Same file names, dataset names,
// shapes and return codes (0, or -1..-4 for file / dataset failures).
#pragma once

#include <string>
#include <vector>

#include "Grid.h"

using std::string;
using std::vector;

// coords/ba/diff/rho0/c0 files of every block (cppsrc/HDF5Functions.cpp:34-142)
int dumpGridToHDF5File(string outputFolder, Grid* myGrid, int timestep, double time, int rank);
// dRho/vel files of every block; prints " - Printing to <file>; Max dRho=<max>"
// (cppsrc/HDF5Functions.cpp:145-247)
int dumpToHDF5File(string outputFolder, Grid* myGrid, int timestep, double time, int rank);
int hdf5outputVector(const vector<vector<vector<vector<double>>>>& data4D, string outputFilename, string Datasetname,
                     int Dimx, int Dimy, int Dimz, double time);
int hdf5outputScalar(const vector<vector<vector<double>>>& data3D, string outputFilename, string Datasetname,
                     int Dimx, int Dimy, int Dimz, double time);
// Reads dataset Datasetname, stored [Dimz][Dimy][Dimx] in row-major order, into
// data3D[x][y][z] (data3D pre-sized [Dimx][Dimy][Dimz]) and prints the HDF5
// datatype class; the reference's dormant restart reader
// (cppsrc/HDF5Functions.cpp:398-463) with the same index mapping, messages and
// return codes.  A dataset whose size differs from Dimx*Dimy*Dimz is a
// dataspace error (-3) here, where the reference reads past its buffer.
int hdf5input(vector<vector<vector<double>>>& data3D, string inputFilename, string Datasetname, int Dimx, int Dimy,
              int Dimz);
