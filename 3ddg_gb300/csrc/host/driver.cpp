// dg3d: drop-in for the reference's 3D-DG driver (cppsrc/driver.cpp:70-291).
//
//   dg3d <parameter file> <output folder>
//
// Same command line, error codes (0 success, 1 bad arguments, 2 bad parameter,
// 3 cannot read, 4 cannot write), parameter-file format, _log.txt echo, console
// progress, HDF5 snapshot files and output cadence (grid + state at step 0,
// state after every NUM_TIME_SUBSTEPS steps).  The mesh, operators and state
// live on the GPU; the state is copied back only at output steps.
//
// Basis inputs: hardcoded_coeff.txt / hardcoded_coeff2.txt / matrices.txt are
// read from the working directory as the reference reads them; when they are
// absent the same tables are generated from LGL mathematics.
#include <sys/stat.h>
#include <sys/time.h>
#include <sys/types.h>

#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>

#include "Basis.h"
#include "Grid.h"
#include "HDF5Functions.h"
#include "dg3d.h"

namespace {

const int ERRCODE_SUCESSFUL_COMPLETION = 0;
const int ERRCODE_INVALID_ARGUMENT = 1;
const int ERRCODE_INVALID_PARAMETER = 2;
const int ERRCODE_CANNOT_READ = 3;
const int ERRCODE_CANNOT_WRITE = 4;

const char* NEEDED_ARGUMENTS =
    "	PARAMETER_FILENAME : path to the file defining simulation parameters\n"
    "	OUTPUT_FILENAME : path to the file that the data will be written to";

double wtime()
{
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

bool exists(const std::string& f)
{
    std::ifstream in(f);
    return in.is_open();
}

}  // namespace

int main(int argc, char* argv[])
{
    std::cout << " - Thread 0 created\n";
    if (argc != 3) {
        std::cerr << "Not enough command line arguments.\n" << NEEDED_ARGUMENTS;
        return ERRCODE_INVALID_ARGUMENT;
    }
    const std::string parameterFilename = argv[1], outputFolder = argv[2];
    const std::string logFilename = outputFolder + "/_log.txt";
    std::cout << " - Parameters from   : " << parameterFilename << "\n";
    std::cout << " - Log will be written to : " << logFilename << "\n";
    std::cout << " - Results in same folder as log\n";
    std::cout << "Setting up I/O\n - Checking Folder\n";
    mkdir(outputFolder.c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH);
    mkdir((outputFolder + "/raw").c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH);
    std::cout << " - Preparing to write\n";
    {
        std::ofstream probe(logFilename);
        if (!probe.is_open()) {
            std::cerr << "Unable to open log file " << logFilename << "\n";
            return ERRCODE_CANNOT_WRITE;
        }
    }
    std::cout << " - Reading parameters\n";
    dg_params p;
    dg_params_default(&p);
    double DT = .001;
    int NUM_TIME_SUBSTEPS = 1, NUM_OUTSTEPS = 1, FREQ_TERMINAL = 1, BOOL_FILE = 1;
    int rc = dg_params_parse(parameterFilename.c_str(), &p, &DT, &NUM_TIME_SUBSTEPS, &NUM_OUTSTEPS, &FREQ_TERMINAL,
                             &BOOL_FILE, logFilename.c_str());
    if (rc == DG_ERR_IO) {
        std::cerr << dg_last_error() << "\n";
        return ERRCODE_CANNOT_READ;
    }
    if (rc != DG_OK) {
        std::cerr << dg_last_error() << "\n";
        return ERRCODE_INVALID_PARAMETER;
    }
    if (FREQ_TERMINAL < 1) FREQ_TERMINAL = 1;

    std::cout << " - Reading basis\n";
    Basis* basis = nullptr;
    std::string matrixFile = "matrices.txt";
    try {
        if (exists("hardcoded_coeff.txt") && exists("hardcoded_coeff2.txt")) {
            basis = new Basis("hardcoded_coeff.txt", "hardcoded_coeff2.txt");
        } else {
            std::cout << " - Coefficient files not found: generating LGL tables\n";
            basis = new Basis(10);
        }
        if (!exists(matrixFile)) {
            std::cout << " - matrices.txt not found: computing mass/stiffness matrices\n";
            matrixFile.clear();
        }
    } catch (const std::exception& e) {
        std::cerr << e.what();
        return ERRCODE_CANNOT_READ;
    }

    const unsigned NUM_TIMESTEPS = (unsigned)NUM_OUTSTEPS * (unsigned)NUM_TIME_SUBSTEPS;
    std::cout << "Creating mesh\n - Initializing grid using matrices from 'matrices.txt'\n";
    Grid* myGrid;
    try {
        myGrid = new Grid(p, matrixFile, basis);
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return ERRCODE_INVALID_PARAMETER;
    }
    Grid myGrid2(*myGrid), k1(*myGrid), k2(*myGrid);
    Grid* oldGrid = myGrid;
    Grid* newGrid = &myGrid2;
    std::ofstream logFile(logFilename, std::ios::app);
    std::cout << " - Logging grid\n";
    if (BOOL_FILE && dumpGridToHDF5File(outputFolder, newGrid, 0, 0.0, 0) != 0) return ERRCODE_CANNOT_WRITE;
    std::cout << " - Logging initial conditions\n";
    if (BOOL_FILE && dumpToHDF5File(outputFolder, newGrid, 0, 0.0, 0) != 0) return ERRCODE_CANNOT_WRITE;

    double t = 0;
    double beginTime = wtime(), prevTime = beginTime, endTime;
    std::cout << "Timestepping\n";
    try {
        for (unsigned i = 0; i < NUM_TIMESTEPS; i += NUM_TIME_SUBSTEPS) {
            endTime = wtime();
            if (i > 0) std::cout << "    - Elapsed runtime:" << int(endTime - beginTime) << "s\n";
            if (i > 0)
                std::cout << "    - Estimated remaining:"
                          << int((endTime - prevTime) * (NUM_TIMESTEPS - i) / NUM_TIME_SUBSTEPS) << "s\n";
            prevTime = endTime;
            for (unsigned j = 0; j < (unsigned)NUM_TIME_SUBSTEPS; j++) {
                if ((i * NUM_TIME_SUBSTEPS + j) % FREQ_TERMINAL == 0) {
                    std::cout << " - Timestep ";
                    std::cout.width(7);
                    std::cout << i + j << "/" << NUM_TIMESTEPS << " (";
                    std::cout.width(3);
                    std::cout << 100 * (i + j) / (NUM_TIMESTEPS ? NUM_TIMESTEPS : 1) << "%) : t=";
                    std::cout.width(5);
                    std::cout << t << "\n";
                }
                Grid* swapGrid = oldGrid;
                oldGrid = newGrid;
                newGrid = swapGrid;
                newGrid->RK33(DT, oldGrid, &k1, &k2, logFile);
                t += DT;
            }
            if (BOOL_FILE && dumpToHDF5File(outputFolder, newGrid, i + NUM_TIME_SUBSTEPS, t, 0) != 0)
                return ERRCODE_CANNOT_WRITE;
        }
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return ERRCODE_INVALID_PARAMETER;
    }
    std::cout << "Post-processing\n";
    endTime = wtime();
    std::cout << "Exiting\nTotal runtime is " << (endTime - beginTime) << "s\n";
    delete myGrid;
    delete basis;
    return ERRCODE_SUCESSFUL_COMPLETION;
}
