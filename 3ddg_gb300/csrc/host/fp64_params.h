// Pre-include (g++ -include fp64_params.h) for building the reference's
// driver with FP64 parameters, the way the reference's own sources build with
// every float promoted to double.  The standard headers, the MPI header and
// this package's class headers are read first, unchanged; after them `float` names `double`,
// so the driver's parameters (ELEMENT_WIDTH, DT, C0, ...) are parsed as
// doubles and select the double Grid constructor.  Float literals keep their
// type.  Without this header the driver's parameters are floats, as in the
// reference as shipped; the simulation itself is FP64 either way.
#pragma once

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

#include "BCParam.h"
#include "Basis.h"
#include "Grid.h"
#include "HDF5Functions.h"
#include "Matrix.h"

// the MPI header the driver includes (an installation's, or single_process/)
#include <mpi.h>

#define float double
