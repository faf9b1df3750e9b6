// The reference keeps one Node object per node (cppsrc/Node.h:32-95).  Here
// node data lives in device buffers (structure of arrays); nodes are read and
// written through Element (getOutputRho, getOutputVelocity, setRho, ...) on a
// host mirror.  This header lets code that includes "Node.h", as the
// reference's driver does (cppsrc/driver.cpp:34), compile unchanged; it
// declares no Node class.
#pragma once

#include "Grid.h"
