// The reference's Block class (cppsrc/Block.h:34-106) is declared with Grid
// and Element in Grid.h.  This header lets code that includes "Block.h"
// compile against this package unchanged.
#pragma once

#include "Grid.h"
