// The reference's Element class (cppsrc/Element.h:35-158) is declared with
// Grid and Block in Grid.h (they share one simulation handle).  This header
// exists so that code including "Element.h", as the reference's driver does
// (cppsrc/driver.cpp:33), compiles against this package unchanged.
#pragma once

#include "Grid.h"
