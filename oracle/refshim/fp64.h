/* Pre-included (g++ -include) to build the FP64-promoted reference ("ref64").
 *
 * Test infrastructure only.  Every standard header the reference uses is
 * included first (through compat.h) so that the keyword substitution below only
 * reaches the reference's own code: node fields, element constants, DT and the
 * parsed parameters all become double.  Float LITERALS keep their float type
 * (e.g. the RK weights 2.0F/3.0F and 1.0F/3.0F in cppsrc/Grid.cpp:826-827 stay
 * float-rounded), exactly as the reference's own FP64 build would compute them.
 */
#include "compat.h"
#define float double
