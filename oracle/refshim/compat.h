/* Pre-included (g++ -include) when compiling the reference C++ sources in place.
 *
 * Test infrastructure only: nothing in the product links or includes this file.
 *
 * The reference's SSTR macro (cppsrc/Element.h:23, cppsrc/Block.h:24) does
 *   static_cast<std::ostringstream&>((std::ostringstream() << std::dec << x)).str()
 * With a C++11 libstdc++ the first insertion into the temporary stream binds the
 * rvalue-stream operator<< template, whose result is an xvalue, and the
 * static_cast to an lvalue reference is rejected by g++ 13.  The non-template
 * overload below is preferred for exactly that first insertion and yields an
 * lvalue, so the macro compiles unchanged and the reference sources stay
 * untouched.
 */
#ifndef DG_REFSHIM_COMPAT_H
#define DG_REFSHIM_COMPAT_H
#include <sstream>
#include <vector>
#include <string>
#include <iostream>
#include <fstream>
#include <cmath>
#include <algorithm>
#include <limits>
#include <bitset>
#include <cstring>
#include <iomanip>
#include <cassert>
#include <ctime>
#include <math.h>
#include <cstdlib>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

inline std::ostringstream& operator<<(std::ostringstream&& os,
                                      std::ios_base& (*manip)(std::ios_base&))
{
    manip(os);
    return os;
}
#endif
