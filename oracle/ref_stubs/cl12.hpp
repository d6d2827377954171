/* Stand-in for the Khronos OpenCL C++ bindings when the reference's CPU
 * "Equivalent" code is compiled for the oracle: that code only needs the C
 * headers below from it. */
#pragma once
#include <climits>
#include <cmath>
#include <cstring>
using std::isinf;
