/* Stand-in for CommonSources/HalfToFloat.hpp: the reference's encoders
 * convert half texels with the `half` type's own float conversion
 * (oracle/ref_stubs/half.h), so nothing else is needed here. */
#pragma once
#include <half.h>
