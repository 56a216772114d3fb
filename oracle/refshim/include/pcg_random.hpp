// Shim for the reference's <pcg_random.hpp> (pcg-cpp): forwards to the copy
// of pcg-cpp that pyarrow vendors in namespace arrow_vendored.  Test
// infrastructure for building the reference's own sources (oracle/refshim).
#pragma once
#include PCG_VENDORED_HEADER
using arrow_vendored::pcg32;
namespace pcg_extras = arrow_vendored::pcg_extras;
