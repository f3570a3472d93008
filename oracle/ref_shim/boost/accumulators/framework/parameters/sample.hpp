// Test-infrastructure shim: forwards to the accumulator framework shim.
#include "../../accumulators_shim.hpp"
