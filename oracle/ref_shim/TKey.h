// Test-infrastructure shim (see RtypesShim.h): nothing of this ROOT header is used.
#include "RtypesShim.h"
